/* polyred_cuda_testing.h — test hooks of libpolyred_cuda.so.
 *
 * Not part of the renderer's interface (include/polyred_cuda.h) and without
 * counterparts in the reference: entry points the library's own tests call
 * to inject failures on the host and to compare the device arithmetic of
 * single functions with its float64 definition. A host renderer never calls
 * them; their names and signatures may change with the library.
 */
#ifndef POLYRED_CUDA_TESTING_H
#define POLYRED_CUDA_TESTING_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Host-side failure injection: the n-th device (cudaMalloc) or page-locked
 * (cudaHostAlloc) allocation the library attempts from now on, in any
 * context or batch of the process, reports cudaErrorMemoryAllocation without
 * calling CUDA, so the call that made it returns PR_ERR_OOM with a detail
 * string; n = 0 turns the injection off. No device work fails: the context
 * stays usable, and a later call retries the allocation. */
int     pr_testing_fail_alloc(int64_t n);
/* Allocation attempts (device and page-locked) since the library loaded. */
int64_t pr_testing_alloc_count(void);

/* The AO march directions (cos, sin: 8 floats each) and, for a W x H frame,
 * how the device marches each (host only, no device): fast[k] 1 when its
 * tap offset table is exact, tiny[k] the component (1 = x, 2 = y) that lies
 * in (-1/99, 0). Returns the number of directions or a negative status. */
int pr_debug_ao_dirs(int W, int H, float* cosv, float* sinv, int8_t* fast, int8_t* tiny);

/* Device arithmetic probes (one thread per element, n device-resident
 * elements; synchronous): */
/* the shade kernel's float32 Pow beside the float64 algorithm */
int pr_debug_pow_probe(const float* x, const float* y, float* fast, float* ref, int n);
/* the AO kernel's float32 Atan and its certified Pow(T, 10000) colour
 * scaling, each beside the float64 algorithm (col, o_fast, o_ref: 4 bytes
 * per element) */
int pr_debug_ao_probe(const float* x, float* atan_fast, float* atan_ref, const float* T, const uint8_t* col,
                      uint8_t* o_fast, uint8_t* o_ref, int n);
/* the float32 emulation of float32(fma(f64, f64, f64)) beside the direct
 * float64 expression */
int pr_debug_fma_probe(const float* a, const float* b, const float* c, float* out, float* out_ref, int n);

/* Host texture probes (no device): the levels build_texture makes — texels
 * into out (capacity cap texels), levels as [n, w0, h0, off0, ...] into desc
 * (1 + 3 * 16 ints), returning the texel count or a negative status — and
 * Texture.Query of n (lod, u, v) triples, with du / dv the FragmentShader
 * lod of (du[k], dv[k]) in place of lod[k]. */
long long pr_debug_texture_build(int w, int h, const uint8_t* rgba, int mipmap, uint32_t* out, size_t cap,
                                 int32_t* desc);
int pr_debug_texture_query(int w, int h, const uint8_t* rgba, int mipmap, int n, const float* lod, const float* du,
                           const float* dv, const float* u, const float* v, uint8_t* out);

#ifdef __cplusplus
}
#endif

#endif /* POLYRED_CUDA_TESTING_H */
