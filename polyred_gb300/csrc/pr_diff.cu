// Differentiable deferred shading: the float radiance of the shade pass and
// its adjoint, with visibility held fixed by the differentiation G-buffer the
// forward frame writes (shade_kernel / ao_kernel).
//
// The radiance follows shade + FragmentShader (render/raster.go:320-356,
// shader/blinn_cpu.go:24-106) before Round and the uint8 conversions:
//   material pixel, channel c:
//     La_c = sum_e Ie col_c                       (col: the 1x1 texture's texel)
//     per light: point    D = lp - x, L = D/|D|, I = Il/|D|
//                directional  L = -dir, I = Il
//       V = unit(cam - x), H = unit(L + V)
//       Ld = clamp(n.L, 0, 1), Ls = clamp(n.H, 0, 1)^s
//     pre_c = La_c + kd_c sum_l Ld col_c I + ks_c sum_l Ls lcol_c I
//     R_c = fac clamp(pre_c, 0, 255),   n = unit(sum_k b_k N_k) (or the face normal)
//   material-less pixel: R_c = 255 sum_k p_k C_k,c
//   background: the background colour.
// The backward pass recomputes every term above from the G-buffer and the
// parameters (nothing per light is stored) and accumulates: per-vertex colour
// and normal gradients by float atomics, per-material and per-light gradients
// by block sums in shared memory, then double atomics.
#include <cuda_runtime.h>

#include <algorithm>

#include "pr_devmath.cuh"
#include "pr_kernels.cuh"

namespace prk {
namespace {

using namespace prd;

constexpr int kDiffThreads = 256;

struct F3 { float x, y, z; };
__device__ __forceinline__ F3 f3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float norm3(F3 a) { return sqrtf(dot(a, a)); }

__device__ __forceinline__ uint32_t find_obj(const uint32_t* first, uint32_t n_obj, uint32_t t) {
    uint32_t lo = 0, hi = n_obj - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (first[mid] <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <bool BACKWARD>
__global__ void __launch_bounds__(kDiffThreads) diff_kernel(const __grid_constant__ DiffParamsK P) {
    // block sums: [mat*7 + {kd0..2, ks0..2, shin}] [light*4 + {pos0..2, I}] [ambient]
    __shared__ float s_acc[kDiffMaxMats * 7 + kMaxLights * 4 + kMaxAmbient];
    const int n_acc = P.n_mats * 7 + P.n_lights * 4 + P.n_ambient;
    if (BACKWARD) {
        for (int k = threadIdx.x; k < n_acc; k += blockDim.x) s_acc[k] = 0.0f;
        __syncthreads();
    }
    const size_t npx = (size_t)P.W * P.H;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npx) {
        const float4 d0 = P.dgb[4 * i], d1 = P.dgb[4 * i + 1], d2 = P.dgb[4 * i + 2], d3 = P.dgb[4 * i + 3];
        const uint32_t t = __float_as_uint(d0.x);
        const int m = __float_as_int(d0.y);
        const uint32_t fl = __float_as_uint(d0.z);
        const float fac = d0.w;
        float R[3] = {0.0f, 0.0f, 0.0f};
        float g[3] = {0.0f, 0.0f, 0.0f};
        if (BACKWARD) {
            const float4 gr = P.grad[i];
            g[0] = gr.x;
            g[1] = gr.y;
            g[2] = gr.z;
        }
        const float alpha = d1.w;
        if (t == 0xFFFFFFFFu) {
            R[0] = P.bg[0];
            R[1] = P.bg[1];
            R[2] = P.bg[2];
        } else if (fl & kDgbUnlit) {
            const float p[3] = {d1.x, d1.y, d1.z};
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float4 C = P.vcol[3 * (size_t)t + k];
                R[0] += 255.0f * p[k] * C.x;
                R[1] += 255.0f * p[k] * C.y;
                R[2] += 255.0f * p[k] * C.z;
                if (BACKWARD && P.g_vcol) {
                    float* gc = reinterpret_cast<float*>(P.g_vcol + 3 * (size_t)t + k);
                    atomicAdd(gc + 0, g[0] * 255.0f * p[k]);
                    atomicAdd(gc + 1, g[1] * 255.0f * p[k]);
                    atomicAdd(gc + 2, g[2] * 255.0f * p[k]);
                }
            }
        } else if ((fl & (kDgbLit | kDgbConst)) && m >= 0 && m < P.n_mats) {
            const pr_material& mat = P.mats[m];
            const float col[3] = {(float)mat.texture[0], (float)mat.texture[1], (float)mat.texture[2]};
            if (fl & kDgbConst) {
                R[0] = fac * col[0];
                R[1] = fac * col[1];
                R[2] = fac * col[2];
            } else {
                const float kd[3] = {P.kd[3 * m], P.kd[3 * m + 1], P.kd[3 * m + 2]};
                const float ks[3] = {P.ks[3 * m], P.ks[3 * m + 1], P.ks[3 * m + 2]};
                const float s = P.shin[m];
                const F3 x = f3(d2.x, d2.y, d2.z);
                // normal
                const bool flat = (fl & kDgbFlat) != 0;
                F3 N[3] = {f3(0, 0, 0), f3(0, 0, 0), f3(0, 0, 0)};
                const float* M = nullptr;
                F3 mv, n;
                float mlen = 1.0f;
                if (flat) {
                    n = f3(d3.x, d3.y, d3.z);
                } else {
                    M = P.obj_normal + 16 * (size_t)find_obj(P.obj_first, P.n_objects, t);
                    const float b[3] = {d1.x, d1.y, d1.z};
                    mv = f3(0, 0, 0);
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        const float4 v = P.vnor[3 * (size_t)t + k];
                        N[k] = f3(M[0] * v.x + M[1] * v.y + M[2] * v.z + M[3] * v.w,
                                  M[4] * v.x + M[5] * v.y + M[6] * v.z + M[7] * v.w,
                                  M[8] * v.x + M[9] * v.y + M[10] * v.z + M[11] * v.w);
                        mv = mv + b[k] * N[k];
                    }
                    mlen = norm3(mv);
                    n = (1.0f / mlen) * mv;
                }
                float La[3] = {0, 0, 0}, Ld[3] = {0, 0, 0}, Ls[3] = {0, 0, 0};
                for (int e = 0; e < P.n_ambient; e++) {
                    La[0] += P.ambient[e] * col[0];
                    La[1] += P.ambient[e] * col[1];
                    La[2] += P.ambient[e] * col[2];
                }
                const F3 Vd = f3(P.cam[0], P.cam[1], P.cam[2]) - x;
                const F3 V = (1.0f / norm3(Vd)) * Vd;
                // per-light terms, recomputed in the backward pass
                auto light_terms = [&](int l, F3& L, float& I, float& dist, F3& H, float& hlen, float& nd, float& nh,
                                       float& ld, float& ls) {
                    const LightK& Lk = P.lights[l];
                    if (Lk.type == PR_LIGHT_POINT) {
                        const F3 D = f3(Lk.pos[0], Lk.pos[1], Lk.pos[2]) - x;
                        dist = norm3(D);
                        L = (1.0f / dist) * D;
                        I = Lk.intensity / dist;
                    } else {
                        L = f3(-Lk.dir[0], -Lk.dir[1], -Lk.dir[2]);
                        dist = 1.0f;
                        I = Lk.intensity;
                    }
                    const F3 Hv = L + V;
                    hlen = norm3(Hv);
                    H = (1.0f / hlen) * Hv;
                    nd = dot(n, L);
                    nh = dot(n, H);
                    ld = fminf(fmaxf(nd, 0.0f), 1.0f);
                    const float nhc = fminf(fmaxf(nh, 0.0f), 1.0f);
                    ls = nhc > 0.0f ? powf(nhc, s) : 0.0f;
                };
                for (int l = 0; l < P.n_lights; l++) {
                    F3 L, H;
                    float I, dist, hlen, nd, nh, ld, ls;
                    light_terms(l, L, I, dist, H, hlen, nd, nh, ld, ls);
                    const LightK& Lk = P.lights[l];
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        Ld[c] += ld * col[c] * I;
                        Ls[c] += ls * Lk.color[c] * I;
                    }
                }
                float pre[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    pre[c] = La[c] + kd[c] * Ld[c] + ks[c] * Ls[c];
                    R[c] = fac * fminf(fmaxf(pre[c], 0.0f), 255.0f);
                }
                if (BACKWARD) {
                    float gg[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) gg[c] = (pre[c] > 0.0f && pre[c] < 255.0f) ? g[c] * fac : 0.0f;
                    float* A = s_acc + 7 * m;
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        if (gg[c] != 0.0f) {
                            atomicAdd(A + c, gg[c] * Ld[c]);
                            atomicAdd(A + 3 + c, gg[c] * Ls[c]);
                        }
                    }
                    const float gcol = gg[0] * col[0] + gg[1] * col[1] + gg[2] * col[2];
                    float* Aa = s_acc + 7 * P.n_mats + 4 * P.n_lights;
                    if (gcol != 0.0f)
                        for (int e = 0; e < P.n_ambient; e++) atomicAdd(Aa + e, gcol);
                    F3 gn = f3(0, 0, 0);
                    float gshin = 0.0f;
                    for (int l = 0; l < P.n_lights; l++) {
                        F3 L, H;
                        float I, dist, hlen, nd, nh, ld, ls;
                        light_terms(l, L, I, dist, H, hlen, nd, nh, ld, ls);
                        const LightK& Lk = P.lights[l];
                        // loss contribution A ld I + B ls I
                        const float Aw = gg[0] * kd[0] * col[0] + gg[1] * kd[1] * col[1] + gg[2] * kd[2] * col[2];
                        const float Bw = gg[0] * ks[0] * Lk.color[0] + gg[1] * ks[1] * Lk.color[1] +
                                         gg[2] * ks[2] * Lk.color[2];
                        if (Aw == 0.0f && Bw == 0.0f) continue;
                        float* Al = s_acc + 7 * P.n_mats + 4 * l;
                        const float dI = (Aw * ld + Bw * ls) * (Lk.type == PR_LIGHT_POINT ? 1.0f / dist : 1.0f);
                        atomicAdd(Al + 3, dI);
                        const float nhc = fminf(fmaxf(nh, 0.0f), 1.0f);
                        if (ls > 0.0f && nhc < 1.0f) gshin += Bw * I * ls * logf(nhc);
                        const float gnd = (nd > 0.0f && nd < 1.0f) ? Aw * I : 0.0f;
                        const float gnh = (nh > 0.0f && nh < 1.0f) ? Bw * I * s * powf(nhc, s - 1.0f) : 0.0f;
                        gn = gn + gnd * L + gnh * H;
                        if (Lk.type == PR_LIGHT_POINT) {
                            // L(D) through n.L and through H = unit(L + V); I = Il/|D|
                            const F3 gL = gnd * n + (gnh / hlen) * (n - nh * H);
                            const F3 gD = (1.0f / dist) * (gL - dot(L, gL) * L) + (-(Aw * ld + Bw * ls) * I / dist) * L;
                            atomicAdd(Al + 0, gD.x);
                            atomicAdd(Al + 1, gD.y);
                            atomicAdd(Al + 2, gD.z);
                        }
                    }
                    if (gshin != 0.0f) atomicAdd(A + 6, gshin);
                    if (!flat && P.g_vnor) {
                        const F3 gm = (1.0f / mlen) * (gn - dot(n, gn) * n);
                        const float b[3] = {d1.x, d1.y, d1.z};
#pragma unroll
                        for (int k = 0; k < 3; k++) {
                            const F3 gN = b[k] * gm;
                            float* gv = reinterpret_cast<float*>(P.g_vnor + 3 * (size_t)t + k);
#pragma unroll
                            for (int j = 0; j < 3; j++) {
                                const float v = M[j] * gN.x + M[4 + j] * gN.y + M[8 + j] * gN.z;
                                if (v != 0.0f) atomicAdd(gv + j, v);
                            }
                        }
                    }
                }
            }
        }
        if (!BACKWARD) P.radiance[i] = make_float4(R[0], R[1], R[2], alpha);
    }
    if (BACKWARD) {
        __syncthreads();
        for (int k = threadIdx.x; k < n_acc; k += blockDim.x) {
            const float v = s_acc[k];
            if (v != 0.0f) atomicAdd(P.g_acc + k, (double)v);
        }
    }
}

__global__ void col_to_float_kernel(const uchar4* col, float4* out, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uchar4 c = col[i];
        out[i] = make_float4(c.x / 255.0f, c.y / 255.0f, c.z / 255.0f, c.w / 255.0f);
    }
}

int check(cudaError_t e) { return e == cudaSuccess ? 0 : (int)e; }

}  // namespace

namespace {
__global__ void fill_u32_kernel(uint32_t* p, uint32_t v, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}
}  // namespace

int launch_fill_u32(uint32_t* p, uint32_t v, size_t n, void* stream) {
    if (n == 0) return 0;
    const size_t nb = std::min<size_t>((n + 255) / 256, 4096);
    fill_u32_kernel<<<(unsigned)nb, 256, 0, (cudaStream_t)stream>>>(p, v, n);
    return check(cudaGetLastError());
}

int launch_col_to_float(const uchar4* col, float4* out, size_t n, void* stream) {
    if (n == 0) return 0;
    col_to_float_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(col, out, n);
    return check(cudaGetLastError());
}

int launch_diff(const DiffParamsK& p, bool backward, void* stream) {
    const size_t npx = (size_t)p.W * p.H;
    if (npx == 0) return 0;
    const unsigned nb = (unsigned)((npx + kDiffThreads - 1) / kDiffThreads);
    if (backward)
        diff_kernel<true><<<nb, kDiffThreads, 0, (cudaStream_t)stream>>>(p);
    else
        diff_kernel<false><<<nb, kDiffThreads, 0, (cudaStream_t)stream>>>(p);
    return check(cudaGetLastError());
}

}  // namespace prk
