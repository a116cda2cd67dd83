// pr_kernels.cuh — data layout shared by the CUDA kernels (pr_kernels.cu) and
// the host orchestration (pr_api.cpp). Plain C++ so the host compiler can
// include it.
#pragma once

#include <cstddef>
#include <cstdint>

#include <vector_types.h>

#include "../../include/polyred_cuda.h"
#include "pr_texture.h"

namespace prk {

constexpr int kMaxLights = 16;
// Counters of a frame: [0] the main pass, [1 + l] shadow pass l, [kClipCnt]
// the clipped sub-triangles' raster tasks.
constexpr int kClipCnt = kMaxLights + 1;
constexpr int kNumCounters = kMaxLights + 2;
constexpr int kMaxAmbient = 16;
constexpr uint32_t kTaskShift = 5;  // a raster task is a 2^kTaskShift-pixel chunk of a bbox (default)
constexpr uint32_t kNone = 0xFFFFFFFFu;
// Per-triangle flags built at scene upload (tri_flags_kernel)
constexpr uint8_t kTriValid = 1u;  // Triangle.IsValid
constexpr uint8_t kTriAO = 2u;     // its fragments' material has AO (AmbientOcclusionShade runs on them)

// Raster record: what the coverage/depth test of one (sub-)triangle needs.
// 16 words = 64 bytes, read with four 16-byte loads (16-byte aligned so a
// local copy can be stored with vector stores too).
struct alignas(16) RasterRec {
    float v[9];     // screen-space vertices after Viewport + Pos(): x0 y0 z0 x1 y1 z1 x2 y2 z2
    float sabc;     // Barycoord's Sabc = ab.Cross(ac).Z (exact reference bits)
    uint32_t bx;    // x0 | x1 << 16 (pixel bbox clamped to the buffer)
    uint32_t by;    // y0 | y1 << 16
    uint32_t seq;   // draw order: tri*8 + clip sub-index (main view), tri (shadow)
    float recipw[3];  // main view: the parent triangle's -1/W (for attributes computed later)
};
static_assert(sizeof(RasterRec) == 64, "RasterRec is four float4");

// Attribute record: the rest of drawClipped's inputs for one sub-triangle.
// 36 words = 144 bytes.
struct alignas(16) AttrRec {
    float recipw[3];  // parent triangle's -1/W (render/raster.go:403-406, 440-443)
    float nor[9];     // vertex normals after Apply(Normal) (xyz per vertex)
    float uv[6];
    uint32_t col[3];  // RGBA8 per vertex
    float m[9];       // world positions m1..m3 (render/raster.go:467-469), xyz
    float fn[4];      // face normal fN (render/raster.go:479)
    int32_t matid;    // flat material id (<0 = vertex colour)
};
static_assert(sizeof(AttrRec) == 144, "AttrRec is nine float4");

struct Counters {
    uint32_t n_rec;       // records emitted (main view)
    uint32_t n_tasks;     // raster tasks emitted
    uint32_t overflow;    // capacity exceeded (records or tasks)
    uint32_t n_clipped;   // input triangles that were clipped
    uint32_t nan_flag;    // a NaN-depth fragment was produced
    uint32_t n_nan;       // number of NaN-depth fragments
    uint32_t need_rec;    // records needed when overflow
    uint32_t need_tasks;  // tasks needed when overflow
    uint32_t n_ao;        // pixels listed for ambient occlusion
    uint32_t take[2];     // raster work-queue heads: the pass, its NaN fix-up pass
    uint32_t n_vis;       // records listed for their attributes (resolve)
    uint32_t pad[4];
};

struct LightK {
    int32_t type, cast;
    float pos[3], dir[3], intensity;
    float color[3];
    float lview[16], lproj[16];
    int32_t sfast;    // 1: the bottom rows of lview, lproj and the map viewport are exactly (0, 0, 0, 1)
    int32_t pad_[3];
};

// Per-view setup parameters (passed by value).
struct SetupParams {
    const float4* pos;
    const float4* nor;
    const float2* uv;
    const uchar4* col;
    const int32_t* mat;
    const uint32_t* obj_first;   // [n_objects + 1]
    const float* obj_model;      // [n_objects][16]
    const float* obj_trans;      // [n_objects][16] this pass's Proj·View·Model, or null: per-block cache
    uint32_t* attr_state;        // per record: 1 = attributes deferred, 0 = written here; null: no bookkeeping
    int defer_attr;              // 1: leave the attribute record to attr_kernel (visible records only)
    const uint32_t* blk_obj;     // [n_tris / 128] object of each 128-triangle block's first triangle
    const float* obj_normal;     // [n_objects][16] Model.Inv().T()
    const int32_t* obj_matbase;  // [n_objects]
    uint32_t n_tris, n_objects;
    int W, H;                    // target size (framebuffer or shadow map)
    int msaa;                    // render.MSAA: the viewport test and clipping use msaa x (W, H); 0 or 1: (W, H)
    int perspective;
    float pv[16];                // Proj.MulM(View)
    float viewport[16];
    int vp_std;                  // 1: viewport has ViewportMatrix's zero/one pattern (apply_viewport)
    float viewport_inv[16], proj_inv[16], view_inv[16];
    RasterRec* rrec;
    AttrRec* arec;
    uint32_t cap_rec;
    uint2* tasks;
    uint32_t cap_tasks;
    uint32_t* first_rec;
    Counters* cnt;
    float* tri_scr;              // differentiation only: [n_tris][12] screen x, y, recipw per vertex
    uint32_t task_shift = kTaskShift;  // log2 pixels per raster task (<= 16)
    uint32_t* clip_list;         // batched main setup: this view's clip list
    const uint8_t* tri_flags;    // [n_tris] Triangle.IsValid, or null (computed inline)
    Counters* cnt_rec;           // clip: the main pass's counters (records, clip list); null: cnt
};

enum RasterMode { kMain = 0, kMainFixup = 1, kShadow = 2, kShadowFixup = 3 };

struct RasterParams {
    const RasterRec* rrec;
    const uint2* tasks;
    const Counters* cnt;     // n_tasks read on the device
    Counters* cnt_w;
    int W, H;
    int mode;
    unsigned long long* keys;  // main: [H][W] (row r = H-1-y)
    uint32_t* nanseq;          // main: min seq of NaN-depth fragments, kNone if none
    uint32_t* beaten;          // main fix-up: 1 if a finite fragment precedes nanseq
    uint32_t* smap;            // shadow: orderable depth keys, index x + y*W
    uint32_t* lastnan;         // shadow: 1 + max seq of NaN-depth fragments, 0 if none
    uint32_t task_shift = kTaskShift;  // as the setup that wrote the tasks
    uint32_t* take = nullptr;          // zeroed work-queue head (warps take grab tasks at a time), or
                                       // null: a static stride over the tasks
    uint32_t grab = 0;                 // tasks per queue grab, a multiple of 32; 0: from the task count
                                       // (64 below 256 tasks per warp of the grid, else 128)
    // a second task list drained after the first (its own counters and
    // queue head, the same records): the NaN fix-up of the main and the
    // clipped lists in one launch
    const uint2* tasks2 = nullptr;
    const Counters* cnt2 = nullptr;
    uint32_t* take2 = nullptr;
};

struct ShadeParams {
    int W, H;
    uint32_t flags;             // PR_FRAME_*
    const uint32_t* win;        // winning seq per pixel
    const float* depth_ao;      // depth where covered, -1 elsewhere (material/ao.go:57-62)
    const uint32_t* first_rec;
    const RasterRec* rrec;
    const AttrRec* arec;
    const pr_material* mats;
    uint32_t n_mats;
    const int32_t* mat_tex;     // [n_mats] image texture of each material (-1: uniform texel), or null: none
    const prt::TexDesc* tex;    // image textures
    const uint32_t* texels;     // their mipmap levels, packed RGBA8
    int n_lights, n_ambient;
    LightK lights[kMaxLights];
    float ambient[kMaxAmbient];
    float cam[3];
    uint8_t background[4];
    float s2w[16];              // ViewInv.MulM(ProjInv).MulM(ViewportInv)
    float shadow_vp[16];        // ViewportMatrix(SW, SH)
    int SW, SH;
    const uint32_t* smaps;      // [n_lights][SH*SW] orderable keys
    uint8_t gamma[256];
    // outputs (device pointers, may be null)
    uchar4* rgba;
    uint32_t* tri_id;
    float* depth;
    float4* gnor;
    float4* gfnor;
    float4* gwpos;
    float4* guvd;
    uchar4* gvcol;
    int32_t* gmat;
    uint32_t* ao_list;          // pixels whose material has AO (null: AO off)
    int ao_listed;              // 1: resolve lists them; shade only leaves their pre-AO colour
    Counters* cnt_w;
    // differentiation only (null otherwise)
    const float* tri_scr;       // [n_tris][12] from the main setup
    float4* dgb;                // [H][W][4] differentiation G-buffer
};

// Differentiation G-buffer pixel flags (float4 0, .z)
constexpr uint32_t kDgbLit = 1u, kDgbFlat = 2u, kDgbConst = 4u, kDgbUnlit = 8u;

struct AoParams {
    int W, H;
    int gamma_on;
    int n_dirs;
    const float* depth;         // depth_ao
    const uint32_t* list;
    const Counters* cnt;
    uchar4* rgba;
    uint8_t gamma[256];
    int8_t dir_fast[8];  // 1: the tap offset table is exact for this frame size
    int8_t dir_tiny[8];  // 1 / 2: the x / y component lies in (-1/99, 0)
    float ao_half_ulp;   // half an ulp of float32 at max(W, H) + 100
    float4* dgb;         // differentiation only: multiply the G-buffer's factor by the AO factor
    float* T;            // [list] the AO total of each listed pixel (ao_T_kernel -> ao_apply_kernel)
};


// Differentiable shading (pr_diff.cu)
constexpr int kDiffMaxMats = 256;
struct DiffParamsK {
    int W, H;
    const float4* dgb;
    const float4* vcol;          // [n_tris*3] RGBA in [0,1]
    const float4* vnor;          // [n_tris*3] object-space normals
    const uint32_t* obj_first;
    uint32_t n_objects;
    const float* obj_normal;     // [n_objects][16]
    int n_mats;
    const float* kd;             // [n_mats][3]
    const float* ks;             // [n_mats][3]
    const float* shin;           // [n_mats]
    const pr_material* mats;     // texture texel, flags
    int n_lights, n_ambient;
    LightK lights[kMaxLights];
    float ambient[kMaxAmbient];
    float cam[3];
    float bg[4];
    float4* radiance;            // forward output
    const float4* grad;          // backward input
    float4* g_vcol;              // backward outputs (may be null)
    float4* g_vnor;
    double* g_acc;               // [n_mats*7 + n_lights*4 + n_ambient]: kd3 ks3 shin | pos3 I | ambient
};

}  // namespace prk

// Launch wrappers implemented in pr_kernels.cu (host-callable).
namespace prk {
int launch_setup_main_only(const SetupParams& p, uint32_t* clip_list, void* stream);
int launch_clip(const SetupParams& p, const uint32_t* clip_list, void* stream);
// Proj·View·Model of every object for n_pass passes: out[pass][o][16] from
// the passes' Proj·View (pv[pass]) in Mat4.MulM's order.
constexpr int kMaxPasses = kMaxLights + 1;
struct PassMats {
    float pv[kMaxPasses][16];
};
int launch_obj_trans(const PassMats& pm, int n_pass, const float* obj_model, uint32_t n_objects, float* out,
                     void* stream);
// Resolve that also lists, once each, the winning records whose attributes
// were deferred (attr_state 1 -> 2) in vis (count in cnt->n_vis), puts the
// NaN bookkeeping (nanseq, beaten) back to kNone / 0 after a frame that used
// it, and, with
// ao_list, the pixels whose winner's material has AO (tri_flags kTriAO) in
// ao_list (count in cnt->n_ao), tile by tile (32 x 8).
int launch_resolve_listing(int W, int H, const unsigned long long* keys, uint32_t* nanseq, uint32_t* beaten,
                           Counters* cnt, uint32_t* win, float* depth_ao, const uint32_t* first_rec,
                           uint32_t* attr_state, uint32_t* vis, const uint8_t* tri_flags, uint32_t* ao_list,
                           void* stream);
// The attribute records of the records resolve listed (P: the main view's setup parameters).
int launch_attr(const SetupParams& p, const uint32_t* vis, void* stream);
int launch_setup_shadow(const SetupParams& p, void* stream);
int launch_raster(const RasterParams& p, int n_blocks, void* stream);
int launch_shadow_fixup_reset(int W, int H, const uint32_t* lastnan, uint32_t* smap, const Counters* cnt,
                              void* stream);
// After a pass that saw a NaN fragment (cnt->nan_flag): a[0..n) = va and, if b, b[0..n) = vb.
int launch_nan_cleanup(size_t n, uint32_t* a, uint32_t va, uint32_t* b, uint32_t vb, const Counters* cnt,
                       void* stream);
int launch_shade(const ShadeParams& p, void* stream);
// AO split so that its march overlaps shading: the list (made by resolve),
// the march writing p.T (after resolve), and the colour scaling and gamma
// of the listed pixels (after both the march and shading).
int launch_ao_T(const AoParams& p, void* stream);
int launch_ao_apply(const AoParams& p, int n_blocks, void* stream);
// passAntialiasing's imageutil.Resize of the n*W x n*H image `in` to W x H
// (rows top-down, both buffers on the device).
int launch_msaa_resize(const uchar4* in, int in_w, int in_h, uchar4* out, int w, int h, void* stream);
int launch_diff(const DiffParamsK& p, bool backward, void* stream);

// ---- batches: many passes (views, shadow maps) per launch ----
struct ResolveParams {
    int W, H;
    const unsigned long long* keys;
    const uint32_t* nanseq;
    const uint32_t* beaten;
    const Counters* cnt;
    uint32_t* win;
    float* depth_ao;
};
// Job j of a launch owns blocks [blk[j], blk[j+1]); blk has n_jobs + 1 entries.
int launch_setup_shadow_batch(const SetupParams* jobs, const uint32_t* blk, int n_jobs, uint32_t n_blocks, void* stream);
int launch_setup_main_batch(const SetupParams* jobs, const uint32_t* blk, int n_jobs, uint32_t n_blocks, void* stream);
int launch_clip_batch(const SetupParams* jobs, const uint32_t* blk, int n_jobs, uint32_t n_blocks, void* stream);
// Per-pass work items (warp batches of 32 tasks) prefixed into items[n_jobs + 1]
// on the device; fixup: only passes with NaN fragments. Also clears *queue.
int launch_batch_scan(const RasterParams* jobs, int n_jobs, uint32_t* items, uint32_t* queue, int fixup, void* stream);
// One persistent launch over the global queue of (pass, warp batch) items.
int launch_raster_batch(const RasterParams* jobs, const uint32_t* items, int n_jobs, uint32_t* queue, int n_blocks,
                        void* stream);
int launch_resolve_batch(const ResolveParams* jobs, const uint32_t* blk, int n_jobs, uint32_t n_blocks, void* stream);
int launch_shade_batch(const ShadeParams* views, const uint32_t* blk, int n_views, uint32_t n_blocks, void* stream);
// Persistent; chunk counters [n_views] zeroed by the caller.
int launch_ao_batch(const AoParams* views, int n_views, uint32_t* chunk_ctr, int n_blocks, void* stream);
int launch_col_to_float(const uchar4* col, float4* out, size_t n, void* stream);
int launch_fill_u32(uint32_t* p, uint32_t v, size_t n, void* stream);
// Triangle.IsValid (kTriValid) and the AO flag of each triangle's material (kTriAO).
int launch_tri_flags(const float4* pos, uint32_t n, uint8_t* flags, const int32_t* mat, const uint32_t* obj_first,
                     const uint32_t* blk_obj, const int32_t* obj_matbase, uint32_t n_objects, const pr_material* mats,
                     uint32_t n_mats, void* stream);
int set_ao_tables(const float* cosv, const float* sinv, int n, void* stream);
int launch_decode_shadow(const uint32_t* smap, float* out, size_t n, void* stream);
int launch_pow_probe(const float* x, const float* y, float* fast, float* ref, int n, void* stream);
int launch_ao_probe(const float* x, float* atan_fast, float* atan_ref, const float* T, const void* col, void* o_fast,
                    void* o_ref, int n, void* stream);
int launch_fma_probe(const float* a, const float* b, const float* c, float* out, float* out_ref, int n,
                     void* stream);
int sm_count();
// Records a status and its detail as the calling thread's last error.
int set_last_error(int status, const char* msg);
}  // namespace prk
