// pr_api.cpp — the C ABI of libpolyred_cuda.so: contexts, scene upload,
// frame orchestration on one CUDA stream, output copies, host math helpers.
// Compiled with -ffp-contract=off (host float32 math must match the
// reference's Go evaluation bit for bit).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/polyred_cuda.h"
#include "../../include/polyred_cuda_testing.h"
#include "pr_hostmath.h"
#include "pr_kernels.cuh"

using prh::M4;

namespace prh {
int build_texture(int w, int h, const uint8_t* rgba, bool mipmap, std::vector<uint32_t>& texels, prt::TexDesc& d);
}

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CUDA_TRY(expr)                                                                          \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess)                                                                  \
            return fail(_e == cudaErrorMemoryAllocation ? PR_ERR_OOM : PR_ERR_CUDA, "%s: %s (%s:%d)", \
                        #expr, cudaGetErrorString(_e), __FILE__, __LINE__);                     \
    } while (0)

#define KTRY(expr)                                                                    \
    do {                                                                              \
        int _e = (expr);                                                              \
        if (_e != 0)                                                                  \
            return fail(PR_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString((cudaError_t)_e)); \
    } while (0)

// Allocation failure injection (pr_testing_fail_alloc): when positive, the
// number of device or page-locked allocations until one reports
// cudaErrorMemoryAllocation without calling CUDA. g_alloc_count counts every
// allocation attempt (pr_testing_alloc_count).
std::atomic<long long> g_alloc_fail_in{0};
std::atomic<long long> g_alloc_count{0};

bool injected_failure() {
    g_alloc_count.fetch_add(1, std::memory_order_relaxed);
    long long k = g_alloc_fail_in.load();
    while (k > 0)
        if (g_alloc_fail_in.compare_exchange_weak(k, k - 1)) return k == 1;
    return false;
}

cudaError_t dev_malloc(void** p, size_t bytes) {
    if (injected_failure()) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

cudaError_t host_malloc(void** p, size_t bytes) {
    if (injected_failure()) return cudaErrorMemoryAllocation;
    return cudaHostAlloc(p, bytes, cudaHostAllocDefault);
}

// A device allocation that only grows. A failed growth leaves it empty
// (p == nullptr, n == 0): the old buffer is freed first, so that the peak
// holds one buffer, and callers keep no capacity derived from it.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    int ensure(size_t want) {
        if (want <= n && p) return PR_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t alloc = std::max<size_t>(want, 1);
        cudaError_t e = dev_malloc((void**)&p, alloc * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(PR_ERR_OOM, "cudaMalloc(%zu bytes): %s", alloc * sizeof(T), cudaGetErrorString(e));
        }
        n = alloc;
        return PR_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

// Page-locked host memory that grows on demand.
struct HostBuf {
    uint8_t* p = nullptr;
    size_t n = 0;
    int ensure(size_t want) {
        if (want <= n && p) return PR_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (host_malloc((void**)&p, std::max<size_t>(want, 1)) != cudaSuccess) {
            p = nullptr;
            return fail(PR_ERR_OOM, "cudaHostAlloc(%zu bytes) failed", want);
        }
        n = std::max<size_t>(want, 1);
        return PR_OK;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
};

// One device copy of a scene: the triangle arrays, the per-object tables,
// the material table and the Triangle.IsValid flags. A context holds two, so
// that pr_frame_submit can fill one while the frame in flight reads the other.
struct SceneBufs {
    uint32_t n_tris = 0;
    std::vector<pr_object> objects;
    std::vector<pr_material> materials;
    DevBuf<float4> pos, nor;
    DevBuf<float2> uv;
    DevBuf<uchar4> col;
    DevBuf<int32_t> mat;
    DevBuf<uint32_t> obj_first;
    DevBuf<uint8_t> tri_flags;  // Triangle.IsValid per input triangle
    DevBuf<float> obj_model, obj_normal;
    DevBuf<int32_t> obj_matbase;
    DevBuf<pr_material> dmats;
    DevBuf<uint32_t> blk_obj;              // object of the first triangle of each 128-triangle block
    DevBuf<uint32_t> texels;               // image textures: every mipmap level, packed RGBA8
    DevBuf<prt::TexDesc> tex;
    DevBuf<int32_t> mat_tex;               // [n_materials] texture of each material, -1: uniform
    bool has_tex = false;
    bool has_ao = false;                   // a material has ambient occlusion
    HostBuf tables;                        // page-locked staging of the small tables (submitted uploads)
    cudaEvent_t ev_uploaded = nullptr;     // the upload into these buffers has landed
    cudaEvent_t ev_released = nullptr;     // the last frame that read them is past shading
    cudaEvent_t ev_released_ao = nullptr;  // ... and past the frame's AO stream work (stream 3)
    void release() {
        pos.release(); nor.release(); uv.release(); col.release(); mat.release();
        obj_first.release(); tri_flags.release(); obj_model.release(); obj_normal.release();
        obj_matbase.release(); dmats.release(); blk_obj.release(); tables.release();
        texels.release(); tex.release(); mat_tex.release();
        has_tex = has_ao = false;
        if (ev_uploaded) cudaEventDestroy(ev_uploaded);
        if (ev_released) cudaEventDestroy(ev_released);
        if (ev_released_ao) cudaEventDestroy(ev_released_ao);
        ev_uploaded = ev_released = ev_released_ao = nullptr;
    }
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    // scene: sb is the one frames read; pr_frame_submit fills sb_back, then swaps
    bool has_scene = false;
    SceneBufs sb, sb_back;
    // submitted frames: scene uploads and host-output copies on their own streams
    cudaStream_t stream_u = nullptr, stream_d = nullptr;
    cudaEvent_t ev_frame = nullptr, ev_d2h = nullptr;
    // raster work space
    DevBuf<prk::RasterRec> rrec;
    DevBuf<prk::AttrRec> arec;
    DevBuf<uint2> tasks;
    DevBuf<uint32_t> first_rec, clip_list;
    DevBuf<uint32_t> attr_state, vis_list;  // deferred attribute records: per-record state, visible list
    uint32_t cap_rec = 0, cap_tasks = 0;
    // framebuffer
    int W = 0, H = 0;
    DevBuf<float> obj_trans;  // [1 + lights][n_objects][16]: Proj·View·Model per pass and object
    DevBuf<unsigned long long> keys;
    DevBuf<uint32_t> nanseq, beaten, win;
    DevBuf<float> depth_ao;
    DevBuf<uint32_t> ao_list;
    int n_ao_dirs = 0;
    float ao_cos[8] = {}, ao_sin[8] = {};
    // shadow maps (persistent across frames)
    int SW = 0, SH = 0, n_slights = 0;
    DevBuf<uint32_t> smap, lastnan;
    bool smap_valid = false;
    DevBuf<prk::Counters> cnt;  // [kNumCounters]
    prk::Counters* h_cnt = nullptr;  // pinned mirror
    // staging for host outputs
    DevBuf<uint8_t> o_rgba, o_vcol, o_msaa;
    DevBuf<uint32_t> o_tri;
    DevBuf<float> o_depth, o_shadow;
    DevBuf<float4> o_nor, o_fnor, o_wpos, o_uvd;
    DevBuf<int32_t> o_mat;
    // differentiable shading
    DevBuf<float> tri_scr;                 // [n_tris][12]
    DevBuf<float> d_kd, d_ks, d_shin;      // [n_mats][3], [n_mats][3], [n_mats]
    DevBuf<float4> d_vcol;                 // scene colours / 255, when the caller gives none
    DevBuf<double> d_acc;
    pr_stats stats{};
    cudaEvent_t ev[6] = {};
    // shadow passes run on their own stream, with their own records and tasks
    cudaStream_t stream_s = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    DevBuf<prk::RasterRec> rrec_s;
    DevBuf<uint2> tasks_s;
    // clipped sub-triangles: clipped and rasterised on a third stream beside the main raster
    cudaStream_t stream_c = nullptr;
    cudaEvent_t ev_setup = nullptr, ev_clip = nullptr;
    DevBuf<uint2> tasks_c;
    // AO's march on stream 3 beside attributes and shading: after resolve,
    // joined before the AO colour scaling
    cudaEvent_t ev_resolved = nullptr, ev_ao0 = nullptr, ev_ao = nullptr;
    bool ao_marched = false;  // the last frame ran the AO march (ev_ao0, ev_ao hold it)
    DevBuf<float> ao_T;
    int n_sms = 1;
};

int set_device(Ctx* c) { CUDA_TRY(cudaSetDevice(c->device)); return PR_OK; }

M4 loadm(const float* p) {
    M4 m;
    std::memcpy(m.m, p, 64);
    return m;
}

// The image textures of a scene descriptor (NULL for descriptors without the field).
const pr_texture* scene_textures(const pr_scene_desc* s) {
    return s->size >= offsetof(pr_scene_desc, textures) + sizeof(void*) ? s->textures : nullptr;
}

bool scene_has_images(const pr_scene_desc* s) {
    const pr_texture* t = scene_textures(s);
    for (uint32_t m = 0; t && m < s->n_materials; m++)
        if (t[m].rgba) return true;
    return false;
}

int validate_scene(const pr_scene_desc* s) {
    if (!s) return fail(PR_ERR_INVALID_ARG, "scene is NULL");
    if (s->size < PR_SCENE_DESC_SIZE_V1) return fail(PR_ERR_INVALID_ARG, "scene->size %u < %u", s->size, PR_SCENE_DESC_SIZE_V1);
    if (s->n_tris > 0 && (!s->pos || !s->nor || !s->uv || !s->col || !s->mat_id))
        return fail(PR_ERR_INVALID_ARG, "scene arrays must be non-NULL when n_tris > 0");
    if (s->n_tris >= (1u << 29)) return fail(PR_ERR_INVALID_ARG, "n_tris %u exceeds 2^29 (draw-order key limit)", s->n_tris);
    if (s->n_objects == 0 && s->n_tris > 0) return fail(PR_ERR_INVALID_ARG, "triangles without objects");
    if (s->n_objects > 0 && !s->objects) return fail(PR_ERR_INVALID_ARG, "objects is NULL");
    if (s->n_materials > 0 && !s->materials) return fail(PR_ERR_INVALID_ARG, "materials is NULL");
    uint64_t expect = 0;
    for (uint32_t o = 0; o < s->n_objects; o++) {
        if (s->objects[o].first_tri != expect)
            return fail(PR_ERR_INVALID_ARG, "object %u: first_tri %u, expected %llu (objects must tile the soup in order)",
                        o, s->objects[o].first_tri, (unsigned long long)expect);
        expect += s->objects[o].n_tris;
        if (expect > s->n_tris)
            return fail(PR_ERR_INVALID_ARG, "object %u ends past the scene's %u triangles", o, s->n_tris);
    }
    if (expect != s->n_tris)
        return fail(PR_ERR_INVALID_ARG, "objects cover %llu triangles, scene has %u", (unsigned long long)expect, s->n_tris);
    const pr_texture* tx = scene_textures(s);
    for (uint32_t m = 0; m < s->n_materials; m++) {
        if (tx && tx[m].rgba) {
            if (tx[m].width < 1 || tx[m].height < 1 || tx[m].width > 16384 || tx[m].height > 16384)
                return fail(PR_ERR_INVALID_ARG, "material %u: texture %dx%d outside 1..16384", m, tx[m].width, tx[m].height);
        } else if (s->materials[m].texture_size != 1) {
            return fail(PR_ERR_UNSUPPORTED, "material %u: texture_size %d without an image", m, s->materials[m].texture_size);
        }
    }
    return PR_OK;
}

template <class T>
int upload(DevBuf<T>& b, const void* src, size_t n, bool dev_src, cudaStream_t st) {
    int rc = b.ensure(n);
    if (rc) return rc;
    if (n == 0) return PR_OK;
    CUDA_TRY(cudaMemcpyAsync(b.p, src, n * sizeof(T), dev_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    return PR_OK;
}

// Copy a scene into b on stream st: the triangle arrays, the per-object
// Model and Normal = Model.Inv().T() (render/raster.go:242-243), the
// material table, and the Triangle.IsValid flags. staged: the small host
// tables go through b's page-locked staging, so nothing waits for the copy;
// otherwise the caller synchronises st before they go out of scope.
int scene_fill(SceneBufs& b, const pr_scene_desc* s, cudaStream_t st, bool staged) {
    int rc;
    const bool dev = (s->flags & PR_SCENE_DEVICE_PTRS) != 0;
    const uint32_t n = s->n_tris, no = s->n_objects, nm = s->n_materials;
    std::vector<uint32_t> first(no + 1);
    std::vector<float> model((size_t)no * 16), normal((size_t)no * 16);
    std::vector<int32_t> mb(no);
    for (uint32_t o = 0; o < no; o++) {
        first[o] = s->objects[o].first_tri;
        M4 m = loadm(s->objects[o].model), mi;
        if (!prh::inv(m, &mi)) return fail(PR_ERR_SINGULAR, "object %u: model matrix is singular", o);
        M4 nm4 = prh::transpose(mi);
        std::memcpy(&model[(size_t)o * 16], m.m, 64);
        std::memcpy(&normal[(size_t)o * 16], nm4.m, 64);
        mb[o] = s->objects[o].mat_base;
    }
    first[no] = n;
    // object of each 128-triangle block's first triangle (the last object starting at or before it)
    const uint32_t nblk = (n + 127) / 128;
    std::vector<uint32_t> blk(std::max<uint32_t>(nblk, 1), 0u);
    for (uint32_t k = 0, o = 0; k < nblk; k++) {
        while (o + 1 < no && first[o + 1] <= k * 128u) o++;
        blk[k] = o;
    }
    if ((rc = upload(b.pos, s->pos, (size_t)n * 3, dev, st))) return rc;
    if ((rc = upload(b.nor, s->nor, (size_t)n * 3, dev, st))) return rc;
    if ((rc = upload(b.uv, s->uv, (size_t)n * 3, dev, st))) return rc;
    if ((rc = upload(b.col, s->col, (size_t)n * 3, dev, st))) return rc;
    if ((rc = upload(b.mat, s->mat_id, (size_t)n, dev, st))) return rc;
    const void* t_first = first.data();
    const void* t_model = model.data();
    const void* t_normal = normal.data();
    const void* t_mb = mb.data();
    const void* t_mats = s->materials;
    const void* t_blk = blk.data();
    if (staged) {
        auto al = [](size_t v) { return (v + 15) & ~(size_t)15; };
        const size_t o_first = 0, o_model = al(o_first + first.size() * 4), o_normal = o_model + model.size() * 4,
                     o_mb = o_normal + normal.size() * 4, o_mats = al(o_mb + mb.size() * 4),
                     o_blk = al(o_mats + (size_t)nm * sizeof(pr_material)), total = o_blk + blk.size() * 4;
        if ((rc = b.tables.ensure(total))) return rc;
        uint8_t* h = b.tables.p;
        std::memcpy(h + o_first, first.data(), first.size() * 4);
        std::memcpy(h + o_model, model.data(), model.size() * 4);
        std::memcpy(h + o_normal, normal.data(), normal.size() * 4);
        std::memcpy(h + o_mb, mb.data(), mb.size() * 4);
        if (nm) std::memcpy(h + o_mats, s->materials, (size_t)nm * sizeof(pr_material));
        std::memcpy(h + o_blk, blk.data(), blk.size() * 4);
        t_blk = h + o_blk;
        t_first = h + o_first;
        t_model = h + o_model;
        t_normal = h + o_normal;
        t_mb = h + o_mb;
        t_mats = h + o_mats;
    }
    if ((rc = upload(b.obj_first, t_first, first.size(), false, st))) return rc;
    if ((rc = upload(b.obj_model, t_model, model.size(), false, st))) return rc;
    if ((rc = upload(b.obj_normal, t_normal, normal.size(), false, st))) return rc;
    if ((rc = upload(b.obj_matbase, t_mb, mb.size(), false, st))) return rc;
    if ((rc = upload(b.dmats, t_mats, nm, false, st))) return rc;
    if ((rc = upload(b.blk_obj, t_blk, blk.size(), false, st))) return rc;
    if ((rc = b.tri_flags.ensure(std::max<uint32_t>(n, 1)))) return rc;
    KTRY(prk::launch_tri_flags(b.pos.p, n, b.tri_flags.p, b.mat.p, b.obj_first.p, b.blk_obj.p, b.obj_matbase.p, no,
                               b.dmats.p, nm, st));
    // image textures: NewTexture's levels built here, once per upload
    b.has_tex = false;
    if (scene_has_images(s)) {
        const pr_texture* tx = scene_textures(s);
        std::vector<uint32_t> texels;
        std::vector<prt::TexDesc> descs;
        std::vector<int32_t> mat_tex(nm, -1);
        try {
            for (uint32_t m = 0; m < nm; m++) {
                if (!tx[m].rgba) continue;
                prt::TexDesc d;
                if (prh::build_texture(tx[m].width, tx[m].height, tx[m].rgba, (s->materials[m].flags & PR_MAT_MIPMAP) != 0,
                                       texels, d))
                    return fail(PR_ERR_INVALID_ARG, "material %u: texture %dx%d rejected", m, tx[m].width, tx[m].height);
                if (texels.size() >= (1ull << 32)) return fail(PR_ERR_INVALID_ARG, "textures exceed 2^32 texels");
                mat_tex[m] = (int32_t)descs.size();
                descs.push_back(d);
            }
        } catch (const std::bad_alloc&) {
            return fail(PR_ERR_OOM, "host allocation failed while building texture mipmaps");
        }
        // pageable sources: each copy has left them when cudaMemcpyAsync returns
        if ((rc = upload(b.texels, texels.data(), texels.size(), false, st))) return rc;
        if ((rc = upload(b.tex, descs.data(), descs.size(), false, st))) return rc;
        if ((rc = upload(b.mat_tex, mat_tex.data(), mat_tex.size(), false, st))) return rc;
        b.has_tex = true;
    }
    b.objects.assign(s->objects, s->objects + no);
    b.materials.assign(s->materials, s->materials + nm);
    b.has_ao = false;
    for (uint32_t m = 0; m < nm; m++) b.has_ao |= (s->materials[m].flags & PR_MAT_AO) != 0;
    b.n_tris = n;
    return PR_OK;
}

int ensure_frame(Ctx* c, int W, int H) {
    size_t n = (size_t)W * H;
    int rc;
    if ((rc = c->keys.ensure(n))) return rc;
    // nanseq / beaten start all-kNone / all-0 and are put back so after any
    // frame that used them, so a new allocation is set once
    const size_t n0 = c->nanseq.n, b0 = c->beaten.n;
    if ((rc = c->nanseq.ensure(n))) return rc;
    if ((rc = c->beaten.ensure(n))) return rc;
    if (c->nanseq.n != n0) CUDA_TRY(cudaMemsetAsync(c->nanseq.p, 0xff, c->nanseq.n * 4, c->stream));
    if (c->beaten.n != b0) CUDA_TRY(cudaMemsetAsync(c->beaten.p, 0, c->beaten.n * 4, c->stream));
    if ((rc = c->win.ensure(n))) return rc;
    if ((rc = c->depth_ao.ensure(n))) return rc;
    if ((rc = c->ao_list.ensure(n))) return rc;
    c->W = W;
    c->H = H;
    return PR_OK;
}

int ensure_work(Ctx* c, uint32_t need_rec, uint32_t need_tasks) {
    int rc;
    if (need_rec > c->cap_rec) {
        uint32_t cap = std::max(need_rec, c->cap_rec * 2);
        c->cap_rec = 0;  // until every buffer holds cap (a failed growth empties one)
        if ((rc = c->rrec.ensure(cap))) return rc;
        if ((rc = c->arec.ensure(cap))) return rc;
        if ((rc = c->attr_state.ensure(cap))) return rc;
        if ((rc = c->vis_list.ensure(cap))) return rc;
        if ((rc = c->rrec_s.ensure(cap))) return rc;
        c->cap_rec = cap;
    }
    if (need_tasks > c->cap_tasks) {
        uint32_t cap = std::max(need_tasks, c->cap_tasks * 2);
        c->cap_tasks = 0;
        if ((rc = c->tasks.ensure(cap))) return rc;
        if ((rc = c->tasks_s.ensure(cap))) return rc;
        if ((rc = c->tasks_c.ensure(cap))) return rc;
        c->cap_tasks = cap;
    }
    return PR_OK;
}

// ViewportMatrix's pattern (pr_hostmath viewport): zeros and ones where
// apply_viewport relies on them.
int viewport_std(const float* m) {
    for (int e : {1, 2, 4, 6, 8, 9, 11, 12, 13, 14})
        if (m[e] != 0.0f) return 0;
    return (m[10] == 1.0f && m[15] == 1.0f) ? 1 : 0;
}

void fill_scene_ptrs(Ctx* c, prk::SetupParams& p) {
    p.pos = c->sb.pos.p;
    p.nor = c->sb.nor.p;
    p.uv = c->sb.uv.p;
    p.col = c->sb.col.p;
    p.mat = c->sb.mat.p;
    p.obj_first = c->sb.obj_first.p;
    p.obj_model = c->sb.obj_model.p;
    p.obj_normal = c->sb.obj_normal.p;
    p.obj_matbase = c->sb.obj_matbase.p;
    p.tri_flags = c->sb.tri_flags.p;
    p.blk_obj = c->sb.blk_obj.p;
    p.n_tris = c->sb.n_tris;
    p.n_objects = (uint32_t)c->sb.objects.size();
}

// render.MSAA of a frame: 1 for descriptors without the field or with 0 / 1.
int frame_msaa(const pr_frame_desc* f) {
    return (f->size >= offsetof(pr_frame_desc, msaa) + sizeof(int32_t) && f->msaa > 1) ? f->msaa : 1;
}

int validate_frame(const Ctx* c, const pr_frame_desc* f) {
    if (!f) return fail(PR_ERR_INVALID_ARG, "frame is NULL");
    if (f->size < PR_FRAME_DESC_SIZE_V1) return fail(PR_ERR_INVALID_ARG, "frame->size %u < %u", f->size, PR_FRAME_DESC_SIZE_V1);
    if (f->size >= offsetof(pr_frame_desc, msaa) + sizeof(int32_t) && (f->msaa < 0 || f->msaa > 16))
        return fail(PR_ERR_INVALID_ARG, "msaa %d outside 0..16", f->msaa);
    const int64_t m = frame_msaa(f);
    if (f->width <= 0 || f->height <= 0 || f->width * m > 16384 || f->height * m > 16384)
        return fail(PR_ERR_INVALID_ARG, "framebuffer %lldx%lld (size %dx%d, msaa %lld) outside 1..16384",
                    (long long)(f->width * m), (long long)(f->height * m), f->width, f->height, (long long)m);
    if (f->n_lights > (uint32_t)prk::kMaxLights) return fail(PR_ERR_UNSUPPORTED, "%u lights > %d", f->n_lights, prk::kMaxLights);
    if (f->n_ambient > (uint32_t)prk::kMaxAmbient)
        return fail(PR_ERR_UNSUPPORTED, "%u ambient lights > %d", f->n_ambient, prk::kMaxAmbient);
    if (f->n_lights > 0 && !f->lights) return fail(PR_ERR_INVALID_ARG, "lights is NULL");
    if (f->n_ambient > 0 && !f->ambient) return fail(PR_ERR_INVALID_ARG, "ambient is NULL");
    int sw = f->shadow_width > 0 ? f->shadow_width : f->width;
    int sh = f->shadow_height > 0 ? f->shadow_height : f->height;
    if (sw > 16384 || sh > 16384) return fail(PR_ERR_INVALID_ARG, "shadow map %dx%d too large", sw, sh);
    (void)c;
    return PR_OK;
}

// Counters and per-phase device times of the last frame; the stream must
// have passed the frame's last event.
void collect_stats(Ctx* c) {
    c->stats.n_raster_tris = c->h_cnt[0].n_rec;
    c->stats.n_clipped_tris = c->h_cnt[0].n_clipped;
    c->stats.n_nan_fragments = c->h_cnt[0].n_nan;
    uint32_t n_tasks = 0;
    for (int k = 0; k < prk::kNumCounters; k++) n_tasks += c->h_cnt[k].n_tasks;
    c->stats.n_raster_tasks = n_tasks;
    // 0 for an interval whose events a failed frame did not record; the
    // error that reports it must not be left for the next launch check
    auto span = [](cudaEvent_t a, cudaEvent_t b) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
            (void)cudaGetLastError();
            ms = 0;
        }
        return ms;
    };
    c->stats.ms_shadow = span(c->ev[0], c->ev[1]);
    c->stats.ms_setup = span(c->ev[0], c->ev[2]);  // concurrent with the shadow passes
    c->stats.ms_raster = span(c->ev[2], c->ev[3]);
    c->stats.ms_shade = span(c->ev[3], c->ev[4]);
    c->stats.ms_total = span(c->ev[0], c->ev[4]);
    c->stats.ms_ao = c->ao_marched ? span(c->ev_ao0, c->ev_ao) : 0.0f;  // the march, beside shading
    c->stats.n_ao_pixels = c->h_cnt[0].n_ao;
}

// Launch checks read cudaGetLastError, which also holds a failure of any
// earlier runtime call of this host thread that nothing consumed (the
// caller's own, for one). Each entry point that launches starts by
// consuming it, so that it is not reported as the library's. A sticky
// error (a fault of the context) survives this and fails the next call.
void clear_stale_error() { (void)cudaGetLastError(); }

// The frame-level fields of the deferred pass: size, flags, materials,
// lights (render/raster.go:275-295), camera, background, matrices, gamma.
void fill_shade_frame(const Ctx* c, const pr_frame_desc* f, const M4& s2w, int SW, int SH, prk::ShadeParams& sp) {
    if (c->sb.has_tex) {
        sp.mat_tex = c->sb.mat_tex.p;
        sp.tex = c->sb.tex.p;
        sp.texels = c->sb.texels.p;
    }
    sp.W = f->width;
    sp.H = f->height;
    sp.flags = f->flags;
    sp.mats = c->sb.dmats.p;
    sp.n_mats = (uint32_t)c->sb.materials.size();
    sp.n_lights = (int)f->n_lights;
    sp.n_ambient = (int)f->n_ambient;
    for (uint32_t l = 0; l < f->n_lights; l++) {
        const pr_light& L = f->lights[l];
        prk::LightK& K = sp.lights[l];
        K.type = L.type;
        K.cast = L.cast_shadow ? 1 : 0;
        for (int k = 0; k < 3; k++) {
            K.pos[k] = L.pos[k];
            K.dir[k] = L.dir[k];
            K.color[k] = (float)L.color[k];
        }
        K.intensity = L.intensity;
        std::memcpy(K.lview, L.shadow_view, 64);
        std::memcpy(K.lproj, L.shadow_proj, 64);
    }
    for (uint32_t e = 0; e < f->n_ambient; e++) sp.ambient[e] = f->ambient[e];
    for (int k = 0; k < 3; k++) sp.cam[k] = f->cam_pos[k];
    std::memcpy(sp.background, f->background, 4);
    std::memcpy(sp.s2w, s2w.m, 64);
    M4 svp = prh::viewport((float)SW, (float)SH);
    std::memcpy(sp.shadow_vp, svp.m, 64);
    auto unit_bottom = [](const float* m) { return m[12] == 0.0f && m[13] == 0.0f && m[14] == 0.0f && m[15] == 1.0f; };
    for (uint32_t l = 0; l < f->n_lights; l++) {
        prk::LightK& K = sp.lights[l];
        K.sfast = unit_bottom(K.lview) && unit_bottom(K.lproj) && unit_bottom(svp.m) ? 1 : 0;
    }
    sp.SW = SW;
    sp.SH = SH;
    prh::gamma_table(sp.gamma);
}

// Matrices of a frame (render/raster.go:232-246, 281-295).
struct FrameMats {
    M4 pv, vp, vp_inv, proj_inv, view_inv, s2w;
};
int frame_mats(const pr_frame_desc* f, FrameMats& m) {
    M4 view = loadm(f->view), proj = loadm(f->proj);
    m.vp = prh::viewport((float)f->width, (float)f->height);
    if (!prh::inv(view, &m.view_inv)) return fail(PR_ERR_SINGULAR, "view matrix is singular");
    if (!prh::inv(proj, &m.proj_inv)) return fail(PR_ERR_SINGULAR, "projection matrix is singular");
    if (!prh::inv(m.vp, &m.vp_inv)) return fail(PR_ERR_SINGULAR, "viewport matrix is singular");
    m.pv = prh::mulm(proj, view);
    m.s2w = prh::mulm(prh::mulm(m.view_inv, m.proj_inv), m.vp_inv);
    return PR_OK;
}

// The requested outputs from the staging buffers to the caller's host memory
// (the image has npx_rgba pixels, the framebuffer fields npx).
int copy_host_outputs(Ctx* c, const pr_outputs* out, size_t npx, size_t npx_rgba, cudaStream_t st) {
    if (out->rgba) CUDA_TRY(cudaMemcpyAsync(out->rgba, c->o_rgba.p, npx_rgba * 4, cudaMemcpyDeviceToHost, st));
    if (out->tri_id) CUDA_TRY(cudaMemcpyAsync(out->tri_id, c->o_tri.p, npx * 4, cudaMemcpyDeviceToHost, st));
    if (out->depth) CUDA_TRY(cudaMemcpyAsync(out->depth, c->o_depth.p, npx * 4, cudaMemcpyDeviceToHost, st));
    if (out->nor) CUDA_TRY(cudaMemcpyAsync(out->nor, c->o_nor.p, npx * 16, cudaMemcpyDeviceToHost, st));
    if (out->face_nor) CUDA_TRY(cudaMemcpyAsync(out->face_nor, c->o_fnor.p, npx * 16, cudaMemcpyDeviceToHost, st));
    if (out->world_pos) CUDA_TRY(cudaMemcpyAsync(out->world_pos, c->o_wpos.p, npx * 16, cudaMemcpyDeviceToHost, st));
    if (out->uvd) CUDA_TRY(cudaMemcpyAsync(out->uvd, c->o_uvd.p, npx * 16, cudaMemcpyDeviceToHost, st));
    if (out->vcol) CUDA_TRY(cudaMemcpyAsync(out->vcol, c->o_vcol.p, npx * 4, cudaMemcpyDeviceToHost, st));
    if (out->mat_id) CUDA_TRY(cudaMemcpyAsync(out->mat_id, c->o_mat.p, npx * 4, cudaMemcpyDeviceToHost, st));
    return PR_OK;
}

// Extra outputs of a differentiable forward frame.
struct DiffHooks {
    float4* dgb;  // [H][W][4] differentiation G-buffer
};

int render_impl(Ctx* c, const pr_frame_desc* f, pr_outputs* out, bool sync, const DiffHooks* dh = nullptr,
                bool submit = false) {
    clear_stale_error();
    int rc = validate_frame(c, f);
    if (rc) return rc;
    // render.MSAA: every pass runs on the n-times framebuffer (the frame is
    // rescaled here); passAntialiasing's resize to the image follows the
    // deferred pass.
    const int M = frame_msaa(f);
    const size_t npx_img = (size_t)f->width * f->height;
    const int W_img = f->width, H_img = f->height;
    pr_frame_desc scaled;
    if (M > 1) {
        if (dh) return fail(PR_ERR_UNSUPPORTED, "MSAA is not available in the adjoint");
        scaled = *f;
        scaled.width *= M;
        scaled.height *= M;
        f = &scaled;
    }
    if (!c->has_scene) return fail(PR_ERR_NO_SCENE, "no scene uploaded");
    if (out && out->size < sizeof(pr_outputs)) return fail(PR_ERR_INVALID_ARG, "outputs->size too small");
    bool out_dev = out && (out->flags & PR_OUT_DEVICE_PTRS);
    if (!sync && !submit && out && !out_dev) return fail(PR_ERR_INVALID_ARG, "pr_render_async needs device output pointers");
    cudaStream_t st = c->stream;
    const int W = f->width, H = f->height;
    const int SW = f->shadow_width > 0 ? f->shadow_width : W;
    const int SH = f->shadow_height > 0 ? f->shadow_height : H;
    const int NL = (int)f->n_lights;
    const bool shadows = (f->flags & PR_FRAME_SHADOWMAP) != 0;

    // ---- host matrices (render/raster.go:232-246, 281-295) ----
    M4 view = loadm(f->view), proj = loadm(f->proj);
    M4 vp = prh::viewport((float)W, (float)H);
    M4 view_inv, proj_inv, vp_inv;
    if (!prh::inv(view, &view_inv)) return fail(PR_ERR_SINGULAR, "view matrix is singular");
    if (!prh::inv(proj, &proj_inv)) return fail(PR_ERR_SINGULAR, "projection matrix is singular");
    if (!prh::inv(vp, &vp_inv)) return fail(PR_ERR_SINGULAR, "viewport matrix is singular");
    M4 pv = prh::mulm(proj, view);
    M4 s2w = prh::mulm(prh::mulm(view_inv, proj_inv), vp_inv);

    if ((rc = set_device(c))) return rc;
    if ((rc = ensure_frame(c, W, H))) return rc;
    uint32_t need_rec0 = c->sb.n_tris + c->sb.n_tris / 8 + 1024;
    if ((rc = ensure_work(c, need_rec0, need_rec0))) return rc;
    if ((rc = c->first_rec.ensure(std::max<uint32_t>(c->sb.n_tris, 1)))) return rc;
    if ((rc = c->clip_list.ensure(std::max<uint32_t>(c->sb.n_tris, 1)))) return rc;

    // Shadow maps: allocated zeroed, reset when their geometry changes
    // (initShadowMaps, render/shadow.go:87), never cleared by a frame.
    if (shadows) {
        if (!c->smap_valid || c->SW != SW || c->SH != SH || c->n_slights != NL) {
            size_t n = (size_t)SW * SH * std::max(NL, 1);
            c->smap_valid = false;  // a failed growth leaves no maps
            if ((rc = c->smap.ensure(n))) return rc;
            // the orderable key of +0.0f is 0x80000000
            KTRY(prk::launch_fill_u32(c->smap.p, 0x80000000u, n, st));
            c->SW = SW;
            c->SH = SH;
            c->n_slights = NL;
            c->smap_valid = true;
        }
        const size_t l0 = c->lastnan.n;
        if ((rc = c->lastnan.ensure((size_t)SW * SH))) return rc;
        // zero, and put back to zero after any pass that wrote it
        if (c->lastnan.n != l0) CUDA_TRY(cudaMemsetAsync(c->lastnan.p, 0, c->lastnan.n * 4, st));
    }

    prk::Counters* dcnt = c->cnt.p;
    size_t npx = (size_t)W * H;
    c->stats = pr_stats{};
    c->stats.size = sizeof(pr_stats);
    c->stats.n_tris_in = c->sb.n_tris;
    uint32_t launches = 0;

    {
        CUDA_TRY(cudaMemsetAsync(dcnt, 0, sizeof(prk::Counters) * prk::kNumCounters, st));
        CUDA_TRY(cudaEventRecord(c->ev[0], st));
        // Proj·View·Model of every object for the main pass (0) and each light (1 + l)
        const uint32_t n_obj = (uint32_t)c->sb.objects.size();
        const int n_pass = shadows ? 1 + NL : 1;
        {
            prk::PassMats pm;
            std::memcpy(pm.pv[0], pv.m, 64);
            for (int l = 0; shadows && l < NL; l++) {
                const M4 lpv = prh::mulm(loadm(f->lights[l].shadow_proj), loadm(f->lights[l].shadow_view));
                std::memcpy(pm.pv[1 + l], lpv.m, 64);
            }
            if ((rc = c->obj_trans.ensure((size_t)n_pass * std::max<uint32_t>(n_obj, 1) * 16))) return rc;
            KTRY(prk::launch_obj_trans(pm, n_pass, c->sb.obj_model.p, n_obj, c->obj_trans.p, st));
            launches += 1;
        }
        // ---- shadow passes (render/raster.go:176-184), on their own stream:
        // only the deferred pass reads the maps ----
        cudaStream_t ss = c->stream_s;
        CUDA_TRY(cudaEventRecord(c->ev_fork, st));
        CUDA_TRY(cudaStreamWaitEvent(ss, c->ev_fork, 0));
        if (shadows) {
            M4 svp = prh::viewport((float)SW, (float)SH);
            for (int l = 0; l < NL; l++) {
                if (!f->lights[l].cast_shadow) continue;
                prk::SetupParams sp{};
                fill_scene_ptrs(c, sp);
                sp.W = SW;
                sp.H = SH;
                sp.msaa = M;
                sp.perspective = 0;
                M4 lpv = prh::mulm(loadm(f->lights[l].shadow_proj), loadm(f->lights[l].shadow_view));
                std::memcpy(sp.pv, lpv.m, 64);
                std::memcpy(sp.viewport, svp.m, 64);
                sp.vp_std = viewport_std(sp.viewport);
                sp.rrec = c->rrec_s.p;
                sp.arec = nullptr;
                sp.cap_rec = c->cap_rec;
                sp.tasks = c->tasks_s.p;
                sp.cap_tasks = c->cap_tasks;
                sp.first_rec = nullptr;
                sp.cnt = dcnt + 1 + l;
                sp.obj_trans = c->obj_trans.p + (size_t)(1 + l) * n_obj * 16;
                if (c->sb.n_tris > c->cap_rec) return fail(PR_ERR_OVERFLOW, "record capacity below triangle count");
                uint32_t* plane = c->smap.p + (size_t)SW * SH * l;
                KTRY(prk::launch_setup_shadow(sp, ss));
                prk::RasterParams rp{};
                rp.rrec = c->rrec_s.p;
                rp.tasks = c->tasks_s.p;
                rp.cnt = dcnt + 1 + l;
                rp.cnt_w = dcnt + 1 + l;
                rp.W = SW;
                rp.H = SH;
                rp.mode = prk::kShadow;
                rp.smap = plane;
                rp.lastnan = c->lastnan.p;
                rp.take = &dcnt[1 + l].take[0];
                KTRY(prk::launch_raster(rp, c->n_sms * 8, ss));
                KTRY(prk::launch_shadow_fixup_reset(SW, SH, c->lastnan.p, plane, dcnt + 1 + l, ss));
                rp.mode = prk::kShadowFixup;
                rp.take = &dcnt[1 + l].take[1];
                KTRY(prk::launch_raster(rp, c->n_sms * 8, ss));
                KTRY(prk::launch_nan_cleanup((size_t)SW * SH, c->lastnan.p, 0u, nullptr, 0u, dcnt + 1 + l, ss));
                launches += 5;
            }
        }
        CUDA_TRY(cudaEventRecord(c->ev[1], ss));
        CUDA_TRY(cudaEventRecord(c->ev_join, ss));
        // ---- forward pass (render/raster.go:226-273) ----
        prk::SetupParams mp{};
        fill_scene_ptrs(c, mp);
        mp.W = W;
        mp.H = H;
        mp.msaa = M;
        mp.perspective = (f->flags & PR_FRAME_PERSPECTIVE) ? 1 : 0;
        std::memcpy(mp.pv, pv.m, 64);
        mp.obj_trans = c->obj_trans.p;
        mp.attr_state = c->attr_state.p;
        mp.defer_attr = 1;  // attribute records for winning records only (attr_kernel after resolve)
        std::memcpy(mp.viewport, vp.m, 64);
        mp.vp_std = viewport_std(mp.viewport);
        std::memcpy(mp.viewport_inv, vp_inv.m, 64);
        std::memcpy(mp.proj_inv, proj_inv.m, 64);
        std::memcpy(mp.view_inv, view_inv.m, 64);
        mp.rrec = c->rrec.p;
        mp.arec = c->arec.p;
        mp.cap_rec = c->cap_rec;
        mp.tasks = c->tasks.p;
        mp.cap_tasks = c->cap_tasks;
        mp.first_rec = c->first_rec.p;
        mp.cnt = dcnt;
        if (dh) {
            if ((rc = c->tri_scr.ensure((size_t)std::max<uint32_t>(c->sb.n_tris, 1) * 12))) return rc;
            mp.tri_scr = c->tri_scr.p;
        }
        CUDA_TRY(cudaMemsetAsync(c->keys.p, 0, npx * 8, st));
        KTRY(prk::launch_setup_main_only(mp, c->clip_list.p, st));
        CUDA_TRY(cudaEventRecord(c->ev[2], st));
        // clipped triangles: their own task list and stream; records and the
        // NaN flag stay the main pass's (visibility is order-independent)
        cudaStream_t sc = c->stream_c;
        prk::Counters* dclip = dcnt + prk::kClipCnt;
        CUDA_TRY(cudaEventRecord(c->ev_setup, st));
        CUDA_TRY(cudaStreamWaitEvent(sc, c->ev_setup, 0));
        prk::SetupParams cp = mp;
        cp.defer_attr = 0;  // clipped sub-triangles carry interpolated attributes: written at once
        cp.cnt = dclip;
        cp.cnt_rec = dcnt;
        cp.tasks = c->tasks_c.p;
        KTRY(prk::launch_clip(cp, c->clip_list.p, sc));
        prk::RasterParams rp{};
        rp.rrec = c->rrec.p;
        rp.tasks = c->tasks.p;
        rp.cnt = dcnt;
        rp.cnt_w = dcnt;
        rp.W = W;
        rp.H = H;
        rp.mode = prk::kMain;
        rp.keys = c->keys.p;
        rp.nanseq = c->nanseq.p;
        rp.beaten = c->beaten.p;
        rp.take = &dcnt[0].take[0];
        prk::RasterParams rc_ = rp;
        rc_.tasks = c->tasks_c.p;
        rc_.cnt = dclip;
        rc_.take = &dclip->take[0];
        rc_.grab = 32;  // a short list (the frame's clipped triangles): spread it over warps
        KTRY(prk::launch_raster(rc_, c->n_sms * 8, sc));
        CUDA_TRY(cudaEventRecord(c->ev_clip, sc));
        KTRY(prk::launch_raster(rp, c->n_sms * 8, st));
        CUDA_TRY(cudaStreamWaitEvent(st, c->ev_clip, 0));
        // the NaN fix-up of both lists in one launch (it returns at once
        // without a NaN fragment)
        rp.mode = prk::kMainFixup;
        rp.take = &dcnt[0].take[1];
        rp.tasks2 = c->tasks_c.p;
        rp.cnt2 = dclip;
        rp.take2 = &dclip->take[1];
        KTRY(prk::launch_raster(rp, c->n_sms * 8, st));
        // AmbientOcclusionShade's march needs only the resolved depths: resolve
        // lists its pixels, and they are marched on stream 3 (free after the
        // clipped raster) while stream 1 writes attributes and shades; the
        // colour scaling joins after shading. A scene without an AO material
        // lists no pixel, and both launches are left out.
        const bool with_ao = out && out->rgba && c->sb.has_ao;
        c->ao_marched = with_ao;
        if (with_ao && (rc = c->ao_T.ensure(npx))) return rc;
        KTRY(prk::launch_resolve_listing(W, H, c->keys.p, c->nanseq.p, c->beaten.p, dcnt, c->win.p, c->depth_ao.p,
                                         c->first_rec.p, c->attr_state.p, c->vis_list.p, c->sb.tri_flags.p,
                                         with_ao ? c->ao_list.p : nullptr, st));
        prk::AoParams ap{};
        if (with_ao) {
            CUDA_TRY(cudaEventRecord(c->ev_resolved, st));
            CUDA_TRY(cudaStreamWaitEvent(sc, c->ev_resolved, 0));
            CUDA_TRY(cudaEventRecord(c->ev_ao0, sc));
            CUDA_TRY(cudaEventRecord(c->sb.ev_released_ao, sc));  // stream 3 reads no scene buffer
            ap.W = W;
            ap.H = H;
            ap.gamma_on = (f->flags & PR_FRAME_GAMMA) ? 1 : 0;
            ap.n_dirs = c->n_ao_dirs;
            ap.ao_half_ulp = prh::ao_classify(c->ao_cos, c->ao_sin, c->n_ao_dirs, W, H, ap.dir_fast, ap.dir_tiny);
            ap.depth = c->depth_ao.p;
            ap.list = c->ao_list.p;
            ap.cnt = dcnt;
            ap.T = c->ao_T.p;
            KTRY(prk::launch_ao_T(ap, sc));
            CUDA_TRY(cudaEventRecord(c->ev_ao, sc));
            launches += 1;
        }
        KTRY(prk::launch_attr(mp, c->vis_list.p, st));
        CUDA_TRY(cudaEventRecord(c->ev[3], st));
        launches += 7;

        // ---- deferred shading + gamma (render/raster.go:275-378) ----
        std::unique_ptr<prk::ShadeParams> sp_owner(new (std::nothrow) prk::ShadeParams());
        if (!sp_owner) return fail(PR_ERR_OOM, "host allocation failed");
        prk::ShadeParams& sp = *sp_owner;
        fill_shade_frame(c, f, s2w, SW, SH, sp);
        sp.win = c->win.p;
        sp.depth_ao = c->depth_ao.p;
        sp.first_rec = c->first_rec.p;
        sp.rrec = c->rrec.p;
        sp.arec = c->arec.p;
        sp.smaps = shadows ? c->smap.p : nullptr;
        sp.ao_list = c->ao_list.p;
        sp.cnt_w = dcnt;
        if (dh) {
            sp.tri_scr = c->tri_scr.p;
            sp.dgb = dh->dgb;
        }
        // outputs: device pointers directly, or ctx staging buffers
        if (out_dev) {
            sp.rgba = (uchar4*)out->rgba;
            sp.tri_id = out->tri_id;
            sp.depth = out->depth;
            sp.gnor = (float4*)out->nor;
            sp.gfnor = (float4*)out->face_nor;
            sp.gwpos = (float4*)out->world_pos;
            sp.guvd = (float4*)out->uvd;
            sp.gvcol = (uchar4*)out->vcol;
            sp.gmat = out->mat_id;
        } else if (out) {
            if (out->rgba) { if ((rc = c->o_rgba.ensure(npx * 4))) return rc; sp.rgba = (uchar4*)c->o_rgba.p; }
            if (out->tri_id) { if ((rc = c->o_tri.ensure(npx))) return rc; sp.tri_id = c->o_tri.p; }
            if (out->depth) { if ((rc = c->o_depth.ensure(npx))) return rc; sp.depth = c->o_depth.p; }
            if (out->nor) { if ((rc = c->o_nor.ensure(npx))) return rc; sp.gnor = c->o_nor.p; }
            if (out->face_nor) { if ((rc = c->o_fnor.ensure(npx))) return rc; sp.gfnor = c->o_fnor.p; }
            if (out->world_pos) { if ((rc = c->o_wpos.ensure(npx))) return rc; sp.gwpos = c->o_wpos.p; }
            if (out->uvd) { if ((rc = c->o_uvd.ensure(npx))) return rc; sp.guvd = c->o_uvd.p; }
            if (out->vcol) { if ((rc = c->o_vcol.ensure(npx * 4))) return rc; sp.gvcol = (uchar4*)c->o_vcol.p; }
            if (out->mat_id) { if ((rc = c->o_mat.ensure(npx))) return rc; sp.gmat = c->o_mat.p; }
        }
        uchar4* rgba_img = sp.rgba;  // the image Render() returns
        if (M > 1 && sp.rgba) {
            if ((rc = c->o_msaa.ensure(npx * 4))) return rc;
            sp.rgba = (uchar4*)c->o_msaa.p;  // the framebuffer's colours
        }
        sp.ao_listed = 1;  // listed by resolve
        CUDA_TRY(cudaStreamWaitEvent(st, c->ev_join, 0));  // the shadow maps are complete
        CUDA_TRY(cudaStreamWaitEvent(st, c->ev_d2h, 0));   // a submitted frame's outputs left the staging
        KTRY(prk::launch_shade(sp, st));
        launches += 1;
        CUDA_TRY(cudaEventRecord(c->sb.ev_released, st));  // the scene buffers are read no more
        CUDA_TRY(cudaEventRecord(c->ev[5], st));
        if (sp.rgba) {
            if (with_ao) {
                // AmbientOcclusionShade's colour scaling and gamma of the listed
                // pixels, once their march (stream 3) and shading are done
                CUDA_TRY(cudaStreamWaitEvent(st, c->ev_ao, 0));
                ap.rgba = sp.rgba;
                ap.dgb = dh ? dh->dgb : nullptr;
                std::memcpy(ap.gamma, sp.gamma, 256);
                KTRY(prk::launch_ao_apply(ap, c->n_sms * 4, st));
                launches += 1;
            }
            if (M > 1) {
                KTRY(prk::launch_msaa_resize(sp.rgba, W, H, rgba_img, W_img, H_img, st));
                launches += 1;
            }
        }
        CUDA_TRY(cudaEventRecord(c->ev[4], st));
        CUDA_TRY(cudaMemcpyAsync(c->h_cnt, dcnt, sizeof(prk::Counters) * prk::kNumCounters, cudaMemcpyDeviceToHost, st));
        if (!sync) {
            c->stats.n_kernel_launches = launches;
            if (submit && out && !out_dev) {
                // host outputs leave on their own stream, beside the next frame
                CUDA_TRY(cudaEventRecord(c->ev_frame, st));
                CUDA_TRY(cudaStreamWaitEvent(c->stream_d, c->ev_frame, 0));
                if ((rc = copy_host_outputs(c, out, npx, npx_img, c->stream_d))) return rc;
                CUDA_TRY(cudaEventRecord(c->ev_d2h, c->stream_d));
            }
            return PR_OK;
        }
        CUDA_TRY(cudaStreamSynchronize(st));
        // capacity check
        uint32_t ov = 0, need_rec = 0, need_tasks = 0;
        for (int k = 0; k < prk::kNumCounters; k++) {
            ov |= c->h_cnt[k].overflow;
            need_rec = std::max(need_rec, c->h_cnt[k].need_rec);
            need_tasks = std::max(need_tasks, c->h_cnt[k].need_tasks);
        }
        if (ov & 4u) return fail(PR_ERR_UNSUPPORTED, "a clipped polygon with NaN coordinates exceeded 9 vertices");
        // A pass whose setup overflowed skipped its raster entirely, and the
        // shadow-map update is a max-fold that is idempotent for a repeated
        // frame, so re-rendering with larger buffers needs no roll-back.
        if (ov) return fail(PR_ERR_OVERFLOW, "internal capacity exceeded (records %u, tasks %u)", need_rec, need_tasks);
    }
    c->stats.n_kernel_launches = launches;
    collect_stats(c);

    // ---- host outputs ----
    if (out && !out_dev && (rc = copy_host_outputs(c, out, npx, npx_img, st))) return rc;
    if (out && out->shadow_maps) {
        size_t ns = (size_t)SW * SH * NL;
        if (!shadows || !c->smap_valid) {
            if (out_dev)
                CUDA_TRY(cudaMemsetAsync(out->shadow_maps, 0, ns * 4, st));
            else
                std::memset(out->shadow_maps, 0, ns * 4);
        } else if (out_dev) {
            KTRY(prk::launch_decode_shadow(c->smap.p, out->shadow_maps, ns, st));
        } else {
            if ((rc = c->o_shadow.ensure(ns))) return rc;
            KTRY(prk::launch_decode_shadow(c->smap.p, c->o_shadow.p, ns, st));
            CUDA_TRY(cudaMemcpyAsync(out->shadow_maps, c->o_shadow.p, ns * 4, cudaMemcpyDeviceToHost, st));
        }
    }
    if (sync) CUDA_TRY(cudaStreamSynchronize(st));
    return PR_OK;
}

}  // namespace

int prk::set_last_error(int status, const char* msg) { return fail(status, "%s", msg); }

extern "C" {

int pr_abi_version(void) { return PR_ABI_VERSION; }

const char* pr_error_string(int status) {
    switch (status) {
        case PR_OK: return "ok";
        case PR_ERR_INVALID_ARG: return "invalid argument";
        case PR_ERR_OOM: return "out of device memory";
        case PR_ERR_CUDA: return "CUDA error";
        case PR_ERR_OVERFLOW: return "internal capacity exceeded";
        case PR_ERR_TIMEOUT: return "device wait timed out";
        case PR_ERR_UNIMPLEMENTED: return "unimplemented";
        case PR_ERR_NO_SCENE: return "no scene uploaded";
        case PR_ERR_UNSUPPORTED: return "unsupported input";
        case PR_ERR_NO_DEVICE: return "no CUDA device";
        case PR_ERR_SINGULAR: return "singular matrix";
        case PR_ERR_FATAL: return "input the reference rejects with a panic";
        default: return "unknown status";
    }
}

const char* pr_last_error(void) { return g_last_error.c_str(); }

int pr_create(int device, void** out_ctx) {
    if (!out_ctx) return fail(PR_ERR_INVALID_ARG, "out_ctx is NULL");
    *out_ctx = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(PR_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    if (device < 0 || device >= ndev) return fail(PR_ERR_INVALID_ARG, "device %d out of range (%d devices)", device, ndev);
    Ctx* c = new (std::nothrow) Ctx();
    if (!c) return fail(PR_ERR_OOM, "host allocation failed");
    c->device = device;
    int rc = set_device(c);
    if (rc) { delete c; return rc; }
    // Stream 3 (clipped raster, then AO's march: the frame's longest chain
    // after resolve) takes the device's highest priority, so that its blocks
    // go first and shading and the shadow passes fill the rest.
    int prio_lo = 0, prio_hi = 0;
    if (cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess) prio_hi = 0;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(PR_ERR_CUDA, "cudaStreamCreate failed");
    }
    for (auto& ev : c->ev) cudaEventCreate(&ev);
    if (cudaStreamCreateWithFlags(&c->stream_s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->stream_c, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_setup, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_clip, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream_u, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream_d, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_frame, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_d2h, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->sb.ev_uploaded, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->sb.ev_released, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->sb_back.ev_uploaded, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->sb_back.ev_released, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->sb.ev_released_ao, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->sb_back.ev_released_ao, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_resolved, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&c->ev_ao0) != cudaSuccess || cudaEventCreate(&c->ev_ao) != cudaSuccess) {
        pr_destroy(c);
        return fail(PR_ERR_CUDA, "stream/event creation failed");
    }
    if ((rc = c->cnt.ensure(prk::kNumCounters))) { pr_destroy(c); return rc; }
    if (host_malloc((void**)&c->h_cnt, sizeof(prk::Counters) * prk::kNumCounters) != cudaSuccess) {
        pr_destroy(c);
        return fail(PR_ERR_OOM, "pinned counter allocation failed");
    }
    c->n_sms = prk::sm_count();
    {
        prh::ao_directions(c->ao_cos, c->ao_sin, &c->n_ao_dirs);
        int e = prk::set_ao_tables(c->ao_cos, c->ao_sin, c->n_ao_dirs, c->stream);
        if (e) {
            pr_destroy(c);
            return fail(PR_ERR_CUDA, "AO table upload: %s", cudaGetErrorString((cudaError_t)e));
        }
    }
    *out_ctx = c;
    return PR_OK;
}

int pr_destroy(void* ctx) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(PR_ERR_INVALID_ARG, "ctx is NULL");
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->stream_u) cudaStreamSynchronize(c->stream_u);
    if (c->stream_d) cudaStreamSynchronize(c->stream_d);
    c->sb.release();
    c->sb_back.release();
    if (c->ev_frame) cudaEventDestroy(c->ev_frame);
    if (c->ev_d2h) cudaEventDestroy(c->ev_d2h);
    if (c->stream_u) cudaStreamDestroy(c->stream_u);
    if (c->stream_d) cudaStreamDestroy(c->stream_d);
    c->rrec.release(); c->arec.release(); c->tasks.release(); c->first_rec.release(); c->attr_state.release(); c->vis_list.release();
    c->clip_list.release();
    c->keys.release(); c->nanseq.release(); c->beaten.release(); c->win.release(); c->depth_ao.release();
    c->ao_list.release();
    c->smap.release(); c->lastnan.release(); c->cnt.release();
    c->o_rgba.release(); c->o_vcol.release(); c->o_msaa.release(); c->o_tri.release(); c->o_depth.release(); c->o_shadow.release();
    c->o_nor.release(); c->o_fnor.release(); c->o_wpos.release(); c->o_uvd.release(); c->o_mat.release();
    c->tri_scr.release(); c->d_kd.release(); c->d_ks.release(); c->d_shin.release(); c->d_vcol.release();
    c->d_acc.release();
    c->rrec_s.release(); c->tasks_s.release(); c->tasks_c.release();
    if (c->ev_setup) cudaEventDestroy(c->ev_setup);
    if (c->ev_clip) cudaEventDestroy(c->ev_clip);
    if (c->ev_resolved) cudaEventDestroy(c->ev_resolved);
    if (c->ev_ao0) cudaEventDestroy(c->ev_ao0);
    if (c->ev_ao) cudaEventDestroy(c->ev_ao);
    c->ao_T.release();
    if (c->stream_c) {
        cudaStreamSynchronize(c->stream_c);
        cudaStreamDestroy(c->stream_c);
    }
    if (c->h_cnt) cudaFreeHost(c->h_cnt);
    for (auto& ev : c->ev)
        if (ev) cudaEventDestroy(ev);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->stream_s) {
        cudaStreamSynchronize(c->stream_s);
        cudaStreamDestroy(c->stream_s);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return PR_OK;
}

int pr_scene_upload(void* ctx, const pr_scene_desc* s) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(PR_ERR_INVALID_ARG, "ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    int rc = validate_scene(s);
    if (rc) return rc;
    if ((rc = set_device(c))) return rc;
    // submitted frames may still read the scene buffers
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream_u));
    CUDA_TRY(cudaStreamSynchronize(c->stream_d));
    clear_stale_error();
    c->has_scene = false;  // until the new scene is complete (a failed upload leaves none)
    if ((rc = scene_fill(c->sb, s, c->stream, false))) return rc;
    CUDA_TRY(cudaStreamSynchronize(c->stream));  // host tables go out of scope
    c->has_scene = true;
    c->smap_valid = false;
    return PR_OK;
}

int pr_frame_submit(void* ctx, const pr_scene_desc* scene, const pr_frame_desc* frame, pr_outputs* out) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(PR_ERR_INVALID_ARG, "ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    int rc = validate_scene(scene);
    if (rc) return rc;
    if (out && out->shadow_maps) return fail(PR_ERR_UNSUPPORTED, "pr_frame_submit does not return shadow maps");
    if ((rc = set_device(c))) return rc;
    SceneBufs& b = c->sb_back;
    clear_stale_error();
    CUDA_TRY(cudaEventSynchronize(b.ev_uploaded));                 // its staging is free again
    CUDA_TRY(cudaStreamWaitEvent(c->stream_u, b.ev_released, 0));  // no frame reads it any more
    CUDA_TRY(cudaStreamWaitEvent(c->stream_u, b.ev_released_ao, 0));
    if ((rc = scene_fill(b, scene, c->stream_u, true))) return rc;
    CUDA_TRY(cudaEventRecord(b.ev_uploaded, c->stream_u));
    std::swap(c->sb, c->sb_back);
    c->has_scene = true;
    c->smap_valid = false;  // as pr_scene_upload
    CUDA_TRY(cudaStreamWaitEvent(c->stream, c->sb.ev_uploaded, 0));
    return render_impl(c, frame, out, false, nullptr, true);
}

int pr_shadow_reset(void* ctx) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(PR_ERR_INVALID_ARG, "ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    c->smap_valid = false;
    return PR_OK;
}

int pr_render(void* ctx, const pr_frame_desc* frame, pr_outputs* out) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(PR_ERR_INVALID_ARG, "ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    int rc = PR_ERR_OVERFLOW;
    // Capacities grow on overflow and the frame is rendered again.
    for (int attempt = 0; attempt < 4 && rc == PR_ERR_OVERFLOW; attempt++) {
        rc = render_impl(c, frame, out, true);
        if (rc == PR_ERR_OVERFLOW) {
            uint32_t need_rec = 0, need_tasks = 0;
            for (int k = 0; k < prk::kNumCounters; k++) {
                need_rec = std::max(need_rec, c->h_cnt[k].need_rec);
                need_tasks = std::max(need_tasks, c->h_cnt[k].need_tasks);
            }
            int r2 = ensure_work(c, need_rec + need_rec / 4, need_tasks + need_tasks / 4);
            if (r2) return r2;
        }
    }
    return rc;
}

int pr_render_async(void* ctx, const pr_frame_desc* frame, pr_outputs* out) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(PR_ERR_INVALID_ARG, "ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    return render_impl(c, frame, out, false);
}

int pr_sync(void* ctx) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(PR_ERR_INVALID_ARG, "ctx is NULL");
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream_d));
    CUDA_TRY(cudaStreamSynchronize(c->stream_u));
    for (int k = 0; k < prk::kNumCounters; k++)
        if (c->h_cnt[k].overflow) return fail(PR_ERR_OVERFLOW, "internal capacity exceeded in an asynchronous frame");
    collect_stats(c);
    return PR_OK;
}

int pr_frame_stats(void* ctx, pr_stats* out) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !out) return fail(PR_ERR_INVALID_ARG, "NULL argument");
    if (out->size < sizeof(pr_stats)) return fail(PR_ERR_INVALID_ARG, "stats->size too small");
    *out = c->stats;
    return PR_OK;
}

int pr_stream(void* ctx, void** out_stream) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !out_stream) return fail(PR_ERR_INVALID_ARG, "NULL argument");
    *out_stream = (void*)c->stream;
    return PR_OK;
}

int pr_host_alloc(size_t bytes, void** out_ptr) {
    if (!out_ptr || bytes == 0) return fail(PR_ERR_INVALID_ARG, "NULL out_ptr or zero bytes");
    *out_ptr = nullptr;
    cudaError_t e = host_malloc(out_ptr, bytes);
    if (e != cudaSuccess) {
        *out_ptr = nullptr;
        return fail(e == cudaErrorMemoryAllocation ? PR_ERR_OOM : PR_ERR_CUDA, "cudaHostAlloc(%zu): %s", bytes,
                    cudaGetErrorString(e));
    }
    return PR_OK;
}

int pr_device_alloc(void* ctx, size_t bytes, void** out_ptr) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !out_ptr || bytes == 0) return fail(PR_ERR_INVALID_ARG, "NULL ctx or out_ptr, or zero bytes");
    *out_ptr = nullptr;
    std::lock_guard<std::mutex> lk(c->mu);
    int rc = set_device(c);
    if (rc) return rc;
    cudaError_t e = dev_malloc(out_ptr, bytes);
    if (e != cudaSuccess) {
        *out_ptr = nullptr;
        return fail(e == cudaErrorMemoryAllocation ? PR_ERR_OOM : PR_ERR_CUDA, "cudaMalloc(%zu): %s", bytes,
                    cudaGetErrorString(e));
    }
    return PR_OK;
}

int pr_device_free(void* ctx, void* ptr) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !ptr) return fail(PR_ERR_INVALID_ARG, "NULL ctx or ptr");
    std::lock_guard<std::mutex> lk(c->mu);
    int rc = set_device(c);
    if (rc) return rc;
    CUDA_TRY(cudaFree(ptr));
    return PR_OK;
}

int pr_device_read(void* ctx, const void* src, size_t bytes, void* dst) {
    Ctx* c = (Ctx*)ctx;
    if (!c || ((!src || !dst) && bytes)) return fail(PR_ERR_INVALID_ARG, "NULL ctx, src or dst");
    if (bytes == 0) return PR_OK;
    std::lock_guard<std::mutex> lk(c->mu);
    int rc = set_device(c);
    if (rc) return rc;
    // after the frames on the context's stream (their outputs land there)
    CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return PR_OK;
}

// ---- test hooks (include/polyred_cuda_testing.h) ----

int pr_testing_fail_alloc(int64_t n) {
    if (n < 0) return fail(PR_ERR_INVALID_ARG, "pr_testing_fail_alloc: negative count");
    g_alloc_fail_in.store(n);
    return PR_OK;
}

int64_t pr_testing_alloc_count(void) { return g_alloc_count.load(); }

int pr_debug_ao_dirs(int W, int H, float* cosv, float* sinv, int8_t* fast, int8_t* tiny) {
    if (!cosv || !sinv || !fast || !tiny) return fail(PR_ERR_INVALID_ARG, "pr_debug_ao_dirs: NULL output");
    if (W <= 0 || H <= 0) return fail(PR_ERR_INVALID_ARG, "pr_debug_ao_dirs: bad frame size");
    int n = 0;
    prh::ao_directions(cosv, sinv, &n);
    prh::ao_classify(cosv, sinv, n, W, H, fast, tiny);
    return n;
}

int pr_host_free(void* ptr) {
    if (!ptr) return fail(PR_ERR_INVALID_ARG, "ptr is NULL");
    cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) return fail(PR_ERR_CUDA, "cudaFreeHost: %s", cudaGetErrorString(e));
    return PR_OK;
}

int pr_view_matrix(const float pos[3], const float target[3], const float up[3], float out[16]) {
    if (!pos || !target || !up || !out) return fail(PR_ERR_INVALID_ARG, "NULL argument");
    M4 m = prh::view_matrix(pos, target, up);
    std::memcpy(out, m.m, 64);
    return PR_OK;
}
int pr_perspective_matrix(float fov, float aspect, float n, float f, float out[16]) {
    if (!out) return fail(PR_ERR_INVALID_ARG, "NULL argument");
    M4 m = prh::perspective(fov, aspect, n, f);
    std::memcpy(out, m.m, 64);
    return PR_OK;
}
int pr_orthographic_matrix(float l, float r, float b, float t, float n, float f, float out[16]) {
    if (!out) return fail(PR_ERR_INVALID_ARG, "NULL argument");
    M4 m = prh::ortho(l, r, b, t, n, f);
    std::memcpy(out, m.m, 64);
    return PR_OK;
}
int pr_mat4_mul(const float a[16], const float b[16], float out[16]) {
    if (!a || !b || !out) return fail(PR_ERR_INVALID_ARG, "NULL argument");
    M4 m = prh::mulm(loadm(a), loadm(b));
    std::memcpy(out, m.m, 64);
    return PR_OK;
}
int pr_mat4_inv(const float m[16], float out[16]) {
    if (!m || !out) return fail(PR_ERR_INVALID_ARG, "NULL argument");
    M4 r;
    if (!prh::inv(loadm(m), &r)) return fail(PR_ERR_SINGULAR, "zero determinant");
    std::memcpy(out, r.m, 64);
    return PR_OK;
}
int pr_shadow_camera(const float light_pos[3], const float scene_center[3], const float cam_view[16],
                     const float cam_proj[16], float out_view[16], float out_proj[16]) {
    if (!light_pos || !scene_center || !cam_view || !cam_proj || !out_view || !out_proj)
        return fail(PR_ERR_INVALID_ARG, "NULL argument");
    M4 v, p;
    if (!prh::shadow_camera(light_pos, scene_center, loadm(cam_view), loadm(cam_proj), &v, &p))
        return fail(PR_ERR_SINGULAR, "camera matrix is singular");
    std::memcpy(out_view, v.m, 64);
    std::memcpy(out_proj, p.m, 64);
    return PR_OK;
}

// ---- differentiable shading ----

namespace {

// Device parameters of a differentiable call: the caller's or the scene's.
int diff_setup(Ctx* c, const pr_frame_desc* f, const pr_diff_params* prm, prk::DiffParamsK& K) {
    int rc;
    const uint32_t nm = (uint32_t)c->sb.materials.size();
    if (c->sb.has_tex) return fail(PR_ERR_UNSUPPORTED, "image textures are not available in the adjoint");
    if (prm && prm->size < sizeof(pr_diff_params)) return fail(PR_ERR_INVALID_ARG, "params->size too small");
    if (prm && prm->n_materials != nm && (prm->kd || prm->ks || prm->shininess))
        return fail(PR_ERR_INVALID_ARG, "params->n_materials (%u) differs from the scene's (%u)", prm->n_materials, nm);
    if (nm > (uint32_t)prk::kDiffMaxMats) return fail(PR_ERR_UNSUPPORTED, "more than %d materials", prk::kDiffMaxMats);
    if (f->n_lights > (uint32_t)prk::kMaxLights || f->n_ambient > (uint32_t)prk::kMaxAmbient)
        return fail(PR_ERR_INVALID_ARG, "too many lights");
    std::vector<float> kd(3 * std::max<uint32_t>(nm, 1)), ks(kd.size()), sh(std::max<uint32_t>(nm, 1));
    for (uint32_t m = 0; m < nm; m++) {
        for (int k = 0; k < 3; k++) {
            kd[3 * m + k] = (prm && prm->kd) ? prm->kd[3 * m + k] : c->sb.materials[m].diffuse[k] / 255.0f;
            ks[3 * m + k] = (prm && prm->ks) ? prm->ks[3 * m + k] : c->sb.materials[m].specular[k] / 255.0f;
        }
        sh[m] = (prm && prm->shininess) ? prm->shininess[m] : c->sb.materials[m].shininess;
    }
    cudaStream_t st = c->stream;
    if ((rc = c->d_kd.ensure(kd.size())) || (rc = c->d_ks.ensure(ks.size())) || (rc = c->d_shin.ensure(sh.size())))
        return rc;
    CUDA_TRY(cudaMemcpyAsync(c->d_kd.p, kd.data(), kd.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(c->d_ks.p, ks.data(), ks.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(c->d_shin.p, sh.data(), sh.size() * 4, cudaMemcpyHostToDevice, st));
    const size_t nv = (size_t)c->sb.n_tris * 3;
    const float4* vcol = prm ? (const float4*)prm->vertex_color : nullptr;
    if (!vcol) {
        if ((rc = c->d_vcol.ensure(std::max<size_t>(nv, 1)))) return rc;
        KTRY(prk::launch_col_to_float(c->sb.col.p, c->d_vcol.p, nv, st));
        vcol = c->d_vcol.p;
    }
    K.W = f->width;
    K.H = f->height;
    K.vcol = vcol;
    K.vnor = (prm && prm->vertex_normal) ? (const float4*)prm->vertex_normal : c->sb.nor.p;
    K.obj_first = c->sb.obj_first.p;
    K.n_objects = (uint32_t)c->sb.objects.size();
    K.obj_normal = c->sb.obj_normal.p;
    K.n_mats = (int)nm;
    K.kd = c->d_kd.p;
    K.ks = c->d_ks.p;
    K.shin = c->d_shin.p;
    K.mats = c->sb.dmats.p;
    K.n_lights = (int)f->n_lights;
    K.n_ambient = (int)f->n_ambient;
    for (uint32_t l = 0; l < f->n_lights; l++) {
        const pr_light& L = f->lights[l];
        prk::LightK& Q = K.lights[l];
        Q.type = L.type;
        Q.cast = L.cast_shadow ? 1 : 0;
        for (int k = 0; k < 3; k++) {
            Q.pos[k] = L.pos[k];
            Q.dir[k] = L.dir[k];
            Q.color[k] = (float)L.color[k];
        }
        Q.intensity = L.intensity;
    }
    for (uint32_t e = 0; e < f->n_ambient; e++) K.ambient[e] = f->ambient[e];
    for (int k = 0; k < 3; k++) K.cam[k] = f->cam_pos[k];
    for (int k = 0; k < 4; k++) K.bg[k] = (float)f->background[k];
    return PR_OK;
}

}  // namespace

int pr_diff_forward(void* ctx, const pr_frame_desc* frame, const pr_diff_params* params, float* radiance, float* gbuf,
                    pr_outputs* out) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(PR_ERR_INVALID_ARG, "ctx is NULL");
    if (!radiance || !gbuf) return fail(PR_ERR_INVALID_ARG, "radiance and gbuf are required");
    if (out && (out->size < sizeof(pr_outputs) || !(out->flags & PR_OUT_DEVICE_PTRS)))
        return fail(PR_ERR_INVALID_ARG, "out must hold device pointers (PR_OUT_DEVICE_PTRS)");
    std::lock_guard<std::mutex> lk(c->mu);
    int rc = validate_frame(c, frame);
    if (rc) return rc;
    if (frame_msaa(frame) > 1) return fail(PR_ERR_UNSUPPORTED, "MSAA is not available in the adjoint");
    if (!c->has_scene) return fail(PR_ERR_NO_SCENE, "no scene uploaded");
    if (c->sb.has_tex) return fail(PR_ERR_UNSUPPORTED, "image textures are not available in the adjoint");
    if ((rc = set_device(c))) return rc;
    // the AO factors need the colour pass: render into ctx storage when the caller wants no image
    pr_outputs o{};
    if (out) o = *out;
    o.size = sizeof(pr_outputs);
    o.flags = PR_OUT_DEVICE_PTRS;
    const size_t npx = (size_t)frame->width * frame->height;
    if (!o.rgba) {
        if ((rc = c->o_rgba.ensure(npx * 4))) return rc;
        o.rgba = c->o_rgba.p;
    }
    DiffHooks dh{(float4*)gbuf};
    rc = PR_ERR_OVERFLOW;
    for (int attempt = 0; attempt < 4 && rc == PR_ERR_OVERFLOW; attempt++) {
        rc = render_impl(c, frame, &o, true, &dh);
        if (rc == PR_ERR_OVERFLOW) {
            uint32_t need_rec = 0, need_tasks = 0;
            for (int k = 0; k < prk::kNumCounters; k++) {
                need_rec = std::max(need_rec, c->h_cnt[k].need_rec);
                need_tasks = std::max(need_tasks, c->h_cnt[k].need_tasks);
            }
            int r2 = ensure_work(c, need_rec + need_rec / 4, need_tasks + need_tasks / 4);
            if (r2) return r2;
        }
    }
    if (rc) return rc;
    prk::DiffParamsK K{};
    if ((rc = diff_setup(c, frame, params, K))) return rc;
    K.dgb = (const float4*)gbuf;
    K.radiance = (float4*)radiance;
    KTRY(prk::launch_diff(K, false, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return PR_OK;
}

int pr_diff_backward(void* ctx, const pr_frame_desc* frame, const pr_diff_params* params, const float* gbuf,
                     const float* grad_radiance, pr_diff_grads* grads) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return fail(PR_ERR_INVALID_ARG, "ctx is NULL");
    if (!gbuf || !grad_radiance || !grads) return fail(PR_ERR_INVALID_ARG, "gbuf, grad_radiance and grads are required");
    if (grads->size < sizeof(pr_diff_grads)) return fail(PR_ERR_INVALID_ARG, "grads->size too small");
    std::lock_guard<std::mutex> lk(c->mu);
    int rc = validate_frame(c, frame);
    if (rc) return rc;
    if (frame_msaa(frame) > 1) return fail(PR_ERR_UNSUPPORTED, "MSAA is not available in the adjoint");
    if (!c->has_scene) return fail(PR_ERR_NO_SCENE, "no scene uploaded");
    if ((rc = set_device(c))) return rc;
    clear_stale_error();
    prk::DiffParamsK K{};
    if ((rc = diff_setup(c, frame, params, K))) return rc;
    cudaStream_t st = c->stream;
    const size_t nv = (size_t)c->sb.n_tris * 3;
    if (grads->vertex_color) CUDA_TRY(cudaMemsetAsync(grads->vertex_color, 0, nv * 16, st));
    if (grads->vertex_normal) CUDA_TRY(cudaMemsetAsync(grads->vertex_normal, 0, nv * 16, st));
    const int nm = K.n_mats, nl = K.n_lights, na = K.n_ambient;
    const size_t n_acc = (size_t)nm * 7 + (size_t)nl * 4 + na;
    if ((rc = c->d_acc.ensure(std::max<size_t>(n_acc, 1)))) return rc;
    CUDA_TRY(cudaMemsetAsync(c->d_acc.p, 0, std::max<size_t>(n_acc, 1) * 8, st));
    K.dgb = (const float4*)gbuf;
    K.grad = (const float4*)grad_radiance;
    K.g_vcol = (float4*)grads->vertex_color;
    K.g_vnor = (float4*)grads->vertex_normal;
    K.g_acc = c->d_acc.p;
    KTRY(prk::launch_diff(K, true, st));
    std::vector<double> acc(std::max<size_t>(n_acc, 1));
    CUDA_TRY(cudaMemcpyAsync(acc.data(), c->d_acc.p, acc.size() * 8, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    for (int m = 0; m < nm; m++) {
        for (int k = 0; k < 3; k++) {
            if (grads->kd) grads->kd[3 * m + k] = acc[7 * m + k];
            if (grads->ks) grads->ks[3 * m + k] = acc[7 * m + 3 + k];
        }
        if (grads->shininess) grads->shininess[m] = acc[7 * m + 6];
    }
    for (int l = 0; l < nl; l++) {
        const double* a = acc.data() + 7 * nm + 4 * l;
        for (int k = 0; k < 3; k++)
            if (grads->light_pos) grads->light_pos[3 * l + k] = frame->lights[l].type == PR_LIGHT_POINT ? a[k] : 0.0;
        if (grads->light_intensity) grads->light_intensity[l] = a[3];
    }
    for (int e = 0; e < na; e++)
        if (grads->ambient) grads->ambient[e] = acc[7 * nm + 4 * nl + e];
    return PR_OK;
}

// Test hook (include/polyred_cuda_testing.h): the shade kernel's float32 Pow
// beside the float64 algorithm on n device-resident argument pairs.
int pr_debug_pow_probe(const float* x, const float* y, float* fast, float* ref, int n) {
    int e = prk::launch_pow_probe(x, y, fast, ref, n, nullptr);
    if (e) return fail(PR_ERR_CUDA, "pow probe launch: %s", cudaGetErrorString((cudaError_t)e));
    CUDA_TRY(cudaDeviceSynchronize());
    return PR_OK;
}

// Test hook (include/polyred_cuda_testing.h): the AO kernel's float32 Atan
// and its certified Pow(T, 10000) colour scaling, each beside the float64
// algorithm, on n device-resident inputs (col, o_fast, o_ref: 4 bytes each).
int pr_debug_ao_probe(const float* x, float* atan_fast, float* atan_ref, const float* T, const uint8_t* col,
                      uint8_t* o_fast, uint8_t* o_ref, int n) {
    int e = prk::launch_ao_probe(x, atan_fast, atan_ref, T, col, o_fast, o_ref, n, nullptr);
    if (e) return fail(PR_ERR_CUDA, "ao probe launch: %s", cudaGetErrorString((cudaError_t)e));
    CUDA_TRY(cudaDeviceSynchronize());
    return PR_OK;
}

// Test hook (include/polyred_cuda_testing.h): runs the device float32
// emulation of float32(fma(f64, f64, f64)) and the direct FP64 expression on
// n device-resident inputs.
int pr_debug_fma_probe(const float* a, const float* b, const float* c, float* out, float* out_ref, int n) {
    int e = prk::launch_fma_probe(a, b, c, out, out_ref, n, nullptr);
    if (e) return fail(PR_ERR_CUDA, "fma probe launch: %s", cudaGetErrorString((cudaError_t)e));
    CUDA_TRY(cudaDeviceSynchronize());
    return PR_OK;
}

}  // extern "C"

// ---- batched rendering ----

namespace {

struct Batch {
    std::mutex mu;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int n_sms = 1;
    std::vector<Ctx*> scenes;
    // tuning
    uint32_t task_shift = prk::kTaskShift;
    int raster_bps = 8;
    // learned capacities, per view of the last shape (records / tasks of the view's main pass and of its shadow passes)
    std::vector<uint32_t> cap_main_rec, cap_main_tasks, cap_shadow_tasks;
    // work buffers
    DevBuf<prk::RasterRec> rrec;
    DevBuf<prk::AttrRec> arec;
    DevBuf<uint2> tasks;
    DevBuf<uint32_t> first_rec, clip_list;
    DevBuf<prk::Counters> cnt;
    DevBuf<unsigned long long> keys;
    DevBuf<uint32_t> nanseq, beaten, win, ao_list, chunk, smaps;
    DevBuf<float> depth_ao;
    // job tables
    DevBuf<prk::SetupParams> d_sj, d_mj;
    DevBuf<prk::RasterParams> d_rj, d_fj;
    DevBuf<prk::ResolveParams> d_res;
    DevBuf<prk::ShadeParams> d_sh;
    DevBuf<prk::AoParams> d_ao;
    DevBuf<uint32_t> d_blk, d_items, d_fitems, d_queue;
    prk::Counters* h_cnt = nullptr;
    size_t h_cnt_n = 0;
    cudaGraphExec_t gexec = nullptr;
    std::string gkey;
    pr_batch_stats stats{};
};

template <class T>
size_t dev_bytes(const DevBuf<T>& b) { return b.n * sizeof(T); }

// Host-side plan and job tables of one batch.
struct BatchPlan {
    uint32_t V = 0, S = 0;                 // views, shadow passes
    std::vector<prk::SetupParams> sj, mj;  // shadow setup [S], main setup [V]
    std::vector<prk::RasterParams> rj, fj; // raster [V + S] (main first), main fix-up [V]
    std::vector<prk::ResolveParams> res;
    std::vector<prk::ShadeParams> sh;
    std::vector<prk::AoParams> ao;
    std::vector<uint32_t> blk;             // blk_s[S+1] blk_m[V+1] blk_r[V+1] blk_sh[V+1]
    uint32_t nb_s = 0, nb_m = 0, nb_r = 0, nb_sh = 0;
    std::vector<int> shadow_view;          // view of each shadow pass
    size_t n_rec = 0, n_rec_main = 0, n_tasks = 0, n_px = 0, n_smap = 0, n_first = 0;
    std::string key;
};

int batch_plan(Batch* b, uint32_t nv, const pr_batch_view* views, BatchPlan& p) {
    p = BatchPlan{};
    p.V = nv;
    if (b->cap_main_rec.size() != nv) {
        b->cap_main_rec.assign(nv, 0);
        b->cap_main_tasks.assign(nv, 0);
        b->cap_shadow_tasks.assign(nv, 0);
    }
    // sizes and offsets
    std::vector<size_t> rec_m(nv), task_m(nv), px(nv), first(nv), sm(nv);
    struct SP { uint32_t v, l; size_t rec, task; };
    std::vector<SP> sps;
    size_t rec = 0, task = 0, npx = 0, nfirst = 0, nsm = 0;
    for (uint32_t v = 0; v < nv; v++) {
        const Ctx* c = b->scenes[views[v].scene];
        const pr_frame_desc* f = views[v].frame;
        const uint32_t n = c->sb.n_tris;
        const uint32_t r0 = n + n / 8 + 1024;
        const uint32_t cr = std::max(r0, b->cap_main_rec[v]), ct = std::max(r0, b->cap_main_tasks[v]);
        rec_m[v] = rec;
        rec += cr;
        task_m[v] = task;
        task += ct;
        b->cap_main_rec[v] = cr;
        b->cap_main_tasks[v] = ct;
        px[v] = npx;
        npx += (size_t)f->width * f->height;
        first[v] = nfirst;
        nfirst += std::max<uint32_t>(n, 1);
    }
    p.n_rec_main = rec;
    for (uint32_t v = 0; v < nv; v++) {
        const Ctx* c = b->scenes[views[v].scene];
        const pr_frame_desc* f = views[v].frame;
        const bool shadows = (f->flags & PR_FRAME_SHADOWMAP) != 0;
        const int SW = f->shadow_width > 0 ? f->shadow_width : f->width;
        const int SH = f->shadow_height > 0 ? f->shadow_height : f->height;
        sm[v] = nsm;
        if (!shadows) continue;
        nsm += (size_t)SW * SH * std::max<uint32_t>(f->n_lights, 1);
        const uint32_t n = c->sb.n_tris;
        const uint32_t ct = std::max(n + n / 8 + 1024, b->cap_shadow_tasks[v]);
        b->cap_shadow_tasks[v] = ct;
        for (uint32_t l = 0; l < f->n_lights; l++) {
            if (!f->lights[l].cast_shadow) continue;
            sps.push_back({v, l, rec, task});
            rec += std::max<uint32_t>(n, 1);
            task += ct;
        }
    }
    p.S = (uint32_t)sps.size();
    p.n_rec = rec;
    p.n_tasks = task;
    p.n_px = npx;
    p.n_first = nfirst;
    p.n_smap = nsm;
    int rc;
    if ((rc = b->rrec.ensure(std::max<size_t>(rec, 1))) || (rc = b->arec.ensure(std::max<size_t>(p.n_rec_main, 1))) ||
        (rc = b->tasks.ensure(std::max<size_t>(task, 1))) || (rc = b->first_rec.ensure(nfirst)) ||
        (rc = b->clip_list.ensure(nfirst)) || (rc = b->cnt.ensure(nv + p.S)) || (rc = b->keys.ensure(npx)) ||
        (rc = b->nanseq.ensure(npx)) || (rc = b->beaten.ensure(npx)) || (rc = b->win.ensure(npx)) ||
        (rc = b->ao_list.ensure(npx)) || (rc = b->depth_ao.ensure(npx)) || (rc = b->chunk.ensure(nv)) ||
        (rc = b->smaps.ensure(std::max<size_t>(nsm, 1))))
        return rc;
    if (b->h_cnt_n < nv + p.S) {
        if (b->h_cnt) cudaFreeHost(b->h_cnt);
        b->h_cnt = nullptr;
        b->h_cnt_n = 0;
        if (host_malloc((void**)&b->h_cnt, sizeof(prk::Counters) * (nv + p.S)) != cudaSuccess) {
            b->h_cnt = nullptr;
            return fail(PR_ERR_OOM, "cudaHostAlloc(%zu bytes) failed", sizeof(prk::Counters) * (nv + p.S));
        }
        b->h_cnt_n = nv + p.S;
    }
    prk::Counters* dcnt = b->cnt.p;
    // shadow passes
    p.sj.resize(p.S);
    p.rj.resize(nv + p.S);
    p.shadow_view.resize(p.S);
    p.blk.push_back(0);
    for (uint32_t s = 0; s < p.S; s++) {
        const SP& q = sps[s];
        Ctx* c = b->scenes[views[q.v].scene];
        const pr_frame_desc* f = views[q.v].frame;
        const int SW = f->shadow_width > 0 ? f->shadow_width : f->width;
        const int SH = f->shadow_height > 0 ? f->shadow_height : f->height;
        prk::SetupParams& sp = p.sj[s];
        fill_scene_ptrs(c, sp);
        sp.W = SW;
        sp.H = SH;
        sp.perspective = 0;
        M4 lpv = prh::mulm(loadm(f->lights[q.l].shadow_proj), loadm(f->lights[q.l].shadow_view));
        std::memcpy(sp.pv, lpv.m, 64);
        M4 svp = prh::viewport((float)SW, (float)SH);
        std::memcpy(sp.viewport, svp.m, 64);
        sp.vp_std = viewport_std(sp.viewport);
        sp.rrec = b->rrec.p + q.rec;
        sp.arec = nullptr;
        sp.cap_rec = std::max<uint32_t>(c->sb.n_tris, 1);
        sp.tasks = b->tasks.p + q.task;
        sp.cap_tasks = b->cap_shadow_tasks[q.v];
        sp.first_rec = nullptr;
        sp.cnt = dcnt + nv + s;
        sp.task_shift = b->task_shift;
        p.shadow_view[s] = (int)q.v;
        prk::RasterParams& rp = p.rj[nv + s];
        rp.rrec = sp.rrec;
        rp.tasks = sp.tasks;
        rp.cnt = sp.cnt;
        rp.cnt_w = sp.cnt;
        rp.W = SW;
        rp.H = SH;
        rp.mode = prk::kShadow;
        rp.smap = b->smaps.p + sm[q.v] + (size_t)SW * SH * q.l;
        rp.lastnan = nullptr;  // NaN depth: the view is re-rendered alone
        rp.task_shift = b->task_shift;
        p.blk.push_back(p.blk.back() + (c->sb.n_tris + 127) / 128);
    }
    p.nb_s = p.blk.back();
    // main passes
    p.mj.resize(nv);
    p.fj.resize(nv);
    p.res.resize(nv);
    p.sh.resize(nv);
    p.ao.resize(nv);
    const size_t om = p.blk.size();
    p.blk.push_back(0);
    for (uint32_t v = 0; v < nv; v++) {
        Ctx* c = b->scenes[views[v].scene];
        const pr_frame_desc* f = views[v].frame;
        FrameMats m;
        if ((rc = frame_mats(f, m))) return rc;
        prk::SetupParams& mp = p.mj[v];
        fill_scene_ptrs(c, mp);
        mp.W = f->width;
        mp.H = f->height;
        mp.perspective = (f->flags & PR_FRAME_PERSPECTIVE) ? 1 : 0;
        std::memcpy(mp.pv, m.pv.m, 64);
        std::memcpy(mp.viewport, m.vp.m, 64);
        mp.vp_std = viewport_std(mp.viewport);
        std::memcpy(mp.viewport_inv, m.vp_inv.m, 64);
        std::memcpy(mp.proj_inv, m.proj_inv.m, 64);
        std::memcpy(mp.view_inv, m.view_inv.m, 64);
        mp.rrec = b->rrec.p + rec_m[v];
        mp.arec = b->arec.p + rec_m[v];
        mp.cap_rec = b->cap_main_rec[v];
        mp.tasks = b->tasks.p + task_m[v];
        mp.cap_tasks = b->cap_main_tasks[v];
        mp.first_rec = b->first_rec.p + first[v];
        mp.clip_list = b->clip_list.p + first[v];
        mp.cnt = dcnt + v;
        mp.task_shift = b->task_shift;
        p.blk.push_back(p.blk.back() + (c->sb.n_tris + 127) / 128);
        const size_t o = px[v];
        prk::RasterParams& rp = p.rj[v];
        rp.rrec = mp.rrec;
        rp.tasks = mp.tasks;
        rp.cnt = mp.cnt;
        rp.cnt_w = mp.cnt;
        rp.W = f->width;
        rp.H = f->height;
        rp.mode = prk::kMain;
        rp.keys = b->keys.p + o;
        rp.nanseq = b->nanseq.p + o;
        rp.beaten = b->beaten.p + o;
        rp.task_shift = b->task_shift;
        p.fj[v] = rp;
        p.fj[v].mode = prk::kMainFixup;
        prk::ResolveParams& R = p.res[v];
        R.W = f->width;
        R.H = f->height;
        R.keys = rp.keys;
        R.nanseq = rp.nanseq;
        R.beaten = rp.beaten;
        R.cnt = mp.cnt;
        R.win = b->win.p + o;
        R.depth_ao = b->depth_ao.p + o;
        prk::ShadeParams& sp = p.sh[v];
        const int SW = f->shadow_width > 0 ? f->shadow_width : f->width;
        const int SH = f->shadow_height > 0 ? f->shadow_height : f->height;
        fill_shade_frame(c, f, m.s2w, SW, SH, sp);
        sp.win = R.win;
        sp.depth_ao = R.depth_ao;
        sp.first_rec = mp.first_rec;
        sp.rrec = mp.rrec;
        sp.arec = mp.arec;
        sp.smaps = (f->flags & PR_FRAME_SHADOWMAP) ? b->smaps.p + sm[v] : nullptr;
        sp.ao_list = b->ao_list.p + o;
        sp.cnt_w = mp.cnt;
        const pr_outputs* out = views[v].out;
        sp.rgba = (uchar4*)out->rgba;
        sp.tri_id = out->tri_id;
        sp.depth = out->depth;
        sp.gnor = (float4*)out->nor;
        sp.gfnor = (float4*)out->face_nor;
        sp.gwpos = (float4*)out->world_pos;
        sp.guvd = (float4*)out->uvd;
        sp.gvcol = (uchar4*)out->vcol;
        sp.gmat = out->mat_id;
        prk::AoParams& ap = p.ao[v];
        ap.W = f->width;
        ap.H = f->height;
        ap.gamma_on = (f->flags & PR_FRAME_GAMMA) ? 1 : 0;
        ap.n_dirs = c->n_ao_dirs;
        ap.ao_half_ulp = prh::ao_classify(c->ao_cos, c->ao_sin, c->n_ao_dirs, f->width, f->height, ap.dir_fast,
                                          ap.dir_tiny);
        ap.depth = R.depth_ao;
        ap.list = sp.ao_list;
        ap.cnt = mp.cnt;
        ap.rgba = sp.rgba;
        std::memcpy(ap.gamma, sp.gamma, 256);
    }
    p.nb_m = p.blk.back();
    const size_t orr = p.blk.size();
    p.blk.push_back(0);
    for (uint32_t v = 0; v < nv; v++)
        p.blk.push_back(p.blk.back() + (uint32_t)(((size_t)views[v].frame->width * views[v].frame->height + 255) / 256));
    p.nb_r = p.blk.back();
    const size_t osh = p.blk.size();
    p.blk.push_back(0);
    for (uint32_t v = 0; v < nv; v++) {
        const uint32_t tx = (uint32_t)(views[v].frame->width + 31) / 32, ty = (uint32_t)(views[v].frame->height + 7) / 8;
        p.blk.push_back(p.blk.back() + tx * ty);
    }
    p.nb_sh = p.blk.back();
    (void)om;
    (void)orr;
    (void)osh;
    // the graph's shape: everything a captured launch depends on
    char kb[128];
    snprintf(kb, sizeof(kb), "%u/%u/%u/%u/%u/%u/%d/%zu/%zu|", nv, p.S, p.nb_s, p.nb_m, p.nb_r, p.nb_sh, b->raster_bps,
             p.n_px, p.n_smap);
    p.key = kb;
    // every pointer the captured launches take as an argument
    const void* args[] = {b->cnt.p, b->keys.p, b->nanseq.p, b->beaten.p, b->chunk.p, b->smaps.p, b->h_cnt,
                          b->d_sj.p, b->d_mj.p, b->d_rj.p, b->d_fj.p, b->d_res.p, b->d_sh.p, b->d_ao.p,
                          b->d_blk.p, b->d_items.p, b->d_fitems.p, b->d_queue.p};
    for (const void* a : args) {
        snprintf(kb, sizeof(kb), "%p,", a);
        p.key += kb;
    }
    for (uint32_t v = 0; v < nv; v++) {
        char vb[64];
        const pr_frame_desc* f = views[v].frame;
        snprintf(vb, sizeof(vb), "%dx%d:%u:%u,", f->width, f->height, (unsigned)(f->flags & PR_FRAME_SHADOWMAP),
                 f->n_lights);
        p.key += vb;
    }
    return PR_OK;
}

// The batch's launch sequence on b->st (captured into a graph by the caller).
int batch_launch(Batch* b, const BatchPlan& p, uint32_t* launches) {
    cudaStream_t st = b->st;
    const uint32_t V = p.V, S = p.S;
    const uint32_t* blk_s = b->d_blk.p;
    const uint32_t* blk_m = blk_s + (S + 1);
    const uint32_t* blk_r = blk_m + (V + 1);
    const uint32_t* blk_sh = blk_r + (V + 1);
    uint32_t n = 0;
    CUDA_TRY(cudaMemsetAsync(b->cnt.p, 0, sizeof(prk::Counters) * (V + S), st));
    CUDA_TRY(cudaMemsetAsync(b->keys.p, 0, p.n_px * 8, st));
    CUDA_TRY(cudaMemsetAsync(b->nanseq.p, 0xff, p.n_px * 4, st));
    CUDA_TRY(cudaMemsetAsync(b->beaten.p, 0, p.n_px * 4, st));
    CUDA_TRY(cudaMemsetAsync(b->chunk.p, 0, V * 4, st));
    if (p.n_smap) {
        KTRY(prk::launch_fill_u32(b->smaps.p, 0x80000000u, p.n_smap, st));  // the key of +0.0f
        n++;
    }
    if (S) {
        KTRY(prk::launch_setup_shadow_batch(b->d_sj.p, blk_s, (int)S, p.nb_s, st));
        n++;
    }
    KTRY(prk::launch_setup_main_batch(b->d_mj.p, blk_m, (int)V, p.nb_m, st));
    KTRY(prk::launch_clip_batch(b->d_mj.p, blk_m, (int)V, p.nb_m, st));
    KTRY(prk::launch_batch_scan(b->d_rj.p, (int)(V + S), b->d_items.p, b->d_queue.p, 0, st));
    KTRY(prk::launch_raster_batch(b->d_rj.p, b->d_items.p, (int)(V + S), b->d_queue.p, b->n_sms * b->raster_bps, st));
    KTRY(prk::launch_batch_scan(b->d_fj.p, (int)V, b->d_fitems.p, b->d_queue.p + 1, 1, st));
    KTRY(prk::launch_raster_batch(b->d_fj.p, b->d_fitems.p, (int)V, b->d_queue.p + 1, b->n_sms * b->raster_bps, st));
    KTRY(prk::launch_resolve_batch(b->d_res.p, blk_r, (int)V, p.nb_r, st));
    KTRY(prk::launch_shade_batch(b->d_sh.p, blk_sh, (int)V, p.nb_sh, st));
    KTRY(prk::launch_ao_batch(b->d_ao.p, (int)V, b->chunk.p, b->n_sms * 4, st));
    n += 10;
    CUDA_TRY(cudaMemcpyAsync(b->h_cnt, b->cnt.p, sizeof(prk::Counters) * (V + S), cudaMemcpyDeviceToHost, st));
    *launches = n;
    return PR_OK;
}

int batch_run(Batch* b, uint32_t nv, const pr_batch_view* views) {
    int rc;
    for (uint32_t v = 0; v < nv; v++) {
        const pr_batch_view& bv = views[v];
        if (bv.scene >= b->scenes.size()) return fail(PR_ERR_INVALID_ARG, "view %u: scene %u not added", v, bv.scene);
        if ((rc = validate_frame(b->scenes[bv.scene], bv.frame))) return rc;
        const pr_outputs* o = bv.out;
        if (!o || o->size < sizeof(pr_outputs) || !(o->flags & PR_OUT_DEVICE_PTRS) || !o->rgba)
            return fail(PR_ERR_INVALID_ARG, "view %u: outputs must be device pointers with rgba set", v);
        if (views[v].frame && views[v].frame->size >= PR_FRAME_DESC_SIZE_V1 && frame_msaa(views[v].frame) > 1)
            return fail(PR_ERR_UNSUPPORTED, "view %u: MSAA is not available in batches", v);
        if (o->shadow_maps) return fail(PR_ERR_UNSUPPORTED, "view %u: shadow_maps output is not batched", v);
    }
    CUDA_TRY(cudaSetDevice(b->device));
    clear_stale_error();
    b->stats.n_retries = 0;
    b->stats.n_fallback_views = 0;
    for (int attempt = 0; attempt < 4; attempt++) {
        BatchPlan p;
        if ((rc = batch_plan(b, nv, views, p))) return rc;
        // device tables (uploaded before every launch; the graph reads them)
        const size_t nblk = p.blk.size();
        if ((rc = b->d_sj.ensure(std::max<size_t>(p.S, 1))) || (rc = b->d_mj.ensure(nv)) ||
            (rc = b->d_rj.ensure(nv + p.S)) || (rc = b->d_fj.ensure(nv)) || (rc = b->d_res.ensure(nv)) ||
            (rc = b->d_sh.ensure(nv)) || (rc = b->d_ao.ensure(nv)) || (rc = b->d_blk.ensure(nblk)) ||
            (rc = b->d_items.ensure(nv + p.S + 1)) || (rc = b->d_fitems.ensure(nv + 1)) || (rc = b->d_queue.ensure(2)))
            return rc;
        if ((rc = batch_plan(b, nv, views, p))) return rc;  // again: pointers of grown tables
        cudaStream_t st = b->st;
        if (p.S) CUDA_TRY(cudaMemcpyAsync(b->d_sj.p, p.sj.data(), p.S * sizeof(prk::SetupParams), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(b->d_mj.p, p.mj.data(), nv * sizeof(prk::SetupParams), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(b->d_rj.p, p.rj.data(), (nv + p.S) * sizeof(prk::RasterParams), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(b->d_fj.p, p.fj.data(), nv * sizeof(prk::RasterParams), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(b->d_res.p, p.res.data(), nv * sizeof(prk::ResolveParams), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(b->d_sh.p, p.sh.data(), nv * sizeof(prk::ShadeParams), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(b->d_ao.p, p.ao.data(), nv * sizeof(prk::AoParams), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(b->d_blk.p, p.blk.data(), nblk * 4, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        uint32_t launches = 0;
        b->stats.graph_reused = 0;
        if (b->gexec && b->gkey == p.key) {
            b->stats.graph_reused = 1;
            launches = b->stats.n_kernel_launches;
        } else {
            if (b->gexec) cudaGraphExecDestroy(b->gexec);
            b->gexec = nullptr;
            b->gkey.clear();
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            int lrc = batch_launch(b, p, &launches);
            cudaError_t ce = cudaStreamEndCapture(st, &g);
            if (lrc) {
                if (g) cudaGraphDestroy(g);
                return lrc;
            }
            if (ce != cudaSuccess) return fail(PR_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
            ce = cudaGraphInstantiate(&b->gexec, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) return fail(PR_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
            b->gkey = p.key;
        }
        CUDA_TRY(cudaEventRecord(b->e0, st));
        CUDA_TRY(cudaGraphLaunch(b->gexec, st));
        CUDA_TRY(cudaEventRecord(b->e1, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        float ms = 0;
        cudaEventElapsedTime(&ms, b->e0, b->e1);
        b->stats.ms_total = ms;
        b->stats.n_kernel_launches = launches;
        b->stats.n_views = nv;
        b->stats.n_passes = nv + p.S;
        b->stats.task_px = 1u << b->task_shift;
        b->stats.raster_blocks = (uint32_t)(b->n_sms * b->raster_bps);
        // capacities: grow the passes that overflowed and run again
        bool grow = false;
        for (uint32_t v = 0; v < nv; v++) {
            const prk::Counters& k = b->h_cnt[v];
            if (k.overflow & 4u) return fail(PR_ERR_UNSUPPORTED, "view %u: a clipped polygon exceeded 9 vertices", v);
            if (k.overflow) {
                grow = true;
                b->cap_main_rec[v] = std::max(b->cap_main_rec[v], k.need_rec + k.need_rec / 4);
                b->cap_main_tasks[v] = std::max(b->cap_main_tasks[v], k.need_tasks + k.need_tasks / 4);
            }
        }
        std::vector<char> redo(nv, 0);
        for (uint32_t s = 0; s < p.S; s++) {
            const prk::Counters& k = b->h_cnt[nv + s];
            const int v = p.shadow_view[s];
            if (k.overflow) {
                grow = true;
                b->cap_shadow_tasks[v] = std::max(b->cap_shadow_tasks[v], k.need_tasks + k.need_tasks / 4);
            } else if (k.nan_flag) {
                redo[v] = 1;
            }
        }
        size_t bytes = dev_bytes(b->rrec) + dev_bytes(b->arec) + dev_bytes(b->tasks) + dev_bytes(b->first_rec) +
                       dev_bytes(b->clip_list) + dev_bytes(b->keys) + dev_bytes(b->nanseq) + dev_bytes(b->beaten) +
                       dev_bytes(b->win) + dev_bytes(b->ao_list) + dev_bytes(b->depth_ao) + dev_bytes(b->smaps);
        b->stats.device_bytes = bytes;
        if (grow) {
            b->stats.n_retries++;
            continue;
        }
        // NaN depth in a shadow pass needs the per-texel fix-up of the single-view path
        for (uint32_t v = 0; v < nv; v++) {
            if (!redo[v]) continue;
            Ctx* c = b->scenes[views[v].scene];
            std::lock_guard<std::mutex> lk(c->mu);
            c->smap_valid = false;
            rc = PR_ERR_OVERFLOW;
            for (int a = 0; a < 4 && rc == PR_ERR_OVERFLOW; a++) {
                rc = render_impl(c, views[v].frame, views[v].out, true);
                if (rc == PR_ERR_OVERFLOW) {
                    uint32_t nr = 0, nt = 0;
                    for (int k = 0; k < prk::kNumCounters; k++) {
                        nr = std::max(nr, c->h_cnt[k].need_rec);
                        nt = std::max(nt, c->h_cnt[k].need_tasks);
                    }
                    int r2 = ensure_work(c, nr + nr / 4, nt + nt / 4);
                    if (r2) return r2;
                }
            }
            if (rc) return rc;
            b->stats.n_fallback_views++;
        }
        return PR_OK;
    }
    return fail(PR_ERR_OVERFLOW, "batch capacities still exceeded after growth");
}

}  // namespace

extern "C" {

int pr_batch_create(int device, void** out_batch) {
    if (!out_batch) return fail(PR_ERR_INVALID_ARG, "out_batch is NULL");
    *out_batch = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return fail(PR_ERR_NO_DEVICE, "no CUDA device %d", device);
    Batch* b = new (std::nothrow) Batch();
    if (!b) return fail(PR_ERR_OOM, "host allocation failed");
    b->device = device;
    CUDA_TRY(cudaSetDevice(device));
    CUDA_TRY(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&b->e0));
    CUDA_TRY(cudaEventCreate(&b->e1));
    b->n_sms = prk::sm_count();
    b->stats.size = sizeof(pr_batch_stats);
    *out_batch = b;
    return PR_OK;
}

int pr_batch_destroy(void* batch) {
    Batch* b = (Batch*)batch;
    if (!b) return fail(PR_ERR_INVALID_ARG, "batch is NULL");
    cudaSetDevice(b->device);
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (Ctx* c : b->scenes) pr_destroy(c);
    b->rrec.release(); b->arec.release(); b->tasks.release(); b->first_rec.release(); b->clip_list.release();
    b->cnt.release(); b->keys.release(); b->nanseq.release(); b->beaten.release(); b->win.release();
    b->ao_list.release(); b->chunk.release(); b->smaps.release(); b->depth_ao.release();
    b->d_sj.release(); b->d_mj.release(); b->d_rj.release(); b->d_fj.release(); b->d_res.release();
    b->d_sh.release(); b->d_ao.release(); b->d_blk.release(); b->d_items.release(); b->d_fitems.release();
    b->d_queue.release();
    if (b->h_cnt) cudaFreeHost(b->h_cnt);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return PR_OK;
}

int pr_batch_add_scene(void* batch, const pr_scene_desc* scene, uint32_t* out_index) {
    Batch* b = (Batch*)batch;
    if (!b || !scene || !out_index) return fail(PR_ERR_INVALID_ARG, "NULL argument");
    if (scene->size >= PR_SCENE_DESC_SIZE_V1 && scene_has_images(scene))
        return fail(PR_ERR_UNSUPPORTED, "image textures are not available in batches");
    std::lock_guard<std::mutex> lk(b->mu);
    void* c = nullptr;
    int rc = pr_create(b->device, &c);
    if (rc) return rc;
    if ((rc = pr_scene_upload(c, scene))) {
        pr_destroy(c);
        return rc;
    }
    CUDA_TRY(cudaStreamSynchronize(((Ctx*)c)->stream));
    b->scenes.push_back((Ctx*)c);
    *out_index = (uint32_t)(b->scenes.size() - 1);
    return PR_OK;
}

int pr_batch_render(void* batch, uint32_t n_views, const pr_batch_view* views) {
    Batch* b = (Batch*)batch;
    if (!b) return fail(PR_ERR_INVALID_ARG, "batch is NULL");
    if (n_views == 0) return PR_OK;
    if (!views) return fail(PR_ERR_INVALID_ARG, "views is NULL");
    std::lock_guard<std::mutex> lk(b->mu);
    return batch_run(b, n_views, views);
}

int pr_batch_tune(void* batch, uint32_t n_views, const pr_batch_view* views, char* report, size_t report_cap) {
    Batch* b = (Batch*)batch;
    if (!b) return fail(PR_ERR_INVALID_ARG, "batch is NULL");
    if (n_views == 0 || !views) return fail(PR_ERR_INVALID_ARG, "no views");
    std::lock_guard<std::mutex> lk(b->mu);
    const uint32_t shifts[] = {5, 6, 8, 10, 12};
    const int bps[] = {2, 4, 8};
    std::string rep = "{\"candidates\": [";
    double best = 1e30;
    uint32_t best_shift = b->task_shift;
    int best_bps = b->raster_bps, rc;
    bool first = true;
    for (uint32_t sh : shifts) {
        for (int g : bps) {
            b->task_shift = sh;
            b->raster_bps = g;
            if ((rc = batch_run(b, n_views, views))) return rc;  // warm-up: capacities, graph
            double t = 0;
            for (int k = 0; k < 3; k++) {
                if ((rc = batch_run(b, n_views, views))) return rc;
                t += b->stats.ms_total;
            }
            t /= 3;
            char buf[96];
            snprintf(buf, sizeof(buf), "%s[%u, %d, %.4f]", first ? "" : ", ", 1u << sh, g, t);
            rep += buf;
            first = false;
            if (t < best) {
                best = t;
                best_shift = sh;
                best_bps = g;
            }
        }
    }
    b->task_shift = best_shift;
    b->raster_bps = best_bps;
    // capacities: what the chosen setting needs, with a margin
    if ((rc = batch_run(b, n_views, views))) return rc;
    size_t rec = 0, tasks = 0;
    for (uint32_t v = 0; v < n_views; v++) {
        const prk::Counters& k = b->h_cnt[v];
        const uint32_t n = b->scenes[views[v].scene]->sb.n_tris;
        b->cap_main_rec[v] = std::max(k.n_rec + k.n_rec / 16 + 64, std::min(b->cap_main_rec[v], n + n / 8 + 1024));
        b->cap_main_tasks[v] = k.n_tasks + k.n_tasks / 16 + 64;
        rec += b->cap_main_rec[v];
        tasks += b->cap_main_tasks[v];
    }
    if ((rc = batch_run(b, n_views, views))) return rc;
    char buf[256];
    snprintf(buf, sizeof(buf),
             "], \"task_px\": %u, \"raster_blocks_per_sm\": %d, \"ms\": %.4f, \"main_record_capacity\": %zu, "
             "\"main_task_capacity\": %zu}",
             1u << b->task_shift, b->raster_bps, b->stats.ms_total, rec, tasks);
    rep += buf;
    if (report && report_cap) {
        std::strncpy(report, rep.c_str(), report_cap - 1);
        report[report_cap - 1] = 0;
    }
    return PR_OK;
}

int pr_batch_get_stats(void* batch, pr_batch_stats* out) {
    Batch* b = (Batch*)batch;
    if (!b || !out) return fail(PR_ERR_INVALID_ARG, "NULL argument");
    if (out->size < sizeof(pr_batch_stats)) return fail(PR_ERR_INVALID_ARG, "out->size too small");
    *out = b->stats;
    return PR_OK;
}

}  // extern "C"
