// pr_api.cpp — the C ABI of libpolyred_cuda.so: contexts, scene upload,
// frame orchestration on one CUDA stream, output copies, host math helpers.
// Compiled with -ffp-contract=off (host float32 math must match the
// reference's Go evaluation bit for bit).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/polyred_cuda.h"
#include "pr_hostmath.h"
#include "pr_kernels.cuh"

using prh::M4;

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

// A device allocation that only grows.
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
        cudaError_t e = cudaMalloc((void**)&p, alloc * sizeof(T));
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

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    // scene
    uint32_t n_tris = 0;
    bool has_scene = false;
    std::vector<pr_object> objects;
    std::vector<pr_material> materials;
    DevBuf<float4> pos, nor;
    DevBuf<float2> uv;
    DevBuf<uchar4> col;
    DevBuf<int32_t> mat;
    DevBuf<uint32_t> obj_first;
    DevBuf<float> obj_model, obj_normal;
    DevBuf<int32_t> obj_matbase;
    DevBuf<pr_material> dmats;
    // raster work space
    DevBuf<prk::RasterRec> rrec;
    DevBuf<prk::AttrRec> arec;
    DevBuf<uint2> tasks;
    DevBuf<uint32_t> first_rec, clip_list;
    uint32_t cap_rec = 0, cap_tasks = 0;
    // framebuffer
    int W = 0, H = 0;
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
    DevBuf<prk::Counters> cnt;  // [kMaxLights + 1]
    prk::Counters* h_cnt = nullptr;  // pinned mirror
    // staging for host outputs
    DevBuf<uint8_t> o_rgba, o_vcol;
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
    int n_sms = 1;
};

int set_device(Ctx* c) { CUDA_TRY(cudaSetDevice(c->device)); return PR_OK; }

M4 loadm(const float* p) {
    M4 m;
    std::memcpy(m.m, p, 64);
    return m;
}

int validate_scene(const pr_scene_desc* s) {
    if (!s) return fail(PR_ERR_INVALID_ARG, "scene is NULL");
    if (s->size < sizeof(pr_scene_desc)) return fail(PR_ERR_INVALID_ARG, "scene->size %u < %zu", s->size, sizeof(pr_scene_desc));
    if (s->n_tris > 0 && (!s->pos || !s->nor || !s->uv || !s->col || !s->mat_id))
        return fail(PR_ERR_INVALID_ARG, "scene arrays must be non-NULL when n_tris > 0");
    if (s->n_tris >= (1u << 29)) return fail(PR_ERR_INVALID_ARG, "n_tris %u exceeds 2^29 (draw-order key limit)", s->n_tris);
    if (s->n_objects == 0 && s->n_tris > 0) return fail(PR_ERR_INVALID_ARG, "triangles without objects");
    if (s->n_objects > 0 && !s->objects) return fail(PR_ERR_INVALID_ARG, "objects is NULL");
    if (s->n_materials > 0 && !s->materials) return fail(PR_ERR_INVALID_ARG, "materials is NULL");
    uint32_t expect = 0;
    for (uint32_t o = 0; o < s->n_objects; o++) {
        if (s->objects[o].first_tri != expect)
            return fail(PR_ERR_INVALID_ARG, "object %u: first_tri %u, expected %u (objects must tile the soup in order)", o,
                        s->objects[o].first_tri, expect);
        expect += s->objects[o].n_tris;
    }
    if (expect != s->n_tris) return fail(PR_ERR_INVALID_ARG, "objects cover %u triangles, scene has %u", expect, s->n_tris);
    for (uint32_t m = 0; m < s->n_materials; m++) {
        if (s->materials[m].texture_size != 1)
            return fail(PR_ERR_UNSUPPORTED, "material %u: only uniform (1x1) textures are supported", m);
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

int ensure_frame(Ctx* c, int W, int H) {
    size_t n = (size_t)W * H;
    int rc;
    if ((rc = c->keys.ensure(n))) return rc;
    if ((rc = c->nanseq.ensure(n))) return rc;
    if ((rc = c->beaten.ensure(n))) return rc;
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
        if ((rc = c->rrec.ensure(cap))) return rc;
        if ((rc = c->arec.ensure(cap))) return rc;
        c->cap_rec = cap;
    }
    if (need_tasks > c->cap_tasks) {
        uint32_t cap = std::max(need_tasks, c->cap_tasks * 2);
        if ((rc = c->tasks.ensure(cap))) return rc;
        c->cap_tasks = cap;
    }
    return PR_OK;
}

void fill_scene_ptrs(Ctx* c, prk::SetupParams& p) {
    p.pos = c->pos.p;
    p.nor = c->nor.p;
    p.uv = c->uv.p;
    p.col = c->col.p;
    p.mat = c->mat.p;
    p.obj_first = c->obj_first.p;
    p.obj_model = c->obj_model.p;
    p.obj_normal = c->obj_normal.p;
    p.obj_matbase = c->obj_matbase.p;
    p.n_tris = c->n_tris;
    p.n_objects = (uint32_t)c->objects.size();
}

int validate_frame(const Ctx* c, const pr_frame_desc* f) {
    if (!f) return fail(PR_ERR_INVALID_ARG, "frame is NULL");
    if (f->size < sizeof(pr_frame_desc)) return fail(PR_ERR_INVALID_ARG, "frame->size %u < %zu", f->size, sizeof(pr_frame_desc));
    if (f->width <= 0 || f->height <= 0 || f->width > 16384 || f->height > 16384)
        return fail(PR_ERR_INVALID_ARG, "frame size %dx%d outside 1..16384", f->width, f->height);
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
    for (int k = 0; k <= prk::kMaxLights; k++) n_tasks += c->h_cnt[k].n_tasks;
    c->stats.n_raster_tasks = n_tasks;
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]); c->stats.ms_shadow = ms;
    cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]); c->stats.ms_setup = ms;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]); c->stats.ms_raster = ms;
    cudaEventElapsedTime(&ms, c->ev[3], c->ev[4]); c->stats.ms_shade = ms;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[4]); c->stats.ms_total = ms;
    cudaEventElapsedTime(&ms, c->ev[5], c->ev[4]); c->stats.ms_ao = ms;
    c->stats.n_ao_pixels = c->h_cnt[0].n_ao;
}

// Extra outputs of a differentiable forward frame.
struct DiffHooks {
    float4* dgb;  // [H][W][4] differentiation G-buffer
};

int render_impl(Ctx* c, const pr_frame_desc* f, pr_outputs* out, bool sync, const DiffHooks* dh = nullptr) {
    int rc = validate_frame(c, f);
    if (rc) return rc;
    if (!c->has_scene) return fail(PR_ERR_NO_SCENE, "no scene uploaded");
    if (out && out->size < sizeof(pr_outputs)) return fail(PR_ERR_INVALID_ARG, "outputs->size too small");
    bool out_dev = out && (out->flags & PR_OUT_DEVICE_PTRS);
    if (!sync && out && !out_dev) return fail(PR_ERR_INVALID_ARG, "pr_render_async needs device output pointers");
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
    uint32_t need_rec0 = c->n_tris + c->n_tris / 8 + 1024;
    if ((rc = ensure_work(c, need_rec0, need_rec0))) return rc;
    if ((rc = c->first_rec.ensure(std::max<uint32_t>(c->n_tris, 1)))) return rc;
    if ((rc = c->clip_list.ensure(std::max<uint32_t>(c->n_tris, 1)))) return rc;

    // Shadow maps: allocated zeroed, reset when their geometry changes
    // (initShadowMaps, render/shadow.go:87), never cleared by a frame.
    if (shadows) {
        if (!c->smap_valid || c->SW != SW || c->SH != SH || c->n_slights != NL) {
            size_t n = (size_t)SW * SH * std::max(NL, 1);
            if ((rc = c->smap.ensure(n))) return rc;
            // the orderable key of +0.0f is 0x80000000
            KTRY(prk::launch_fill_u32(c->smap.p, 0x80000000u, n, st));
            c->SW = SW;
            c->SH = SH;
            c->n_slights = NL;
            c->smap_valid = true;
        }
        if ((rc = c->lastnan.ensure((size_t)SW * SH))) return rc;
    }

    prk::Counters* dcnt = c->cnt.p;
    size_t npx = (size_t)W * H;
    c->stats = pr_stats{};
    c->stats.size = sizeof(pr_stats);
    c->stats.n_tris_in = c->n_tris;
    uint32_t launches = 0;

    {
        CUDA_TRY(cudaMemsetAsync(dcnt, 0, sizeof(prk::Counters) * (prk::kMaxLights + 1), st));
        CUDA_TRY(cudaEventRecord(c->ev[0], st));
        // ---- shadow passes (render/raster.go:176-184) ----
        if (shadows) {
            M4 svp = prh::viewport((float)SW, (float)SH);
            for (int l = 0; l < NL; l++) {
                if (!f->lights[l].cast_shadow) continue;
                prk::SetupParams sp{};
                fill_scene_ptrs(c, sp);
                sp.W = SW;
                sp.H = SH;
                sp.perspective = 0;
                M4 lpv = prh::mulm(loadm(f->lights[l].shadow_proj), loadm(f->lights[l].shadow_view));
                std::memcpy(sp.pv, lpv.m, 64);
                std::memcpy(sp.viewport, svp.m, 64);
                sp.rrec = c->rrec.p;
                sp.arec = nullptr;
                sp.cap_rec = c->cap_rec;
                sp.tasks = c->tasks.p;
                sp.cap_tasks = c->cap_tasks;
                sp.first_rec = c->first_rec.p;
                sp.cnt = dcnt + 1 + l;
                if (c->n_tris > c->cap_rec) return fail(PR_ERR_OVERFLOW, "record capacity below triangle count");
                uint32_t* plane = c->smap.p + (size_t)SW * SH * l;
                CUDA_TRY(cudaMemsetAsync(c->lastnan.p, 0, (size_t)SW * SH * 4, st));
                KTRY(prk::launch_setup_shadow(sp, st));
                prk::RasterParams rp{};
                rp.rrec = c->rrec.p;
                rp.tasks = c->tasks.p;
                rp.cnt = dcnt + 1 + l;
                rp.cnt_w = dcnt + 1 + l;
                rp.W = SW;
                rp.H = SH;
                rp.mode = prk::kShadow;
                rp.smap = plane;
                rp.lastnan = c->lastnan.p;
                KTRY(prk::launch_raster(rp, c->n_sms * 8, st));
                KTRY(prk::launch_shadow_fixup_reset(SW, SH, c->lastnan.p, plane, dcnt + 1 + l, st));
                rp.mode = prk::kShadowFixup;
                KTRY(prk::launch_raster(rp, c->n_sms * 8, st));
                launches += 4;
            }
        }
        CUDA_TRY(cudaEventRecord(c->ev[1], st));
        // ---- forward pass (render/raster.go:226-273) ----
        prk::SetupParams mp{};
        fill_scene_ptrs(c, mp);
        mp.W = W;
        mp.H = H;
        mp.perspective = (f->flags & PR_FRAME_PERSPECTIVE) ? 1 : 0;
        std::memcpy(mp.pv, pv.m, 64);
        std::memcpy(mp.viewport, vp.m, 64);
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
            if ((rc = c->tri_scr.ensure((size_t)std::max<uint32_t>(c->n_tris, 1) * 12))) return rc;
            mp.tri_scr = c->tri_scr.p;
        }
        CUDA_TRY(cudaMemsetAsync(c->keys.p, 0, npx * 8, st));
        CUDA_TRY(cudaMemsetAsync(c->nanseq.p, 0xff, npx * 4, st));
        CUDA_TRY(cudaMemsetAsync(c->beaten.p, 0, npx * 4, st));
        KTRY(prk::launch_setup_main(mp, c->clip_list.p, st));
        CUDA_TRY(cudaEventRecord(c->ev[2], st));
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
        KTRY(prk::launch_raster(rp, c->n_sms * 8, st));
        rp.mode = prk::kMainFixup;
        KTRY(prk::launch_raster(rp, c->n_sms * 8, st));
        KTRY(prk::launch_resolve(W, H, c->keys.p, c->nanseq.p, c->beaten.p, dcnt, c->win.p, c->depth_ao.p, st));
        CUDA_TRY(cudaEventRecord(c->ev[3], st));
        launches += 5;

        // ---- deferred shading + gamma (render/raster.go:275-378) ----
        std::unique_ptr<prk::ShadeParams> sp_owner(new (std::nothrow) prk::ShadeParams());
        if (!sp_owner) return fail(PR_ERR_OOM, "host allocation failed");
        prk::ShadeParams& sp = *sp_owner;
        sp.W = W;
        sp.H = H;
        sp.flags = f->flags;
        sp.win = c->win.p;
        sp.depth_ao = c->depth_ao.p;
        sp.first_rec = c->first_rec.p;
        sp.rrec = c->rrec.p;
        sp.arec = c->arec.p;
        sp.mats = c->dmats.p;
        sp.n_mats = (uint32_t)c->materials.size();
        sp.n_lights = NL;
        sp.n_ambient = (int)f->n_ambient;
        for (int l = 0; l < NL; l++) {
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
        sp.SW = SW;
        sp.SH = SH;
        sp.smaps = shadows ? c->smap.p : nullptr;
        prh::gamma_table(sp.gamma);
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
        KTRY(prk::launch_shade(sp, st));
        launches += 1;
        CUDA_TRY(cudaEventRecord(c->ev[5], st));
        if (sp.rgba) {
            // AmbientOcclusionShade + gamma for the pixels the shade kernel listed
            prk::AoParams ap{};
            ap.W = W;
            ap.H = H;
            ap.gamma_on = (f->flags & PR_FRAME_GAMMA) ? 1 : 0;
            ap.n_dirs = c->n_ao_dirs;
            ap.ao_half_ulp = prh::ao_classify(c->ao_cos, c->ao_sin, c->n_ao_dirs, W, H, ap.dir_fast, ap.dir_tiny);
            ap.depth = c->depth_ao.p;
            ap.list = c->ao_list.p;
            ap.cnt = dcnt;
            ap.rgba = sp.rgba;
            ap.dgb = dh ? dh->dgb : nullptr;
            std::memcpy(ap.gamma, sp.gamma, 256);
            KTRY(prk::launch_ao(ap, st));
            launches += 1;
        }
        CUDA_TRY(cudaEventRecord(c->ev[4], st));
        CUDA_TRY(cudaMemcpyAsync(c->h_cnt, dcnt, sizeof(prk::Counters) * (prk::kMaxLights + 1), cudaMemcpyDeviceToHost, st));
        if (!sync) {
            c->stats.n_kernel_launches = launches;
            return PR_OK;
        }
        CUDA_TRY(cudaStreamSynchronize(st));
        // capacity check
        uint32_t ov = 0, need_rec = 0, need_tasks = 0;
        for (int k = 0; k <= prk::kMaxLights; k++) {
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
    if (out && !out_dev) {
        if (out->rgba) CUDA_TRY(cudaMemcpyAsync(out->rgba, c->o_rgba.p, npx * 4, cudaMemcpyDeviceToHost, st));
        if (out->tri_id) CUDA_TRY(cudaMemcpyAsync(out->tri_id, c->o_tri.p, npx * 4, cudaMemcpyDeviceToHost, st));
        if (out->depth) CUDA_TRY(cudaMemcpyAsync(out->depth, c->o_depth.p, npx * 4, cudaMemcpyDeviceToHost, st));
        if (out->nor) CUDA_TRY(cudaMemcpyAsync(out->nor, c->o_nor.p, npx * 16, cudaMemcpyDeviceToHost, st));
        if (out->face_nor) CUDA_TRY(cudaMemcpyAsync(out->face_nor, c->o_fnor.p, npx * 16, cudaMemcpyDeviceToHost, st));
        if (out->world_pos) CUDA_TRY(cudaMemcpyAsync(out->world_pos, c->o_wpos.p, npx * 16, cudaMemcpyDeviceToHost, st));
        if (out->uvd) CUDA_TRY(cudaMemcpyAsync(out->uvd, c->o_uvd.p, npx * 16, cudaMemcpyDeviceToHost, st));
        if (out->vcol) CUDA_TRY(cudaMemcpyAsync(out->vcol, c->o_vcol.p, npx * 4, cudaMemcpyDeviceToHost, st));
        if (out->mat_id) CUDA_TRY(cudaMemcpyAsync(out->mat_id, c->o_mat.p, npx * 4, cudaMemcpyDeviceToHost, st));
    }
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
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(PR_ERR_CUDA, "cudaStreamCreate failed");
    }
    for (auto& ev : c->ev) cudaEventCreate(&ev);
    if ((rc = c->cnt.ensure(prk::kMaxLights + 1))) { pr_destroy(c); return rc; }
    if (cudaMallocHost((void**)&c->h_cnt, sizeof(prk::Counters) * (prk::kMaxLights + 1)) != cudaSuccess) {
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
    c->pos.release(); c->nor.release(); c->uv.release(); c->col.release(); c->mat.release();
    c->obj_first.release(); c->obj_model.release(); c->obj_normal.release(); c->obj_matbase.release();
    c->dmats.release(); c->rrec.release(); c->arec.release(); c->tasks.release(); c->first_rec.release();
    c->clip_list.release();
    c->keys.release(); c->nanseq.release(); c->beaten.release(); c->win.release(); c->depth_ao.release();
    c->ao_list.release();
    c->smap.release(); c->lastnan.release(); c->cnt.release();
    c->o_rgba.release(); c->o_vcol.release(); c->o_tri.release(); c->o_depth.release(); c->o_shadow.release();
    c->o_nor.release(); c->o_fnor.release(); c->o_wpos.release(); c->o_uvd.release(); c->o_mat.release();
    c->tri_scr.release(); c->d_kd.release(); c->d_ks.release(); c->d_shin.release(); c->d_vcol.release();
    c->d_acc.release();
    if (c->h_cnt) cudaFreeHost(c->h_cnt);
    for (auto& ev : c->ev)
        if (ev) cudaEventDestroy(ev);
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
    bool dev = (s->flags & PR_SCENE_DEVICE_PTRS) != 0;
    cudaStream_t st = c->stream;
    uint32_t n = s->n_tris;
    if ((rc = upload(c->pos, s->pos, (size_t)n * 3, dev, st))) return rc;
    if ((rc = upload(c->nor, s->nor, (size_t)n * 3, dev, st))) return rc;
    if ((rc = upload(c->uv, s->uv, (size_t)n * 3, dev, st))) return rc;
    if ((rc = upload(c->col, s->col, (size_t)n * 3, dev, st))) return rc;
    if ((rc = upload(c->mat, s->mat_id, (size_t)n, dev, st))) return rc;
    c->objects.assign(s->objects, s->objects + s->n_objects);
    c->materials.assign(s->materials, s->materials + s->n_materials);
    // Per-object Model and Normal = Model.Inv().T() (render/raster.go:242-243)
    uint32_t no = s->n_objects;
    std::vector<uint32_t> first(no + 1);
    std::vector<float> model((size_t)no * 16), normal((size_t)no * 16);
    std::vector<int32_t> mb(no);
    for (uint32_t o = 0; o < no; o++) {
        first[o] = s->objects[o].first_tri;
        M4 m = loadm(s->objects[o].model), mi;
        if (!prh::inv(m, &mi)) return fail(PR_ERR_SINGULAR, "object %u: model matrix is singular", o);
        M4 nm = prh::transpose(mi);
        std::memcpy(&model[(size_t)o * 16], m.m, 64);
        std::memcpy(&normal[(size_t)o * 16], nm.m, 64);
        mb[o] = s->objects[o].mat_base;
    }
    first[no] = n;
    if ((rc = upload(c->obj_first, first.data(), first.size(), false, st))) return rc;
    if ((rc = upload(c->obj_model, model.data(), model.size(), false, st))) return rc;
    if ((rc = upload(c->obj_normal, normal.data(), normal.size(), false, st))) return rc;
    if ((rc = upload(c->obj_matbase, mb.data(), mb.size(), false, st))) return rc;
    if ((rc = upload(c->dmats, c->materials.data(), c->materials.size(), false, st))) return rc;
    CUDA_TRY(cudaStreamSynchronize(st));  // host vectors above go out of scope
    c->n_tris = n;
    c->has_scene = true;
    c->smap_valid = false;
    return PR_OK;
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
            for (int k = 0; k <= prk::kMaxLights; k++) {
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
    for (int k = 0; k <= prk::kMaxLights; k++)
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
    const uint32_t nm = (uint32_t)c->materials.size();
    if (prm && prm->size < sizeof(pr_diff_params)) return fail(PR_ERR_INVALID_ARG, "params->size too small");
    if (prm && prm->n_materials != nm && (prm->kd || prm->ks || prm->shininess))
        return fail(PR_ERR_INVALID_ARG, "params->n_materials (%u) differs from the scene's (%u)", prm->n_materials, nm);
    if (nm > (uint32_t)prk::kDiffMaxMats) return fail(PR_ERR_UNSUPPORTED, "more than %d materials", prk::kDiffMaxMats);
    if (f->n_lights > (uint32_t)prk::kMaxLights || f->n_ambient > (uint32_t)prk::kMaxAmbient)
        return fail(PR_ERR_INVALID_ARG, "too many lights");
    std::vector<float> kd(3 * std::max<uint32_t>(nm, 1)), ks(kd.size()), sh(std::max<uint32_t>(nm, 1));
    for (uint32_t m = 0; m < nm; m++) {
        for (int k = 0; k < 3; k++) {
            kd[3 * m + k] = (prm && prm->kd) ? prm->kd[3 * m + k] : c->materials[m].diffuse[k] / 255.0f;
            ks[3 * m + k] = (prm && prm->ks) ? prm->ks[3 * m + k] : c->materials[m].specular[k] / 255.0f;
        }
        sh[m] = (prm && prm->shininess) ? prm->shininess[m] : c->materials[m].shininess;
    }
    cudaStream_t st = c->stream;
    if ((rc = c->d_kd.ensure(kd.size())) || (rc = c->d_ks.ensure(ks.size())) || (rc = c->d_shin.ensure(sh.size())))
        return rc;
    CUDA_TRY(cudaMemcpyAsync(c->d_kd.p, kd.data(), kd.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(c->d_ks.p, ks.data(), ks.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(c->d_shin.p, sh.data(), sh.size() * 4, cudaMemcpyHostToDevice, st));
    const size_t nv = (size_t)c->n_tris * 3;
    const float4* vcol = prm ? (const float4*)prm->vertex_color : nullptr;
    if (!vcol) {
        if ((rc = c->d_vcol.ensure(std::max<size_t>(nv, 1)))) return rc;
        KTRY(prk::launch_col_to_float(c->col.p, c->d_vcol.p, nv, st));
        vcol = c->d_vcol.p;
    }
    K.W = f->width;
    K.H = f->height;
    K.vcol = vcol;
    K.vnor = (prm && prm->vertex_normal) ? (const float4*)prm->vertex_normal : c->nor.p;
    K.obj_first = c->obj_first.p;
    K.n_objects = (uint32_t)c->objects.size();
    K.obj_normal = c->obj_normal.p;
    K.n_mats = (int)nm;
    K.kd = c->d_kd.p;
    K.ks = c->d_ks.p;
    K.shin = c->d_shin.p;
    K.mats = c->dmats.p;
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
    if (!c->has_scene) return fail(PR_ERR_NO_SCENE, "no scene uploaded");
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
            for (int k = 0; k <= prk::kMaxLights; k++) {
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
    if (!c->has_scene) return fail(PR_ERR_NO_SCENE, "no scene uploaded");
    if ((rc = set_device(c))) return rc;
    prk::DiffParamsK K{};
    if ((rc = diff_setup(c, frame, params, K))) return rc;
    cudaStream_t st = c->stream;
    const size_t nv = (size_t)c->n_tris * 3;
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

// Test hook (not part of the public header): the AO kernel's float32 Atan
// and its certified Pow(T, 10000) colour scaling, each beside the float64
// algorithm, on n device-resident inputs (col, o_fast, o_ref: 4 bytes each).
int pr_debug_ao_probe(const float* x, float* atan_fast, float* atan_ref, const float* T, const uint8_t* col,
                      uint8_t* o_fast, uint8_t* o_ref, int n) {
    int e = prk::launch_ao_probe(x, atan_fast, atan_ref, T, col, o_fast, o_ref, n, nullptr);
    if (e) return fail(PR_ERR_CUDA, "ao probe launch: %s", cudaGetErrorString((cudaError_t)e));
    CUDA_TRY(cudaDeviceSynchronize());
    return PR_OK;
}

// Test hook (not part of the public header): runs the device float32
// emulation of float32(fma(f64, f64, f64)) and the direct FP64 expression on
// n device-resident inputs.
int pr_debug_fma_probe(const float* a, const float* b, const float* c, float* out, float* out_ref, int n) {
    int e = prk::launch_fma_probe(a, b, c, out, out_ref, n, nullptr);
    if (e) return fail(PR_ERR_CUDA, "fma probe launch: %s", cudaGetErrorString((cudaError_t)e));
    CUDA_TRY(cudaDeviceSynchronize());
    return PR_OK;
}

}  // extern "C"
