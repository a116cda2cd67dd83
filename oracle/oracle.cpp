// oracle.cpp — CPU restatement of polyred's render path, single-worker order.
//
// TEST INFRASTRUCTURE. This is the reference the CUDA path is compared with; it
// is used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg. The product (libpolyred_cuda.so) never links or calls it.
//
// It restates, for render.NewRenderer(..., render.CPU(), render.Workers(1)):
//   Renderer.Render            render/raster.go:155-199
//   passShadows / drawDepth    render/shadow.go:92-228
//   cpuForwardPass / draw      render/raster.go:226-273, 380-444
//   clipTriangle               render/clipping.go:18-157
//   drawClipped                render/raster.go:462-572
//   FragmentBuffer DepthTest/Set  buffer/buffer.go:221-280
//   passDeferred / shade       render/raster.go:275-359
//   FragmentShader             shader/blinn_cpu.go:24-106
//   shadingVisibility          render/shadow.go:230-283
//   AmbientOcclusionShade      material/ao.go:20-73
//   GammaCorrection / sRGB LUT shader/gamma.go:13-18, color/srgb.go:15-75
// Build: g++ -O2 -ffp-contract=off -fno-fast-math (see oracle/build.sh).
//
// Threads: with threads > 1 the forward and shadow rasters split the screen
// into row bands and each band thread walks every triangle in submission
// order, writing only its own rows; shading splits pixels. The result is
// identical to threads == 1 (each pixel still sees the single-worker
// sequence), which is what makes a multi-core CPU baseline comparable.
#include "oracle.h"

#include <algorithm>
#include <array>
#include <thread>
#include <vector>

#include "vecmath.h"

using namespace orc;
using gomath::go_f2i;
using gomath::go_f2u8;
using gomath::pclamp;
using gomath::pround;

namespace {

struct Vtx {  // primitive.Vertex
    V4 pos, nor;
    uint8_t col[4];
    V2 uv;
};

struct Frag {  // buffer.Fragment
    bool ok;
    int64_t x, y;
    float depth, u, v, du, dv;
    V4 nor;
    uint8_t col[4];
    int64_t matid;
    V4 fnor, wpos;
    uint32_t tri;  // input triangle index of the stored fragment (tri-ID output)
};

struct FB {
    int W, H;
    Frag* f;     // W*H fragments, shared by band workers
    int y0, y1;  // raster rows this worker may write [y0, y1)
    bool in(int64_t x, int64_t y) const { return x >= 0 && x < W && y >= 0 && y < H; }
    // FragmentOffset(x, H-y-1) (buffer/buffer.go:209-213)
    Frag& at(int64_t x, int64_t y) const { return f[(size_t)(H - y - 1) * W + (size_t)x]; }
};

struct MVP {
    M4 model, view, proj, viewport, normal, viewInv, projInv, viewportInv, trans;
};

// sRGB LUT (color/srgb.go:57-75): 1024 + 1 float64 entries.
struct SRGB {
    double lut[1025];
    uint8_t table[256];  // GammaCorrection per channel value (shader/gamma.go:13-18)
    SRGB() {
        for (int i = 0; i < 1024; i++) {
            double v = (double)i / 1024;
            lut[i] = v <= 0.0031308 ? v * 12.92 : 1.055 * gomath::go_pow(v, 5.0 / 12.0) - 0.055;
        }
        lut[1024] = lut[1023];
        for (int c = 0; c < 256; c++) {
            float v = (float)c / 255.0f;
            table[c] = go_f2u8(from_linear(v) * 255.0f + 0.5f);
        }
    }
    // FromLinear2sRGB (color/srgb.go:15-33), float32 instance
    float from_linear(float v) const {
        if (v <= 0) return 0;
        if (v == 1) return 1;
        float i = v * 1024.0f;
        int64_t ifl = go_f2i(i) & 1023;
        float v0 = (float)lut[ifl];
        float v1 = (float)lut[ifl + 1];
        i -= (float)ifl;
        return v0 * (1.0f - i) + v1 * i;
    }
};
const SRGB& srgb() {
    static SRGB s;
    return s;
}

struct OTex;

struct Ctx {
    const pr_scene_desc* sc;
    const pr_frame_desc* fr;
    const std::vector<const OTex*>* mat_tex = nullptr;  // image texture of each material, or null
    int W, H, SW, SH;
    int M;  // render.MSAA: W, H are already M times the image
    bool perspect;
    FB* fb;
};

V4 load4(const float* p) { return {p[0], p[1], p[2], p[3]}; }
M4 loadm(const float* p) {
    M4 m;
    std::memcpy(m.m, p, sizeof(m.m));
    return m;
}

Vtx vertex(const pr_scene_desc* sc, uint32_t t, int k) {
    Vtx v;
    size_t i = (size_t)t * 3 + k;
    v.pos = load4(sc->pos + i * 4);
    v.nor = load4(sc->nor + i * 4);
    std::memcpy(v.col, sc->col + i * 4, 4);
    v.uv = {sc->uv[i * 2], sc->uv[i * 2 + 1]};
    return v;
}

// ---------------------------------------------------------------- forward

// drawClipped (render/raster.go:462-572)
void draw_clipped(Ctx& c, const MVP& mvp, const Vtx& t1, const Vtx& t2, const Vtx& t3,
                  const float recipw[3], int64_t matid, uint32_t tri) {
    FB& buf = *c.fb;
    V4 m1 = apply4(apply4(apply4(t1.pos, mvp.viewportInv), mvp.projInv), mvp.viewInv);
    V4 m2 = apply4(apply4(apply4(t2.pos, mvp.viewportInv), mvp.projInv), mvp.viewInv);
    V4 m3 = apply4(apply4(apply4(t3.pos, mvp.viewportInv), mvp.projInv), mvp.viewInv);
    V3 ps[3] = {to3(t1.pos), to3(t2.pos), to3(t3.pos)};
    AABB aabb = new_aabb(ps, 3);
    int64_t xmin = go_f2i(pround(aabb.mn.x) - 1);
    int64_t xmax = go_f2i(pround(aabb.mx.x) + 1);
    int64_t ymin = go_f2i(pround(aabb.mn.y) - 1);
    int64_t ymax = go_f2i(pround(aabb.mx.y) + 1);
    V4 fN = unit4(cross4(sub4(m2, m1), sub4(m3, m1)));
    // The reference loops over the whole rectangle and skips pixels outside
    // the buffer; clamping to the buffer visits the same pixels.
    int64_t x0 = std::max<int64_t>(xmin, 0), x1 = std::min<int64_t>(xmax, buf.W - 1);
    int64_t y0 = std::max<int64_t>(ymin, buf.y0), y1 = std::min<int64_t>(ymax, buf.y1 - 1);
    bool persp = c.perspect;
    for (int64_t x = x0; x <= x1; x++) {
        for (int64_t y = y0; y <= y1; y++) {
            V2 p = {(float)x + 0.5f, (float)y + 0.5f};
            float bc[3];
            barycoord(p, to2(t1.pos), to2(t2.pos), to2(t3.pos), bc);
            const float eps = 1e-7f;
            if (bc[0] < -eps || bc[1] < -eps || bc[2] < -eps) continue;
            float z = bc[0] * t1.pos.z + bc[1] * t2.pos.z + bc[2] * t3.pos.z;
            Frag& old = buf.at(x, y);
            // DepthTest (buffer/buffer.go:269-280)
            if (!(!old.ok || z > old.depth)) continue;
            float wc1 = recipw[0] * bc[0], wc2 = recipw[1] * bc[1], wc3 = recipw[2] * bc[2];
            float norm = 1.0f;
            if (persp) norm = 1 / (wc1 + wc2 + wc3);
            float uvX = (wc1 * t1.uv.x + wc2 * t2.uv.x + wc3 * t3.uv.x) * norm;
            float uvY = (wc1 * t1.uv.y + wc2 * t2.uv.y + wc3 * t3.uv.y) * norm;
            float du = 0, dv = 0;
            if (matid >= 0) {
                V2 q1 = {p.x + 1, p.y};
                V2 q2 = {p.x, p.y + 1};
                float bcx[3], bcy[3];
                barycoord(q1, to2(t1.pos), to2(t2.pos), to2(t3.pos), bcx);
                float wc1x = recipw[0] * bcx[0], wc2x = recipw[1] * bcx[1], wc3x = recipw[2] * bcx[2];
                float normx = 1 / (wc1x + wc2x + wc3x);
                barycoord(q2, to2(t1.pos), to2(t2.pos), to2(t3.pos), bcy);
                float wc1y = recipw[0] * bcy[0], wc2y = recipw[1] * bcy[1], wc3y = recipw[2] * bcy[2];
                float normy = 1 / (wc1y + wc2y + wc3y);
                float uvdU = (wc1x * t1.uv.x + wc2x * t2.uv.x + wc3x * t3.uv.x) * normx;
                float uvdX = (wc1x * t1.uv.y + wc2x * t2.uv.y + wc3x * t3.uv.y) * normx;
                float uvdV = (wc1y * t1.uv.x + wc2y * t2.uv.x + wc3y * t3.uv.x) * normy;
                float uvdY = (wc1y * t1.uv.y + wc2y * t2.uv.y + wc3y * t3.uv.y) * normy;
                du = (uvdU - uvX) * (uvdU - uvX) + (uvdX - uvY) * (uvdX - uvY);
                dv = (uvdV - uvX) * (uvdV - uvX) + (uvdY - uvY) * (uvdY - uvY);
            }
            V4 n = unit4(V4{bc[0] * t1.nor.x + bc[1] * t2.nor.x + bc[2] * t3.nor.x,
                            bc[0] * t1.nor.y + bc[1] * t2.nor.y + bc[2] * t3.nor.y,
                            bc[0] * t1.nor.z + bc[1] * t2.nor.z + bc[2] * t3.nor.z, 0});
            // interpWorldPos (render/raster.go:453-460)
            V4 wp = {bc[0] * m1.x + bc[1] * m2.x + bc[2] * m3.x, bc[0] * m1.y + bc[1] * m2.y + bc[2] * m3.y,
                     bc[0] * m1.z + bc[1] * m2.z + bc[2] * m3.z, 1};
            uint8_t col[4];
            for (int k = 0; k < 4; k++) {
                float s = (wc1 * (float)t1.col[k] + wc2 * (float)t2.col[k] + wc3 * (float)t3.col[k]) * norm;
                col[k] = go_f2u8(pclamp(s, 0, 255));
            }
            // Set (buffer/buffer.go:221-266): store unless Ok && depth <= old
            if (old.ok && z <= old.depth) continue;
            Frag nf;
            nf.ok = true;
            nf.x = x;
            nf.y = y;
            nf.depth = z;
            nf.u = uvX;
            nf.v = uvY;
            nf.du = du;
            nf.dv = dv;
            nf.nor = n;
            std::memcpy(nf.col, col, 4);
            nf.matid = matid;
            nf.fnor = fN;
            nf.wpos = wp;
            nf.tri = tri;
            old = nf;
        }
    }
}

// plane / sutherlandHodgman (render/clipping.go:18-68)
struct Plane { V4 pos, nor; };
bool in_front(const Plane& p, V4 v) { return dot4(sub4(v, p.pos), p.nor) > 0; }
V4 intersect_seg(const Plane& p, V4 v0, V4 v1) {
    V4 u = sub4(v1, v0);
    V4 w = sub4(v0, p.pos);
    float d = dot4(p.nor, u);
    float n = -dot4(p.nor, w);
    float s = n / d;
    return add4(v0, scale4(u, s, s, s, s));
}
std::vector<V4> sutherland_hodgman(const std::vector<V4>& points, float w, float h) {
    const Plane planes[6] = {
        {{w, 0, 0, 1}, {-1, 0, 0, 1}}, {{0, 0, 0, 1}, {1, 0, 0, 1}},
        {{0, h, 0, 1}, {0, -1, 0, 1}}, {{0, 0, 0, 1}, {0, 1, 0, 1}},
        {{0, 0, 1, 1}, {0, 0, -1, 1}}, {{0, 0, -1, 1}, {0, 0, 1, 1}},
    };
    std::vector<V4> output = points;
    for (const Plane& pl : planes) {
        std::vector<V4> input = output;
        output.clear();
        if (input.empty()) return {};
        V4 s = input.back();
        for (const V4& e : input) {
            if (in_front(pl, e)) {
                if (!in_front(pl, s)) output.push_back(intersect_seg(pl, s, e));
                output.push_back(e);
            } else if (in_front(pl, s)) {
                output.push_back(intersect_seg(pl, s, e));
            }
            s = e;
        }
    }
    return output;
}

// clipTriangle (render/clipping.go:70-157): fan over the clipped polygon,
// each new vertex re-interpolated by screen barycentrics of the parent.
Vtx clip_vertex(V4 cp, const Vtx& v1, const Vtx& v2, const Vtx& v3) {
    float b[3];
    barycoord(V2{cp.x, cp.y}, to2(v1.pos), to2(v2.pos), to2(v3.pos), b);
    Vtx r;
    r.pos = {b[0] * v1.pos.x + b[1] * v2.pos.x + b[2] * v3.pos.x,
             b[0] * v1.pos.y + b[1] * v2.pos.y + b[2] * v3.pos.y,
             b[0] * v1.pos.z + b[1] * v2.pos.z + b[2] * v3.pos.z, 1};
    r.uv = {b[0] * v1.uv.x + b[1] * v2.uv.x + b[2] * v3.uv.x, b[0] * v1.uv.y + b[1] * v2.uv.y + b[2] * v3.uv.y};
    r.nor = {b[0] * v1.nor.x + b[1] * v2.nor.x + b[2] * v3.nor.x,
             b[0] * v1.nor.y + b[1] * v2.nor.y + b[2] * v3.nor.y,
             b[0] * v1.nor.z + b[1] * v2.nor.z + b[2] * v3.nor.z, 0};
    for (int k = 0; k < 4; k++)
        r.col[k] = go_f2u8(pclamp(b[0] * (float)v1.col[k] + b[1] * (float)v2.col[k] + b[2] * (float)v3.col[k], 0, 255));
    return r;
}

// draw (render/raster.go:380-444)
void draw(Ctx& c, const MVP& mvp, const Vtx& in1, const Vtx& in2, const Vtx& in3, int64_t matid,
          uint32_t tri, bool* clipped) {
    Vtx t1, t2, t3;
    const Vtx* ins[3] = {&in1, &in2, &in3};
    Vtx* outs[3] = {&t1, &t2, &t3};
    for (int k = 0; k < 3; k++) {
        outs[k]->pos = mulv(mvp.trans, ins[k]->pos);
        std::memcpy(outs[k]->col, ins[k]->col, 4);
        outs[k]->uv = ins[k]->uv;
        outs[k]->nor = apply4(ins[k]->nor, mvp.normal);
    }
    float recipw[3] = {1, 1, 1};
    if (c.perspect) {
        recipw[0] = -1 / t1.pos.w;
        recipw[1] = -1 / t2.pos.w;
        recipw[2] = -1 / t3.pos.w;
    }
    t1.pos = pos4(apply4(t1.pos, mvp.viewport));
    t2.pos = pos4(apply4(t2.pos, mvp.viewport));
    t3.pos = pos4(apply4(t3.pos, mvp.viewport));
    // cullBackFace (render/cull.go:26-28)
    if (cross4(sub4(t2.pos, t1.pos), sub4(t3.pos, t1.pos)).z < 0) return;
    V3 ps[3] = {to3(t1.pos), to3(t2.pos), to3(t3.pos)};
    // viewportAABB: Max = MSAA * the (already MSAA-sized) buffer
    AABB vp{{0, 0, -1}, {(float)(c.M * c.W), (float)(c.M * c.H), 1}};
    if (!aabb_intersect(vp, new_aabb(ps, 3))) return;
    if (aabb_contains(vp, ps, 3)) {
        draw_clipped(c, mvp, t1, t2, t3, recipw, matid, tri);
        return;
    }
    if (clipped) *clipped = true;
    std::vector<V4> clips = sutherland_hodgman({t1.pos, t2.pos, t3.pos}, (float)(c.M * c.W), (float)(c.M * c.H));
    for (size_t i = 2; i < clips.size(); i++) {
        Vtx a = clip_vertex(clips[0], t1, t2, t3);
        Vtx b = clip_vertex(clips[i - 1], t1, t2, t3);
        Vtx d = clip_vertex(clips[i], t1, t2, t3);
        draw_clipped(c, mvp, a, b, d, recipw, matid, tri);
    }
}

bool build_mvp(const Ctx& c, const pr_object& ob, MVP* mvp) {
    mvp->view = loadm(c.fr->view);
    mvp->proj = loadm(c.fr->proj);
    mvp->viewport = viewport((float)c.W, (float)c.H);
    mvp->model = loadm(ob.model);
    M4 mi;
    if (!inv(mvp->model, &mi)) return false;
    mvp->normal = transpose(mi);
    if (!inv(mvp->view, &mvp->viewInv)) return false;
    if (!inv(mvp->proj, &mvp->projInv)) return false;
    if (!inv(mvp->viewport, &mvp->viewportInv)) return false;
    mvp->trans = mulm(mulm(mvp->proj, mvp->view), mvp->model);
    return true;
}

int forward_pass(Ctx& c, orc_stats* st) {
    const pr_scene_desc* sc = c.sc;
    for (uint32_t o = 0; o < sc->n_objects; o++) {
        const pr_object& ob = sc->objects[o];
        MVP mvp;
        if (!build_mvp(c, ob, &mvp)) return PR_ERR_SINGULAR;
        for (uint32_t t = ob.first_tri; t < ob.first_tri + ob.n_tris; t++) {
            int64_t matid = sc->mat_id[t];
            if (matid >= 0) matid += ob.mat_base;
            Vtx v1 = vertex(sc, t, 0), v2 = vertex(sc, t, 1), v3 = vertex(sc, t, 2);
            if (!tri_is_valid(v1.pos, v2.pos, v3.pos)) continue;
            bool clipped = false;
            draw(c, mvp, v1, v2, v3, matid, t, &clipped);
            if (st && clipped) st->n_clipped++;
        }
    }
    return PR_OK;
}

// ---------------------------------------------------------------- shadows

// drawDepth (render/shadow.go:152-219) + shadowDepthTest (:221-228), rows [y0,y1)
void draw_depth(const Ctx& c, float* depths, const MVP& mvp, const Vtx& v1, const Vtx& v2,
                const Vtx& v3, int y0r, int y1r) {
    V4 p[3];
    const Vtx* vs[3] = {&v1, &v2, &v3};
    for (int k = 0; k < 3; k++) p[k] = pos4(apply4(mulv(mvp.trans, vs[k]->pos), mvp.viewport));
    if (cross4(sub4(p[1], p[0]), sub4(p[2], p[0])).z < 0) return;
    // cullViewFrustum (render/cull.go:15-23)
    V3 vpc[3] = {{(float)(c.SW * c.M), (float)(c.SH * c.M), 1}, {0, 0, 0}, {0, 0, -1}};
    AABB vp = new_aabb(vpc, 3);
    V3 ps[3] = {to3(p[0]), to3(p[1]), to3(p[2])};
    AABB ta = new_aabb(ps, 3);
    if (!aabb_intersect(vp, ta)) return;
    int64_t xmin = go_f2i(pround(ta.mn.x) - 1);
    int64_t xmax = go_f2i(pround(ta.mx.x) + 1);
    int64_t ymin = go_f2i(pround(ta.mn.y) - 1);
    int64_t ymax = go_f2i(pround(ta.mx.y) + 1);
    int64_t x0 = std::max<int64_t>(xmin, 0), x1 = std::min<int64_t>(xmax, c.SW - 1);
    int64_t y0 = std::max<int64_t>(ymin, y0r), y1 = std::min<int64_t>(ymax, y1r - 1);
    for (int64_t x = x0; x <= x1; x++) {
        for (int64_t y = y0; y <= y1; y++) {
            V2 pp = {(float)x + 0.5f, (float)y + 0.5f};
            float bc[3];
            barycoord(pp, to2(p[0]), to2(p[1]), to2(p[2]), bc);
            const float eps = 1e-7f;
            if (bc[0] < -eps || bc[1] < -eps || bc[2] < -eps) continue;
            float z = bc[0] * p[0].z + bc[1] * p[1].z + bc[2] * p[2].z;
            size_t idx = (size_t)x + (size_t)y * c.SW;
            if (!(z <= depths[idx])) depths[idx] = z;
        }
    }
}

int shadow_pass(const Ctx& c, int li, float* depths, int y0r, int y1r) {
    const pr_light& L = c.fr->lights[li];
    const pr_scene_desc* sc = c.sc;
    for (uint32_t o = 0; o < sc->n_objects; o++) {
        const pr_object& ob = sc->objects[o];
        MVP mvp;
        mvp.model = loadm(ob.model);
        mvp.view = loadm(L.shadow_view);
        mvp.proj = loadm(L.shadow_proj);
        mvp.viewport = viewport((float)c.SW, (float)c.SH);
        mvp.trans = mulm(mulm(mvp.proj, mvp.view), mvp.model);
        M4 mi;
        if (!inv(mvp.model, &mi)) return PR_ERR_SINGULAR;  // mvp.Normal (render/shadow.go:135)
        for (uint32_t t = ob.first_tri; t < ob.first_tri + ob.n_tris; t++) {
            Vtx v1 = vertex(sc, t, 0), v2 = vertex(sc, t, 1), v3 = vertex(sc, t, 2);
            if (!tri_is_valid(v1.pos, v2.pos, v3.pos)) continue;
            draw_depth(c, depths, mvp, v1, v2, v3, y0r, y1r);
        }
    }
    return PR_OK;
}

// ---------------------------------------------------------------- shading

struct ShadeUniforms {
    M4 viewport, s2w;
    std::vector<M4> lview, lproj;
    M4 shadow_vp;
    float ao_cos[8], ao_sin[8];
    int n_ao_dirs;
};

// shadingVisibility (render/shadow.go:230-283): true = occluded
bool shading_visibility(const Ctx& c, const ShadeUniforms& u, int li, const Frag& info, const float* depths) {
    const pr_light& L = c.fr->lights[li];
    if (!L.cast_shadow) return true;
    V4 sc = pos4(apply4(apply4(apply4(apply4(V4{(float)info.x, (float)info.y, info.depth, 1}, u.s2w), u.lview[li]),
                               u.lproj[li]),
                        u.shadow_vp));
    int64_t lx = go_f2i(sc.x), ly = go_f2i(sc.y);
    // Go int arithmetic wraps (two's complement).
    int64_t idx = (int64_t)((uint64_t)lx + (uint64_t)ly * (uint64_t)(int64_t)c.SW);
    int64_t len = (int64_t)c.SW * c.SH;
    float shadow = 0;
    if (idx > 0 && idx < len) {
        float sz = depths[idx];
        const float bias = 0.03f;
        if (sc.z < sz - bias) shadow++;
    }
    return shadow > 0;
}

// ---- textures: buffer.NewTexture and Texture.Query (buffer/texture.go:35-187)

// ---- passAntialiasing: imageutil.Resize (internal/imageutil/resize.go:16-181)

float resize_linear(float in) {
    in = std::fabs(in);
    if (in <= 1) return 1 - in;
    return 0;
}

// createWeights8 with the linear kernel: int16 taps (x256) and start indices
void create_weights8(int dy, int filter_length, float scale, std::vector<int16_t>& coeffs, std::vector<int>& start,
                     int& len) {
    len = filter_length * (int)std::max(std::ceil(scale), 1.0f);
    float factor = std::min(1.0f / scale, 1.0f);
    coeffs.assign((size_t)dy * len, 0);
    start.assign(dy, 0);
    for (int y = 0; y < dy; y++) {
        float interp = scale * ((float)y + 0.5f) - 0.5f;
        start[y] = (int)interp - len / 2 + 1;
        interp -= (float)start[y];
        for (int i = 0; i < len; i++) {
            float in = (interp - (float)i) * factor;
            coeffs[(size_t)y * len + i] = (int16_t)(resize_linear(in) * 256);
        }
    }
}

// resizeRGBA: `in` has in_dx pixels per row; writes out (out_dx x out_dy),
// out row y column x from in row x (the passes transpose).
void resize_rgba(const uint8_t* in, int in_dx, uint8_t* out, int out_dx, int out_dy,
                 const std::vector<int16_t>& coeffs, const std::vector<int>& start, int len) {
    const int maxX = in_dx - 1;
    for (int x = 0; x < out_dx; x++) {
        const uint8_t* row = in + (size_t)x * in_dx * 4;
        for (int y = 0; y < out_dy; y++) {
            int32_t rgba[4] = {0, 0, 0, 0}, sum = 0;
            for (int i = 0; i < len; i++) {
                int32_t coeff = coeffs[(size_t)y * len + i];
                if (coeff == 0) continue;
                int xi = start[y] + i;
                if ((unsigned)xi < (unsigned)maxX)
                    xi *= 4;
                else if (xi >= maxX)
                    xi = 4 * maxX;
                else
                    xi = 0;
                for (int k = 0; k < 4; k++) rgba[k] += coeff * (int32_t)row[xi + k];
                sum += coeff;
            }
            for (int k = 0; k < 4; k++) {
                int v = rgba[k] / sum;
                out[((size_t)y * out_dx + x) * 4 + k] = (uint8_t)std::min(std::max(v, 0), 255);
            }
        }
    }
}

void resize_image(const uint8_t* img, int dx, int dy, int width, int height, uint8_t* out) {
    float scale_x = (float)dx / (float)width, scale_y = (float)dy / (float)height;
    std::vector<int16_t> coeffs;
    std::vector<int> start;
    int len;
    std::vector<uint8_t> temp((size_t)dy * width * 4);  // Dx = dy, Dy = width (transposed)
    create_weights8(width, 2, scale_x, coeffs, start, len);
    resize_rgba(img, dx, temp.data(), dy, width, coeffs, start, len);
    create_weights8(height, 2, scale_y, coeffs, start, len);
    resize_rgba(temp.data(), dy, out, width, height, coeffs, start, len);
}


struct OImg {  // image.RGBA: rows top-down
    int w = 0, h = 0;
    std::vector<uint8_t> pix;
};

struct OTex {
    bool use_mipmap = true;
    std::vector<OImg> mipmap;
};

// imageutil.Resize(width, height, img) (internal/imageutil/resize.go:16-66)
OImg go_resize_img(int width, int height, const OImg& img) {
    float scale_x, scale_y;  // calcFactors (resize.go:124-144)
    const float old_w = (float)img.w, old_h = (float)img.h;
    if (width == 0) {
        if (height == 0) {
            scale_x = 1.0f;
            scale_y = 1.0f;
        } else {
            scale_y = old_h / (float)height;
            scale_x = scale_y;
        }
    } else {
        scale_x = old_w / (float)width;
        if (height == 0)
            scale_y = scale_x;
        else
            scale_y = old_h / (float)height;
    }
    if (width == 0) width = (int)(0.7f + old_w / scale_x);
    if (height == 0) height = (int)(0.7f + old_h / scale_y);
    if (width == img.w && height == img.h) return img;
    if (img.w <= 0 || img.h <= 0) return img;
    std::vector<uint8_t> temp((size_t)img.h * width * 4);  // image.NewRGBA(Rect(0, 0, Dy, width))
    OImg out;
    out.w = width;
    out.h = height;
    out.pix.assign((size_t)width * height * 4, 0);
    std::vector<int16_t> coeffs;
    std::vector<int> start;
    int len;
    create_weights8(width, 2, scale_x, coeffs, start, len);
    resize_rgba(img.pix.data(), img.w, temp.data(), img.h, width, coeffs, start, len);
    create_weights8(height, 2, scale_y, coeffs, start, len);
    resize_rgba(temp.data(), img.h, out.pix.data(), width, height, coeffs, start, len);
    return out;
}

// NewTexture (buffer/texture.go:35-67): every level a Resize of the image
OTex new_texture(const OImg& image, bool use_mipmap) {
    OTex t;
    t.use_mipmap = use_mipmap;
    const int dx = image.w, dy = image.h;
    if (dx == 1 && dy == 1) {
        t.mipmap.push_back(image);
        return t;
    }
    const int L = (int)(float)gomath::go_log2((double)gomath::pmax((float)dx, (float)dy)) + 1;
    t.mipmap.resize(L);
    t.mipmap[0] = image;
    for (int i = 1; i < L; i++) {
        const int p = (int)(float)std::pow(2.0, (double)(float)i);
        t.mipmap[i] = go_resize_img(dx / p, dy / p, image);
    }
    return t;
}

typedef std::array<uint8_t, 4> RGBA;

RGBA rgba_at(const OImg& b, int64_t x, int64_t y) {  // image.RGBA.RGBAAt
    if (x < 0 || y < 0 || x >= b.w || y >= b.h) return RGBA{0, 0, 0, 0};
    const uint8_t* p = &b.pix[((size_t)y * b.w + (size_t)x) * 4];
    return RGBA{p[0], p[1], p[2], p[3]};
}

RGBA lerp_c(RGBA from, RGBA to, float t) {  // math.LerpC (math/interpolate.go:55-62)
    RGBA r;
    for (int k = 0; k < 4; k++) r[k] = go_f2u8((float)from[k] + t * ((float)to[k] - (float)from[k]));
    return r;
}

float go_floor32(float x) { return (float)std::floor((double)x); }

RGBA query_l0(const OTex& t, float u, float v) {
    const OImg& tex = t.mipmap[0];
    const float dx = (float)tex.w, dy = (float)tex.h;
    if (dx == 1 && dy == 1) return rgba_at(tex, 0, 0);
    const int64_t x = go_f2i(go_floor32(u * (dx - 1)));
    const int64_t y = go_f2i(go_floor32(v * (dy - 1)));
    return rgba_at(tex, x, y);
}

RGBA query_bilinear(const OTex& t, int lod, float u, float v) {
    const OImg& buf = t.mipmap[lod];
    const int dx = buf.w, dy = buf.h;
    if (dx == 1 && dy == 1) return rgba_at(buf, 0, 0);
    const float x = u * ((float)dx - 1);
    const float y = v * ((float)dy - 1);
    const float x0 = go_floor32(x), y0 = go_floor32(y);
    const int64_t i = go_f2i(x0), j = go_f2i(y0);
    RGBA p1 = rgba_at(buf, i, j), p2, p3, p4;
    if (i < dx - 1)
        p2 = rgba_at(buf, i + 1, j);
    else
        p2 = rgba_at(buf, i, j);
    RGBA interpo1 = lerp_c(p1, p2, x - x0);
    if (j < dy - 1)
        p3 = rgba_at(buf, i, j + 1);
    else
        p3 = rgba_at(buf, i, j);
    if (i < dx - 1 && j < dy - 1)
        p4 = rgba_at(buf, i + 1, j + 1);
    else
        p4 = rgba_at(buf, i, j);
    RGBA interpo2 = lerp_c(p3, p4, x - x0);
    return lerp_c(interpo1, interpo2, y - y0);
}

// math.Modf on float32 through float64; Modf(+-Inf) = +-Inf, NaN
float go_modf32(float f, float* ip) {
    if (std::isinf(f)) {
        *ip = f;
        return NAN;
    }
    double i;
    const double fr = std::modf((double)f, &i);
    *ip = (float)i;
    return (float)fr;
}

// Texture.Query (buffer/texture.go:83-129); where the reference indexes
// the mipmap out of range (NaN lod), transparent black.
RGBA texture_query(const OTex& t, float lod, float u, float v) {
    float iu, iv;
    u = go_modf32(u, &iu);
    if (iu != 0 && u == 0) u = 1;
    if (u < 0) u = 1 - u;
    v = go_modf32(v, &iv);
    if (iv != 0 && v == 0) v = 1;
    if (v < 0) v = 1 - v;
    if (!t.use_mipmap) return query_l0(t, u, v);
    const int n = (int)t.mipmap.size();
    if (lod < 0)
        lod = 0;
    else if (lod >= (float)n)
        lod = (float)(n - 1);
    if (lod <= 1) return query_bilinear(t, 0, u, v);
    lod -= 1;
    const int64_t h = go_f2i(go_floor32(lod));
    const int64_t l = h + 1;
    if (h < 0 || h >= n) return RGBA{0, 0, 0, 0};
    if (l >= n) return query_bilinear(t, (int)h, u, v);
    const float p = lod - (float)h;
    if ((float)std::fabs((double)(p - 0)) <= 1e-7f) return query_bilinear(t, (int)h, u, v);
    return lerp_c(query_bilinear(t, (int)h, u, v), query_bilinear(t, (int)l, u, v), p);
}

// FragmentShader's lod and query (shader/blinn_cpu.go:28-36)
RGBA texture_colour(const OTex& t, float du, float dv, float u, float v) {
    float lod = 0;
    if (t.use_mipmap) {
        float siz = (float)t.mipmap[0].w * (float)std::sqrt((double)gomath::pmax(du, dv));
        if (siz < 1) siz = 1;
        lod = (float)gomath::go_log2((double)siz);
    }
    return texture_query(t, lod, u, 1 - v);
}

// FragmentShader (shader/blinn_cpu.go:24-106)
void fragment_shader(const pr_material& m, const Frag& info, V3 cam, const pr_light* ls, int nl,
                     const float* amb, int na, uint8_t out[4], const OTex* tex = nullptr) {
    // Uniform textures: Query returns the single texel whatever lod/u/v
    // (buffer/texture.go:83-129, queryBilinear 1x1 path :150-156).
    uint8_t col[4] = {m.texture[0], m.texture[1], m.texture[2], m.texture[3]};
    if (tex) {
        const RGBA c = texture_colour(*tex, info.du, info.dv, info.u, info.v);
        std::memcpy(col, c.data(), 4);
    }
    if (nl == 0) {
        std::memcpy(out, col, 4);
        return;
    }
    float LaR = 0, LaG = 0, LaB = 0;
    for (int e = 0; e < na; e++) {
        LaR += amb[e] * (float)col[0];
        LaG += amb[e] * (float)col[1];
        LaB += amb[e] * (float)col[2];
    }
    float LdR = 0, LdG = 0, LdB = 0, LsR = 0, LsG = 0, LsB = 0;
    V4 n = (m.flags & PR_MAT_FLAT_SHADING) ? info.fnor : info.nor;
    V4 x = info.wpos;
    for (int i = 0; i < nl; i++) {
        const pr_light& l = ls[i];
        V4 L;
        float I;
        if (l.type == PR_LIGHT_POINT) {
            V4 Ldir = sub4(V4{l.pos[0], l.pos[1], l.pos[2], 1}, x);
            L = unit4(Ldir);
            I = l.intensity / len4(Ldir);
        } else {
            L = scale4(V4{l.dir[0], l.dir[1], l.dir[2], 0}, -1, -1, -1, 1);
            I = l.intensity;
        }
        V4 V = unit4(sub4(V4{cam.x, cam.y, cam.z, 1}, x));
        V4 H = unit4(add4(L, V));
        float Ld = pclamp(dot4(n, L), 0, 1);
        float Ls = (float)gomath::go_pow((double)pclamp(dot4(n, H), 0, 1), (double)m.shininess);
        LdR += Ld * (float)col[0] * I;
        LdG += Ld * (float)col[1] * I;
        LdB += Ld * (float)col[2] * I;
        LsR += Ls * (float)l.color[0] * I;
        LsG += Ls * (float)l.color[1] * I;
        LsB += Ls * (float)l.color[2] * I;
    }
    float r = pround(LaR + ((float)m.diffuse[0] * LdR / 255.0f) + ((float)m.specular[0] * LsR / 255.0f));
    float g = pround(LaG + ((float)m.diffuse[1] * LdG / 255.0f) + ((float)m.specular[1] * LsG / 255.0f));
    float b = pround(LaB + ((float)m.diffuse[2] * LdB / 255.0f) + ((float)m.specular[2] * LsB / 255.0f));
    out[0] = go_f2u8(pclamp(r, 0, 255));
    out[1] = go_f2u8(pclamp(g, 0, 255));
    out[2] = go_f2u8(pclamp(b, 0, 255));
    out[3] = go_f2u8(pclamp((float)col[3], 0, 255));
}

// maxElevationAngle (material/ao.go:49-73)
float max_elevation_angle(FB& buf, const Frag& info, float dirX, float dirY) {
    V4 p = {(float)info.x, (float)info.y, 0, 1};
    V4 dir = {dirX, dirY, 0, 0};
    float maxangle = 0;
    for (float t = 0; t < 100; t += 1) {
        V4 cur = add4(p, scale4(dir, t, t, 1, 1));
        int64_t cx = go_f2i(cur.x), cy = go_f2i(cur.y);
        if (!buf.in(cx, cy)) return maxangle;
        float distance = len4(sub4(p, cur));
        if (distance < 1) continue;
        const Frag& sh = buf.at(cx, cy);
        int64_t px = go_f2i(p.x), py = go_f2i(p.y);
        const Frag& tr = buf.at(px, py);
        float shadeDepth = sh.depth, traceDepth = tr.depth;
        if (!sh.ok) shadeDepth = -1;
        if (!tr.ok) traceDepth = -1;
        float elevation = shadeDepth - traceDepth;
        maxangle = (float)gomath::go_max((double)maxangle, gomath::go_atan((double)(elevation / distance)));
    }
    return maxangle;
}

// AmbientOcclusionShade (material/ao.go:20-47)
void ambient_occlusion(FB& buf, const ShadeUniforms& u, const Frag& info, const uint8_t col[4], uint8_t out[4]) {
    const float halfPi = 1.57079632679489661923f;
    const float norm = 12.5663706143591729539f;  // float32((Pi/2)*8)
    float total = 0;
    for (int k = 0; k < u.n_ao_dirs; k++) total += halfPi - max_elevation_angle(buf, info, u.ao_cos[k], u.ao_sin[k]);
    total /= norm;
    total = (float)gomath::go_pow((double)total, 10000.0);
    out[0] = go_f2u8(total * (float)col[0]);
    out[1] = go_f2u8(total * (float)col[1]);
    out[2] = go_f2u8(total * (float)col[2]);
    out[3] = col[3];
}

// shade (render/raster.go:324-359) for the fragment stored at raster (x, y)
void shade_pixel(const Ctx& c, const ShadeUniforms& u, const std::vector<float>& shadow_depths, int64_t x,
                 int64_t y, uint8_t out[4]) {
    FB& buf = *c.fb;
    const Frag& info = buf.at(x, y);
    if (!info.ok) {
        std::memcpy(out, c.fr->background, 4);
        return;
    }
    const pr_scene_desc* sc = c.sc;
    const pr_material* mat = nullptr;
    if (info.matid >= 0 && info.matid < (int64_t)sc->n_materials) mat = &sc->materials[info.matid];
    uint8_t col[4];
    std::memcpy(col, info.col, 4);
    if (mat) {
        V3 cam = {c.fr->cam_pos[0], c.fr->cam_pos[1], c.fr->cam_pos[2]};
        const OTex* tex = c.mat_tex ? (*c.mat_tex)[info.matid] : nullptr;
        fragment_shader(*mat, info, cam, c.fr->lights, (int)c.fr->n_lights, c.fr->ambient, (int)c.fr->n_ambient, col,
                        tex);
        if ((c.fr->flags & PR_FRAME_SHADOWMAP) && (mat->flags & PR_MAT_RECEIVE_SHADOW)) {
            float visibles = 0;
            size_t plane = (size_t)c.SW * c.SH;
            for (int i = 0; i < (int)c.fr->n_lights; i++)
                if (shading_visibility(c, u, i, info, shadow_depths.data() + plane * i)) visibles++;
            float w = (float)gomath::go_pow(0.5, (double)visibles);
            col[0] = go_f2u8((float)col[0] * w);
            col[1] = go_f2u8((float)col[1] * w);
            col[2] = go_f2u8((float)col[2] * w);
        }
    }
    if (mat && (mat->flags & PR_MAT_AO)) {
        ambient_occlusion(buf, u, info, col, out);
        return;
    }
    std::memcpy(out, col, 4);
}

template <class F>
void parallel_rows(int threads, int H, F&& fn) {
    if (threads <= 1) {
        fn(0, H);
        return;
    }
    std::vector<std::thread> ts;
    int per = (H + threads - 1) / threads;
    for (int i = 0; i < threads; i++) {
        int y0 = i * per, y1 = std::min(H, (i + 1) * per);
        if (y0 >= y1) break;
        ts.emplace_back([&, y0, y1] { fn(y0, y1); });
    }
    for (auto& t : ts) t.join();
}

}  // namespace

// ---------------------------------------------------------------- C API

extern "C" {

void orc_ao_directions(float cosv[8], float sinv[8], int* n) {
    // for a := float32(0.0); a < TwoPi-1e-4; a += Pi/4 (material/ao.go:28)
    const float limit = (float)(6.28318530717958647692 - 1e-4);
    const float step = 0.785398163397448309616f;
    int k = 0;
    for (float a = 0; a < limit && k < 8; a += step) {
        cosv[k] = (float)std::cos((double)a);
        sinv[k] = (float)std::sin((double)a);
        k++;
    }
    *n = k;
}

// ---- building blocks for the known-answer tests ----

void orc_barycoord(const float p[2], const float t1[2], const float t2[2], const float t3[2], float out[3]) {
    barycoord(V2{p[0], p[1]}, V2{t1[0], t1[1]}, V2{t2[0], t2[1]}, V2{t3[0], t3[1]}, out);
}
void orc_view_matrix(const float pos[3], const float target[3], const float up[3], float out[16]) {
    M4 m = view_matrix(V3{pos[0], pos[1], pos[2]}, V3{target[0], target[1], target[2]}, V3{up[0], up[1], up[2]});
    std::memcpy(out, m.m, 64);
}
void orc_perspective_matrix(float fov, float aspect, float n, float f, float out[16]) {
    M4 m = perspective_matrix(fov, aspect, n, f);
    std::memcpy(out, m.m, 64);
}
void orc_ortho_matrix(float l, float r, float b, float t, float n, float f, float out[16]) {
    M4 m = ortho_matrix(l, r, b, t, n, f);
    std::memcpy(out, m.m, 64);
}
void orc_mat4_mul(const float a[16], const float b[16], float out[16]) {
    M4 m = mulm(loadm(a), loadm(b));
    std::memcpy(out, m.m, 64);
}
int orc_mat4_inv(const float m[16], float out[16]) {
    M4 r;
    if (!inv(loadm(m), &r)) return PR_ERR_SINGULAR;
    std::memcpy(out, r.m, 64);
    return PR_OK;
}
int orc_aabb_intersect(const float a_min[3], const float a_max[3], const float b_min[3], const float b_max[3]) {
    AABB a{{a_min[0], a_min[1], a_min[2]}, {a_max[0], a_max[1], a_max[2]}};
    AABB b{{b_min[0], b_min[1], b_min[2]}, {b_max[0], b_max[1], b_max[2]}};
    return aabb_intersect(a, b) ? 1 : 0;
}
int orc_aabb_contains(const float a_min[3], const float a_max[3], const float* pts, int n) {
    AABB a{{a_min[0], a_min[1], a_min[2]}, {a_max[0], a_max[1], a_max[2]}};
    std::vector<V3> v(n);
    for (int i = 0; i < n; i++) v[i] = {pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]};
    return aabb_contains(a, v.data(), n) ? 1 : 0;
}
void orc_new_aabb(const float* pts, int n, float out_min[3], float out_max[3]) {
    std::vector<V3> v(n);
    for (int i = 0; i < n; i++) v[i] = {pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]};
    AABB a = new_aabb(v.data(), n);
    out_min[0] = a.mn.x; out_min[1] = a.mn.y; out_min[2] = a.mn.z;
    out_max[0] = a.mx.x; out_max[1] = a.mx.y; out_max[2] = a.mx.z;
}
int orc_tri_is_valid(const float p1[4], const float p2[4], const float p3[4]) {
    return tri_is_valid(load4(p1), load4(p2), load4(p3)) ? 1 : 0;
}
// Triangle.Normal / NewTriangle face normal (geometry/primitive/triangle.go:19-37)
void orc_tri_face_normal(const float p1[4], const float p2[4], const float p3[4], float out[4]) {
    V4 v2v1 = sub4(load4(p1), load4(p2));
    V4 v2v3 = sub4(load4(p3), load4(p2));
    V4 n = unit4(cross4(v2v3, v2v1));
    std::memcpy(out, &n, 16);
}
void orc_fragment_shader(const pr_material* m, const float nor[4], const float face_nor[4], const float wpos[4],
                         const float cam[3], const pr_light* lights, int n_lights, const float* ambient,
                         int n_ambient, uint8_t out[4]) {
    Frag f;
    std::memset(&f, 0, sizeof(f));
    f.ok = true;
    f.nor = load4(nor);
    f.fnor = load4(face_nor);
    f.wpos = load4(wpos);
    fragment_shader(*m, f, V3{cam[0], cam[1], cam[2]}, lights, n_lights, ambient, n_ambient, out);
}
void orc_interp_world_pos(const float bc[3], const float m1[4], const float m2[4], const float m3[4], float out[4]) {
    out[0] = bc[0] * m1[0] + bc[1] * m2[0] + bc[2] * m3[0];
    out[1] = bc[0] * m1[1] + bc[1] * m2[1] + bc[2] * m3[1];
    out[2] = bc[0] * m1[2] + bc[1] * m2[2] + bc[2] * m3[2];
    out[3] = 1;
}
void orc_gamma_table(uint8_t out[256]) { std::memcpy(out, srgb().table, 256); }
float orc_from_linear_srgb(float v) { return srgb().from_linear(v); }
double orc_go_pow(double x, double y) { return gomath::go_pow(x, y); }
double orc_go_atan(double x) { return gomath::go_atan(x); }
float orc_fma32(float x, float y, float z) { return gomath::fma32(x, y, z); }
int64_t orc_go_f2i(float x) { return go_f2i(x); }
uint8_t orc_go_f2u8(float x) { return go_f2u8(x); }

// initShadowMaps' light camera (render/shadow.go:41-85)
int orc_shadow_camera(const float light_pos[3], const float center[3], const float cam_view[16],
                      const float cam_proj[16], float out_view[16], float out_proj[16]) {
    V3 lp{light_pos[0], light_pos[1], light_pos[2]};
    V3 ct{center[0], center[1], center[2]};
    M4 lv = view_matrix(lp, ct, V3{0, 1, 0});
    M4 vinv, pinv;
    if (!inv(loadm(cam_view), &vinv) || !inv(loadm(cam_proj), &pinv)) return PR_ERR_SINGULAR;
    M4 tm = mulm(mulm(lv, vinv), pinv);
    const float corners[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {-1, 1, 1},
                                 {-1, -1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, -1}};
    V3 v[8];
    for (int i = 0; i < 8; i++) v[i] = to3(pos4(apply4(V4{corners[i][0], corners[i][1], corners[i][2], 1}, tm)));
    AABB a = new_aabb(v, 8);
    float le = a.mn.x, ri = a.mx.x, bo = a.mn.y, to = a.mx.y, ne = a.mx.z, fa = a.mn.z - 2;
    M4 pr = ortho_matrix(le, ri, bo, to, ne, fa);
    std::memcpy(out_view, lv.m, 64);
    std::memcpy(out_proj, pr.m, 64);
    return PR_OK;
}

// NewTexture's levels (level 0 alone without mipmaps): texels into out
// (capacity cap, in texels), [n, w0, h0, off0, ...] into desc (1 + 3*16).
long long orc_texture_build(int w, int h, const uint8_t* rgba, int mipmap, uint8_t* out, size_t cap, int32_t* desc) {
    if (w < 1 || h < 1 || !rgba) return PR_ERR_INVALID_ARG;
    OImg img;
    img.w = w;
    img.h = h;
    img.pix.assign(rgba, rgba + (size_t)w * h * 4);
    OTex t = new_texture(img, mipmap != 0);
    const int n = mipmap ? (int)t.mipmap.size() : 1;
    size_t off = 0;
    if (desc) std::memset(desc, 0, sizeof(int32_t) * (1 + 3 * 16));
    if (desc) desc[0] = n;
    for (int i = 0; i < n && i < 16; i++) {
        const OImg& lv = t.mipmap[i];
        if (desc) {
            desc[1 + 3 * i] = lv.w;
            desc[2 + 3 * i] = lv.h;
            desc[3 + 3 * i] = (int32_t)off;
        }
        const size_t cnt = (size_t)lv.w * lv.h;
        if (out && off + cnt <= cap) std::memcpy(out + off * 4, lv.pix.data(), cnt * 4);
        off += cnt;
    }
    return (long long)off;
}

// Texture.Query of n (lod, u, v) triples, or with du / dv the
// FragmentShader's lod of (du[k], dv[k]); v is passed to Query as given.
int orc_texture_query(int w, int h, const uint8_t* rgba, int mipmap, int n, const float* lod, const float* du,
                      const float* dv, const float* u, const float* v, uint8_t* out) {
    if (w < 1 || h < 1 || !rgba || !u || !v || !out || (!lod && !(du && dv))) return PR_ERR_INVALID_ARG;
    OImg img;
    img.w = w;
    img.h = h;
    img.pix.assign(rgba, rgba + (size_t)w * h * 4);
    OTex t = new_texture(img, mipmap != 0);
    for (int k = 0; k < n; k++) {
        float l = lod ? lod[k] : 0.0f;
        if (du && dv) {
            l = 0;
            if (t.use_mipmap) {
                float siz = (float)t.mipmap[0].w * (float)std::sqrt((double)gomath::pmax(du[k], dv[k]));
                if (siz < 1) siz = 1;
                l = (float)gomath::go_log2((double)siz);
            }
        }
        const RGBA c = texture_query(t, l, u[k], v[k]);
        std::memcpy(out + 4 * k, c.data(), 4);
    }
    return PR_OK;
}

// imageutil.Resize of a dx x dy RGBA image (rows top-down) to w x h.
int orc_resize(const uint8_t* img, int dx, int dy, int w, int h, uint8_t* out) {
    if (!img || !out || dx <= 0 || dy <= 0 || w <= 0 || h <= 0) return PR_ERR_INVALID_ARG;
    if (dx == w && dy == h) {
        std::memcpy(out, img, (size_t)dx * dy * 4);
        return PR_OK;
    }
    resize_image(img, dx, dy, w, h, out);
    return PR_OK;
}

int orc_render(const pr_scene_desc* sc, const pr_frame_desc* fr, float* shadow_state, int threads,
               pr_outputs* out, orc_stats* st) {
    if (!sc || !fr || fr->width <= 0 || fr->height <= 0) return PR_ERR_INVALID_ARG;
    Ctx c;
    c.sc = sc;
    c.fr = fr;
    c.M = (fr->size >= offsetof(pr_frame_desc, msaa) + sizeof(int32_t) && fr->msaa > 1) ? fr->msaa : 1;
    // the materials' image textures (NewTexture once per render here)
    std::vector<OTex> textures;
    std::vector<const OTex*> mat_tex(sc->n_materials, nullptr);
    const pr_texture* stex = sc->size >= offsetof(pr_scene_desc, textures) + sizeof(void*) ? sc->textures : nullptr;
    if (stex) {
        textures.reserve(sc->n_materials);
        for (uint32_t m = 0; m < sc->n_materials; m++) {
            if (!stex[m].rgba) continue;
            OImg img;
            img.w = stex[m].width;
            img.h = stex[m].height;
            img.pix.assign(stex[m].rgba, stex[m].rgba + (size_t)img.w * img.h * 4);
            textures.push_back(new_texture(img, (sc->materials[m].flags & PR_MAT_MIPMAP) != 0));
            mat_tex[m] = &textures.back();
        }
        c.mat_tex = &mat_tex;
    }
    c.W = fr->width * c.M;
    c.H = fr->height * c.M;
    c.SW = fr->shadow_width > 0 ? fr->shadow_width : c.W;
    c.SH = fr->shadow_height > 0 ? fr->shadow_height : c.H;
    c.perspect = (fr->flags & PR_FRAME_PERSPECTIVE) != 0;
    if (st) std::memset(st, 0, sizeof(*st));
    std::vector<Frag> frags((size_t)c.W * c.H);
    for (auto& f : frags) {
        std::memset(&f, 0, sizeof(f));
        f.tri = PR_TRI_NONE;
    }
    FB fb;
    fb.W = c.W;
    fb.H = c.H;
    fb.f = frags.data();
    fb.y0 = 0;
    fb.y1 = c.H;
    c.fb = &fb;
    if (threads < 1) threads = 1;

    size_t plane = (size_t)c.SW * c.SH;
    std::vector<float> sdepth(plane * fr->n_lights, 0.0f);
    if (shadow_state) std::memcpy(sdepth.data(), shadow_state, sdepth.size() * sizeof(float));

    // passShadows (render/raster.go:176-184)
    if (fr->flags & PR_FRAME_SHADOWMAP) {
        for (uint32_t i = 0; i < fr->n_lights; i++) {
            if (!fr->lights[i].cast_shadow) continue;
            int rc = PR_OK;
            float* d = sdepth.data() + plane * i;
            parallel_rows(threads, c.SH, [&](int y0, int y1) {
                int r = shadow_pass(c, (int)i, d, y0, y1);
                if (r != PR_OK) rc = r;
            });
            if (rc != PR_OK) return rc;
        }
    }

    // passForward: band workers share the fragment storage, each owning rows
    // [y0, y1); every band walks all triangles in submission order.
    int rc = PR_OK;
    {
        int per = (c.H + threads - 1) / threads;
        std::vector<int> rcs(threads, PR_OK);
        std::vector<orc_stats> sts(threads);
        std::vector<std::thread> ts;
        auto band = [&](int i, int y0, int y1) {
            Ctx ci = c;
            FB view = fb;
            view.y0 = y0;
            view.y1 = y1;
            ci.fb = &view;
            std::memset(&sts[i], 0, sizeof(orc_stats));
            rcs[i] = forward_pass(ci, &sts[i]);
        };
        for (int i = 0; i < threads; i++) {
            int y0 = i * per, y1 = std::min(c.H, (i + 1) * per);
            if (y0 >= y1) break;
            if (threads == 1)
                band(i, y0, y1);
            else
                ts.emplace_back(band, i, y0, y1);
        }
        for (auto& t : ts) t.join();
        for (int i = 0; i < threads; i++)
            if (rcs[i] != PR_OK) rc = rcs[i];
        if (st) st->n_clipped = sts[0].n_clipped;
    }
    if (rc != PR_OK) return rc;

    // passDeferred + passAntialiasing
    ShadeUniforms u;
    u.viewport = viewport((float)c.W, (float)c.H);
    M4 viewInv, projInv, vpInv;
    if (!inv(loadm(fr->view), &viewInv) || !inv(loadm(fr->proj), &projInv) || !inv(u.viewport, &vpInv))
        return PR_ERR_SINGULAR;
    u.s2w = mulm(mulm(viewInv, projInv), vpInv);
    u.shadow_vp = viewport((float)c.SW, (float)c.SH);
    for (uint32_t i = 0; i < fr->n_lights; i++) {
        u.lview.push_back(loadm(fr->lights[i].shadow_view));
        u.lproj.push_back(loadm(fr->lights[i].shadow_proj));
    }
    orc_ao_directions(u.ao_cos, u.ao_sin, &u.n_ao_dirs);
    std::vector<uint8_t> color((size_t)c.W * c.H * 4);
    const SRGB& s = srgb();
    bool gamma = (fr->flags & PR_FRAME_GAMMA) != 0;
    parallel_rows(threads, c.H, [&](int r0, int r1) {
        for (int r = r0; r < r1; r++) {
            int64_t y = c.H - 1 - r;
            for (int x = 0; x < c.W; x++) {
                uint8_t px[4];
                shade_pixel(c, u, sdepth, x, y, px);
                if (gamma)
                    for (int k = 0; k < 3; k++) px[k] = s.table[px[k]];
                std::memcpy(&color[((size_t)r * c.W + x) * 4], px, 4);
            }
        }
    });

    if (shadow_state) std::memcpy(shadow_state, sdepth.data(), sdepth.size() * sizeof(float));
    if (out) {
        size_t n = (size_t)c.W * c.H;
        if (out->rgba) {
            if (c.M > 1)
                resize_image(color.data(), c.W, c.H, fr->width, fr->height, out->rgba);
            else
                std::memcpy(out->rgba, color.data(), n * 4);
        }
        for (size_t i = 0; i < n; i++) {
            const Frag& f = frags[i];
            if (out->tri_id) out->tri_id[i] = f.ok ? f.tri : PR_TRI_NONE;
            if (out->depth) out->depth[i] = f.ok ? f.depth : 0.0f;
            if (out->nor) std::memcpy(out->nor + i * 4, &f.nor, 16);
            if (out->face_nor) std::memcpy(out->face_nor + i * 4, &f.fnor, 16);
            if (out->world_pos) std::memcpy(out->world_pos + i * 4, &f.wpos, 16);
            if (out->uvd) {
                float q[4] = {f.u, f.v, f.du, f.dv};
                std::memcpy(out->uvd + i * 4, q, 16);
            }
            if (out->vcol) std::memcpy(out->vcol + i * 4, f.col, 4);
            if (out->mat_id) out->mat_id[i] = f.ok ? (int32_t)f.matid : -1;
        }
        if (out->shadow_maps) std::memcpy(out->shadow_maps, sdepth.data(), sdepth.size() * sizeof(float));
    }
    return PR_OK;
}

}  // extern "C"
