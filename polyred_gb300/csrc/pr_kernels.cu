// pr_kernels.cu — the GB300 (sm_103a) render path kernels.
//
// Frame = [shadow setup + raster per casting light] -> main setup -> raster
//         -> (NaN fix-up) -> resolve -> shade (attributes, Blinn-Phong,
//         shadow lookups, AO, gamma, RGBA8 pack).
//
// Visibility is order independent: each fragment issues a 64-bit atomicMax of
// (orderable depth << 32 | ~seq), which leaves at every pixel the first
// fragment (in the reference's single-worker draw order) with the greatest
// depth — exactly what buffer.FragmentBuffer's sequential DepthTest/Set
// (buffer/buffer.go:221-280) keeps. A NaN-depth fragment only wins when it is
// the first fragment of its pixel; a rare fix-up pass settles that.
//
// Compiled with -fmad=false -prec-div=true -prec-sqrt=true -ftz=false.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "pr_devmath.cuh"
#include "pr_hostmath.h"
#include "pr_kernels.cuh"

using namespace prd;

namespace prk {
namespace {

constexpr float kEps = 1e-7f;  // math.Epsilon as float32 (math/math.go:31)

PR_DEV V4 ld4(const float4 q) { return {q.x, q.y, q.z, q.w}; }

// Mat4.MulM (math/mat4.go:201-220), plain float32 sums left to right.
PR_DEV void mulm(const float* m, const float* n, float* r) {
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            r[i * 4 + j] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[i * 4 + 0], n[0 * 4 + j]), __fmul_rn(m[i * 4 + 1], n[1 * 4 + j])),
                                               __fmul_rn(m[i * 4 + 2], n[2 * 4 + j])),
                                     __fmul_rn(m[i * 4 + 3], n[3 * 4 + j]));
}

PR_DEV bool approx_eq(float a, float b) { return fabsf(__fsub_rn(a, b)) <= kEps; }
PR_DEV bool approx_less(float a, float b) { return a < b && fabsf(__fsub_rn(a, b)) > kEps; }
PR_DEV bool le_approx(float a, float b) { return approx_eq(a, b) || approx_less(a, b); }

// Triangle.IsValid (geometry/primitive/triangle.go:63-80)
PR_DEV bool tri_is_valid(V4 p1, V4 p2, V4 p3) {
    V4 a = sub4(p2, p1), b = sub4(p3, p1);
    if (approx_eq(a.x, 0) && approx_eq(a.y, 0) && approx_eq(a.z, 0)) return false;
    if (approx_eq(b.x, 0) && approx_eq(b.y, 0) && approx_eq(b.z, 0)) return false;
    float d = __fdiv_rn(dot4(a, b), __fmul_rn(len4(a), len4(b)));
    return !approx_eq(d, 1.0f) && !approx_eq(d, -1.0f);
}

struct Box { float mnx, mny, mnz, mxx, mxy, mxz; };
// NewAABB over three points (geometry/primitive/box.go:15-27)
PR_DEV Box box3(V4 a, V4 b, V4 c) {
    Box r;
    r.mnx = pmin(pmin(pmin(3.40282347e38f, a.x), b.x), c.x);
    r.mny = pmin(pmin(pmin(3.40282347e38f, a.y), b.y), c.y);
    r.mnz = pmin(pmin(pmin(3.40282347e38f, a.z), b.z), c.z);
    r.mxx = pmax(pmax(pmax(-3.40282347e38f, a.x), b.x), c.x);
    r.mxy = pmax(pmax(pmax(-3.40282347e38f, a.y), b.y), c.y);
    r.mxz = pmax(pmax(pmax(-3.40282347e38f, a.z), b.z), c.z);
    return r;
}
// AABB.Intersect with the reference's maxZ := Min(aabb.Max.Y, aabb2.Max.Z)
// (geometry/primitive/box.go:32-41); `a` is the viewport box.
PR_DEV bool box_intersect(const Box& a, const Box& b) {
    float minX = pmax(a.mnx, b.mnx), minY = pmax(a.mny, b.mny), minZ = pmax(a.mnz, b.mnz);
    float maxX = pmin(a.mxx, b.mxx), maxY = pmin(a.mxy, b.mxy), maxZ = pmin(a.mxy, b.mxz);
    return minX <= maxX && minY <= maxY && minZ <= maxZ;
}
PR_DEV bool box_contains(const Box& a, V4 v) {
    return le_approx(a.mnx, v.x) && le_approx(a.mny, v.y) && le_approx(a.mnz, v.z) && le_approx(v.x, a.mxx) &&
           le_approx(v.y, a.mxy) && le_approx(v.z, a.mxz);
}

// Pixel rectangle of drawClipped / drawDepth (render/raster.go:473-477),
// clamped to the W x H buffer. Returns false when empty.
// The viewport box and clip extent of a pass: float32(MSAA * size), the
// reference's MSAA*buf.Bounds().Dx() with the buffer already n times the
// image (render/raster.go:414-441, render/cull.go:15-23). Pixel boxes stay
// clamped to the target (buf.In).
PR_DEV float ext_w(const SetupParams& P) { return (float)(P.msaa > 1 ? P.W * P.msaa : P.W); }
PR_DEV float ext_h(const SetupParams& P) { return (float)(P.msaa > 1 ? P.H * P.msaa : P.H); }

// The pixels of the reference's box that the inside test can accept: those
// whose centre lies within a margin m of the triangle's bounding box; every
// other pixel fails drawClipped's test bc >= -Epsilon (render/raster.go:491)
// for certain, so leaving it out changes no fragment.
//
// Why. Let S_j (j = 0..2) be the exact cross products of the exact vertex
// differences with the pixel centre p, S their sum (the exact Sabc), bc_j =
// S_j / S. If p.x >= max_x + m, then p.x - max_x = sum_j bc_j (x_j - max_x)
// <= N w_x with N the sum of the negative bc_j and w_x the box width, so
// some bc_j <= -m / (2 w_x) (at most two are negative): |S_j| >=
// m |S| / (2 w_x), opposite in sign to S (the same for the other sides and
// for y). The test's float32 values: each cross product is formed from
// rounded differences (relative error u = 2^-24 each) as fma64f(vx, wy,
// -RN(vy wx)), within 3u (|vx wy| + |vy wx|) of its rounded-input value, so
// within dS = 6u E U of the exact one, E = w_x + w_y bounding every edge's
// L1 length and U = E + 4 every |p - vertex|_1 over the box (the reference
// box lies within the bounding box padded by 1.5 px); Sabc within dA = 6u E^2.
// When L = |Sabc| - dA > 2 dA, the signs hold and the computed b_j =
// RN(S_j' / Sabc') <= -(|S_j| - dS) / (|S| + dA) (1 - u) < -Epsilon as soon
// as |S_j| - dS >= 2e-7 (|Sabc| + 2 dA), which m_x = 2 w_x (dS + 2.1e-7
// (|Sabc| + 2 dA)) / L guarantees. All in upward rounding; degenerate,
// near-degenerate and non-finite triangles keep the reference box (their
// NaN and infinite barycentrics can pass the test anywhere in it).
PR_DEV void tighten_box(V4 a, V4 b, V4 c, float sabc, long long& x0, long long& x1, long long& y0, long long& y1) {
    const float mnx = fminf(fminf(a.x, b.x), c.x), mxx = fmaxf(fmaxf(a.x, b.x), c.x);
    const float mny = fminf(fminf(a.y, b.y), c.y), mxy = fmaxf(fmaxf(a.y, b.y), c.y);
    if (!(isfinite(mnx) && isfinite(mxx) && isfinite(mny) && isfinite(mxy) && isfinite(sabc))) return;
    const float wx = __fsub_ru(mxx, mnx), wy = __fsub_ru(mxy, mny);
    const float E = __fadd_ru(wx, wy), U = __fadd_ru(E, 4.0f);
    const float k6u = 3.6e-7f;  // >= 6 * 2^-24
    const float dS = __fmul_ru(__fmul_ru(k6u, E), U), dA = __fmul_ru(__fmul_ru(k6u, E), E);
    const float as = fabsf(sabc);
    const float L = __fsub_rd(as, dA);
    if (!(L > __fmul_ru(2.0f, dA)) || !(L > 0.0f)) return;
    const float q = __fdiv_ru(__fadd_ru(dS, __fmul_ru(2.1e-7f, __fadd_ru(as, __fmul_ru(2.0f, dA)))), L);
    const float mx = __fmul_ru(__fmul_ru(2.0f, wx), q), my = __fmul_ru(__fmul_ru(2.0f, wy), q);
    // centres x + 0.5 in [mnx - mx, mxx + mx], rounded outward
    const float lx = ceilf(__fsub_rd(__fsub_rd(mnx, mx), 0.5f)), hx = floorf(__fsub_ru(__fadd_ru(mxx, mx), 0.5f));
    const float ly = ceilf(__fsub_rd(__fsub_rd(mny, my), 0.5f)), hy = floorf(__fsub_ru(__fadd_ru(mxy, my), 0.5f));
    if (!(lx <= hx && ly <= hy)) {  // no pixel centre can pass
        x0 = 1;
        x1 = 0;
        return;
    }
    // within the reference box (|coordinates| < 2^16 there): float compares, then exact conversions
    if (lx > (float)x0) x0 = (long long)lx;
    if (hx < (float)x1) x1 = (long long)hx;
    if (ly > (float)y0) y0 = (long long)ly;
    if (hy < (float)y1) y1 = (long long)hy;
}

// The reference's pixel box (rounded bounding box padded by one, clamped
// to the target), narrowed by tighten_box; false: no pixel to test.
PR_DEV bool pixel_box(V4 a, V4 b, V4 c, float sabc, int W, int H, uint32_t* bx, uint32_t* by, uint32_t* area) {
    Box r = box3(a, b, c);
    long long xmin = go_f2i(__fsub_rn(pround(r.mnx), 1.0f));
    long long xmax = go_f2i(__fadd_rn(pround(r.mxx), 1.0f));
    long long ymin = go_f2i(__fsub_rn(pround(r.mny), 1.0f));
    long long ymax = go_f2i(__fadd_rn(pround(r.mxy), 1.0f));
    long long x0 = xmin < 0 ? 0 : xmin, x1 = xmax > W - 1 ? W - 1 : xmax;
    long long y0 = ymin < 0 ? 0 : ymin, y1 = ymax > H - 1 ? H - 1 : ymax;
    if (x0 > x1 || y0 > y1) return false;
    tighten_box(a, b, c, sabc, x0, x1, y0, y1);
    if (x0 > x1 || y0 > y1) return false;
    *bx = (uint32_t)x0 | ((uint32_t)x1 << 16);
    *by = (uint32_t)y0 | ((uint32_t)y1 << 16);
    *area = (uint32_t)((x1 - x0 + 1) * (y1 - y0 + 1));
    return true;
}

PR_DEV uint32_t find_object(const uint32_t* first, uint32_t n_obj, uint32_t t) {
    uint32_t lo = 0, hi = n_obj - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (first[mid] <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

PR_DEV uint32_t pack_col(uchar4 c) { return (uint32_t)c.x | ((uint32_t)c.y << 8) | ((uint32_t)c.z << 16) | ((uint32_t)c.w << 24); }
PR_DEV float col_ch(uint32_t c, int k) { return small_u2f((c >> (8 * k)) & 0xffu); }

struct SubVtx {
    V4 pos;
    V4 nor;
    float u, v;
    uint32_t col;
};

// clipTriangle's re-interpolated vertex (render/clipping.go:75-102)
PR_DEV SubVtx clip_vertex(V4 cp, const SubVtx* t, float psabc) {
    float b[3];
    barycoord_s(cp.x, cp.y, t[0].pos.x, t[0].pos.y, t[1].pos.x, t[1].pos.y, t[2].pos.x, t[2].pos.y, psabc, b);
    SubVtx r;
    auto lerp3 = [&](float a0, float a1, float a2) {
        return __fadd_rn(__fadd_rn(__fmul_rn(b[0], a0), __fmul_rn(b[1], a1)), __fmul_rn(b[2], a2));
    };
    r.pos = {lerp3(t[0].pos.x, t[1].pos.x, t[2].pos.x), lerp3(t[0].pos.y, t[1].pos.y, t[2].pos.y),
             lerp3(t[0].pos.z, t[1].pos.z, t[2].pos.z), 1.0f};
    r.u = lerp3(t[0].u, t[1].u, t[2].u);
    r.v = lerp3(t[0].v, t[1].v, t[2].v);
    r.nor = {lerp3(t[0].nor.x, t[1].nor.x, t[2].nor.x), lerp3(t[0].nor.y, t[1].nor.y, t[2].nor.y),
             lerp3(t[0].nor.z, t[1].nor.z, t[2].nor.z), 0.0f};
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float s = lerp3(col_ch(t[0].col, k), col_ch(t[1].col, k), col_ch(t[2].col, k));
        c |= go_f2u8(pclamp(s, 0.0f, 255.0f)) << (8 * k);
    }
    r.col = c;
    return r;
}

// plane.intersectSegment(v0, v1) (render/clipping.go:23-30)
PR_DEV V4 intersect_segment(V4 P, V4 N, V4 v0, V4 v1) {
    V4 u = sub4(v1, v0);
    V4 w = sub4(v0, P);
    float d = dot4(N, u);
    float nn = -dot4(N, w);
    float sc = __fdiv_rn(nn, d);
    return add4(v0, V4{__fmul_rn(u.x, sc), __fmul_rn(u.y, sc), __fmul_rn(u.z, sc), __fmul_rn(u.w, sc)});
}

// Sutherland-Hodgman against the six screen-space planes
// (render/clipping.go:31-68). Returns the vertex count (<= 9), or -1 when a
// polygon with NaN coordinates outgrows that bound.
PR_DEV int sutherland_hodgman(const V4* in3, float w, float h, V4* out) {
    V4 buf[2][10];
    int n = 3;
    for (int i = 0; i < 3; i++) buf[0][i] = in3[i];
    int cur = 0;
    const float pp[6][4] = {{w, 0, 0, 1}, {0, 0, 0, 1}, {0, h, 0, 1}, {0, 0, 0, 1}, {0, 0, 1, 1}, {0, 0, -1, 1}};
    const float pn[6][4] = {{-1, 0, 0, 1}, {1, 0, 0, 1}, {0, -1, 0, 1}, {0, 1, 0, 1}, {0, 0, -1, 1}, {0, 0, 1, 1}};
    for (int pl = 0; pl < 6; pl++) {
        if (n == 0) return 0;
        V4 P = {pp[pl][0], pp[pl][1], pp[pl][2], pp[pl][3]};
        V4 N = {pn[pl][0], pn[pl][1], pn[pl][2], pn[pl][3]};
        const V4* inp = buf[cur];
        V4* o = buf[cur ^ 1];
        int m = 0;
        V4 s = inp[n - 1];
        bool fs = dot4(sub4(s, P), N) > 0.0f;  // plane.pointInFront
        for (int i = 0; i < n; i++) {
            V4 e = inp[i];
            const bool fe = dot4(sub4(e, P), N) > 0.0f;
            // A convex polygon gains at most one vertex per plane (<= 9 in
            // all); more means NaN coordinates broke convexity.
            if (m + (fe && !fs ? 2 : 1) > 9) return -1;
            if (fe) {
                if (!fs) o[m++] = intersect_segment(P, N, s, e);
                o[m++] = e;
            } else if (fs) {
                o[m++] = intersect_segment(P, N, s, e);
            }
            s = e;
            fs = fe;  // the same test of the same vertex
        }
        n = m;
        cur ^= 1;
    }
    for (int i = 0; i < n; i++) out[i] = buf[cur][i];
    return n;
}

// sutherland_hodgman over a group of kClipLanes (16) lanes, lane i holding
// polygon vertex i (n <= 9 between planes). For each plane every lane
// tests the edge from the previous vertex to its own, exactly as the loop
// above does at step i, and places its 0, 1 or 2 output vertices at the
// exclusive prefix sum of the counts, so each output polygon is the loop's,
// vertex for vertex; the loop's overflow check at step i sees the same
// prefix count. All 32 lanes of the warp call; a lane outside [0, n) holds
// nothing. Returns the vertex count (or -1) to every lane of the group, and
// lane i < count gets vertex i in *v. ring: the group's 2 x 10 vertices of
// shared scratch.
constexpr int kClipLanes = 16;  // >= 9 polygon vertices
PR_DEV int sutherland_hodgman_group(V4* v, int n, float w, float h, uint32_t sub, V4 (*ring)[10]) {
    const unsigned full = 0xffffffffu;
    const uint32_t gbase = (threadIdx.x & 31u) & ~(uint32_t)(kClipLanes - 1);
    const float pp[6][4] = {{w, 0, 0, 1}, {0, 0, 0, 1}, {0, h, 0, 1}, {0, 0, 0, 1}, {0, 0, 1, 1}, {0, 0, -1, 1}};
    const float pn[6][4] = {{-1, 0, 0, 1}, {1, 0, 0, 1}, {0, -1, 0, 1}, {0, 1, 0, 1}, {0, 0, -1, 1}, {0, 0, 1, 1}};
    int res = n;
    for (int pl = 0; pl < 6; pl++) {
        const V4 P = {pp[pl][0], pp[pl][1], pp[pl][2], pp[pl][3]};
        const V4 N = {pn[pl][0], pn[pl][1], pn[pl][2], pn[pl][3]};
        const bool act = (int)sub < n;  // n == 0 (an empty polygon, or a finished group): no lane acts
        const V4 e = *v;
        const bool fe = act && dot4(sub4(e, P), N) > 0.0f;
        const int src = sub == 0u ? n - 1 : (int)sub - 1;  // the previous vertex (the last one for vertex 0)
        V4 sv;
        sv.x = __shfl_sync(full, e.x, src < 0 ? 0 : src, kClipLanes);
        sv.y = __shfl_sync(full, e.y, src < 0 ? 0 : src, kClipLanes);
        sv.z = __shfl_sync(full, e.z, src < 0 ? 0 : src, kClipLanes);
        sv.w = __shfl_sync(full, e.w, src < 0 ? 0 : src, kClipLanes);
        const bool fs = __shfl_sync(full, (int)fe, src < 0 ? 0 : src, kClipLanes) != 0;
        const int cnt = !act ? 0 : fe ? (fs ? 1 : 2) : (fs ? 1 : 0);
        int incl = cnt;
#pragma unroll
        for (int d = 1; d < kClipLanes; d <<= 1) {
            const int t = __shfl_up_sync(full, incl, d, kClipLanes);
            if ((int)sub >= d) incl += t;
        }
        const int m = incl - cnt;  // the loop's m at this step
        const int total = __shfl_sync(full, incl, kClipLanes - 1, kClipLanes);
        const bool over = act && m + (fe && !fs ? 2 : 1) > 9;
        const bool any_over = ((__ballot_sync(full, over) >> gbase) & ((1u << kClipLanes) - 1u)) != 0u;
        V4* o = ring[pl & 1];
        if (act && !any_over) {
            if (fe) {
                if (!fs) o[m] = intersect_segment(P, N, sv, e);
                o[m + (fs ? 0 : 1)] = e;
            } else if (fs) {
                o[m] = intersect_segment(P, N, sv, e);
            }
        }
        __syncwarp();
        if (n > 0) res = any_over ? -1 : total;
        n = (n > 0 && !any_over) ? total : 0;
        if ((int)sub < n) *v = o[sub];  // ring[pl & 1] is next written two planes on, after a sync
    }
    return res;
}

// Vec4.Apply kept out of line in the per-triangle setup kernels: a dozen
// inlined copies of twelve emulated float64 FMAs each overflow the
// instruction cache (no_instruction stalls dominated), one shared copy
// does not.
__device__ __noinline__ V4 apply4_outline(V4 v, const float* m) { return apply4(v, m); }

// A screen-space vertex back in world space (render/raster.go:467-469).
PR_DEV V4 world_of(const SetupParams& P, V4 pos) {
    return apply4_outline(apply4_outline(apply4_outline(pos, P.viewport_inv), P.proj_inv), P.view_inv);
}

// The attribute record of record ridx (drawClipped's per-vertex inputs).
// mw: the vertices' world positions when the caller has them (the chain
// below of each vertex's screen position), else null.
PR_DEV void write_attr(const SetupParams& P, uint32_t ridx, const SubVtx* v, const float* recipw, int matid,
                       const V4* mw) {
    AttrRec A;
    V4 m[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        A.recipw[k] = recipw[k];
        A.nor[k * 3 + 0] = v[k].nor.x;
        A.nor[k * 3 + 1] = v[k].nor.y;
        A.nor[k * 3 + 2] = v[k].nor.z;
        A.uv[k * 2 + 0] = v[k].u;
        A.uv[k * 2 + 1] = v[k].v;
        A.col[k] = v[k].col;
        // render/raster.go:467-469
        m[k] = mw ? mw[k] : world_of(P, v[k].pos);
        A.m[k * 3 + 0] = m[k].x;
        A.m[k * 3 + 1] = m[k].y;
        A.m[k * 3 + 2] = m[k].z;
    }
    V4 fn = unit4(cross4(sub4(m[1], m[0]), sub4(m[2], m[0])));  // render/raster.go:479
    A.fn[0] = fn.x; A.fn[1] = fn.y; A.fn[2] = fn.z; A.fn[3] = fn.w;
    A.matid = matid;
    const float4* as = reinterpret_cast<const float4*>(&A);
    float4* ad = reinterpret_cast<float4*>(P.arec + ridx);
#pragma unroll
    for (int k = 0; k < 9; k++) ad[k] = as[k];
}

// Build and store the records of one sub-triangle; returns its pixel area
// (0 = nothing to raster, and then nothing is stored) and writes its bbox
// words. With P.defer_attr the
// attribute record is left to attr_kernel, which writes it only for records
// that win a pixel.
PR_DEV uint32_t write_sub(const SetupParams& P, uint32_t ridx, uint32_t seq, const SubVtx* v, const float* recipw,
                          int matid, const V4* mw = nullptr) {
    RasterRec R;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        R.v[3 * k + 0] = v[k].pos.x;
        R.v[3 * k + 1] = v[k].pos.y;
        R.v[3 * k + 2] = v[k].pos.z;
        R.recipw[k] = recipw ? recipw[k] : 0.0f;
    }
    R.sabc = sabc_of(R.v[0], R.v[1], R.v[3], R.v[4], R.v[6], R.v[7]);
    R.seq = seq;
    uint32_t area = 0;
    // no pixel to test: no task will name the record, no pixel can pick it
    // as its winner, so nothing reads it
    if (!pixel_box(v[0].pos, v[1].pos, v[2].pos, R.sabc, P.W, P.H, &R.bx, &R.by, &area)) return 0;
    const float4* rs = reinterpret_cast<const float4*>(&R);
    float4* rd = reinterpret_cast<float4*>(P.rrec + ridx);
#pragma unroll
    for (int k = 0; k < 4; k++) rd[k] = rs[k];
    if (P.attr_state) P.attr_state[ridx] = P.defer_attr ? 1u : 0u;
    if (P.arec && !P.defer_attr) write_attr(P, ridx, v, recipw, matid, mw);
    return area;
}

// Vec4.Apply(ViewportMatrix) for a matrix of ViewportMatrix's pattern
// [sx 0 0 tx; 0 sy 0 ty; 0 0 1 0; 0 0 0 1] (P.vp_std). A zero first factor,
// or a factor 1 with a +-0 addend, rounds exactly in float64 and float32
// alike, so only the sx and sy terms need the float64-FMA emulation; the
// matrix's own entries stay in every term (signs of zero included).
__device__ __noinline__ V4 apply_viewport_exact(V4 v, const float* m) { return apply4(v, m); }
PR_DEV V4 apply_viewport(V4 v, const float* m) {
    bool bad = false;
    const V4 r = {fma64f_try(m[0], v.x, __fmaf_rn(m[1], v.y, __fmaf_rn(m[2], v.z, __fmul_rn(m[3], v.w))), bad),
                  __fmaf_rn(m[4], v.x, fma64f_try(m[5], v.y, __fmaf_rn(m[6], v.z, __fmul_rn(m[7], v.w)), bad)),
                  __fmaf_rn(m[8], v.x, __fmaf_rn(m[9], v.y, __fmaf_rn(m[10], v.z, __fmul_rn(m[11], v.w)))),
                  __fmaf_rn(m[12], v.x, __fmaf_rn(m[13], v.y, __fmaf_rn(m[14], v.z, __fmul_rn(m[15], v.w))))};
    return __builtin_expect(bad, 0) ? apply_viewport_exact(v, m) : r;
}
PR_DEV V4 viewport_apply(const SetupParams& P, V4 v) {
    return P.vp_std ? apply_viewport(v, P.viewport) : apply4_outline(v, P.viewport);
}

// ---- warp-aggregated reservations (all 32 lanes must call them) ----------

PR_DEV uint32_t lane_id() { return threadIdx.x & 31u; }

// Reserve n slots per lane from *counter with one atomic per warp; returns
// this lane's first slot. Sets *total to the warp's total.
PR_DEV uint32_t warp_reserve(uint32_t* counter, uint32_t n, uint32_t* total) {
    const uint32_t lane = lane_id();
    uint32_t incl = n;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (uint32_t)d) incl += v;
    }
    const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
    *total = tot;
    uint32_t base = 0;
    if (tot != 0 && lane == 31) base = atomicAdd(counter, tot);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + incl - n;
}

PR_DEV uint32_t n_tasks_of(uint32_t area, uint32_t shift) { return (area + (1u << shift) - 1u) >> shift; }

// Write the raster tasks of up to 8 records (areas given); all lanes call.
// A lane with one record of more than kWarpEmit tasks (a large triangle:
// thousands of tasks for a ground plane) leaves their writing to the whole
// warp, which would otherwise wait on that lane's serial stores.
constexpr uint32_t kWarpEmit = 8;
PR_DEV void emit_tasks_warp(const SetupParams& P, const uint32_t* ridx, const uint32_t* area, int n) {
    uint32_t mine = 0;
    for (int i = 0; i < n; i++) mine += n_tasks_of(area[i], P.task_shift);
    uint32_t tot;
    uint32_t o = warp_reserve(&P.cnt->n_tasks, mine, &tot);
    if (tot == 0) return;  // warp-uniform
    const bool fits = o + mine <= P.cap_tasks;
    if (mine != 0 && !fits) {
        atomicOr(&P.cnt->overflow, 2u);
        atomicMax(&P.cnt->need_tasks, o + mine);
    }
    const bool shared = fits && n == 1 && mine > kWarpEmit;
    if (fits && !shared) {
        for (int i = 0; i < n; i++) {
            uint32_t nt = n_tasks_of(area[i], P.task_shift);
            for (uint32_t c = 0; c < nt; c++) P.tasks[o++] = make_uint2(ridx[i], c);
        }
    }
    const uint32_t r0 = n > 0 ? ridx[0] : 0u;
    for (unsigned big = __ballot_sync(0xffffffffu, shared); big; big &= big - 1u) {
        const int l = __ffs(big) - 1;
        const uint32_t lo = __shfl_sync(0xffffffffu, o, l), ln = __shfl_sync(0xffffffffu, mine, l);
        const uint32_t lr = __shfl_sync(0xffffffffu, r0, l);
        for (uint32_t c = lane_id(); c < ln; c += 32u) P.tasks[lo + c] = make_uint2(lr, c);
    }
}

// draw's transform and culls for triangle t (render/raster.go:380-436):
// Proj.MulM(View).MulM(Model).MulV, -1/W, Viewport Apply + Pos, back-face,
// viewport AABB; then the per-vertex attributes of surviving triangles
// (the normal matrix Apply does not influence the culls).
// The objects of one setup block's triangles (usually one) and their
// Proj·View·Model, computed once per block in the order of Mat4.MulM.
constexpr int kBlkObj = 8;
struct ObjCache {
    uint32_t o0, n;  // first object; n > kBlkObj: not cached
    uint32_t first[kBlkObj + 1];
    float trans[kBlkObj][16];
};

// Block-wide (every thread calls): triangles [t0, t0 + blockDim.x).
PR_DEV void obj_cache_fill(const SetupParams& P, uint32_t t0, ObjCache& C) {
    if (threadIdx.x == 0) {
        const uint32_t t1 = min(t0 + blockDim.x, P.n_tris) - 1u;
        const uint32_t o0 = find_object(P.obj_first, P.n_objects, t0);
        C.o0 = o0;
        C.n = find_object(P.obj_first, P.n_objects, t1) - o0 + 1u;
    }
    __syncthreads();
    const uint32_t n = C.n, o0 = C.o0;
    if (n <= (uint32_t)kBlkObj) {
        for (uint32_t e = threadIdx.x; e < n * 16u; e += blockDim.x) {
            const uint32_t k = e >> 4, i = (e >> 2) & 3u, j = e & 3u;
            const float* m = P.pv + i * 4;
            const float* q = P.obj_model + (size_t)(o0 + k) * 16;
            C.trans[k][e & 15u] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], q[j]), __fmul_rn(m[1], q[4 + j])),
                                                      __fmul_rn(m[2], q[8 + j])),
                                           __fmul_rn(m[3], q[12 + j]));
        }
        for (uint32_t e = threadIdx.x; e <= n; e += blockDim.x) C.first[e] = P.obj_first[o0 + e];
    }
    __syncthreads();
}

// Object of triangle t and its Proj·View·Model: from the pass's table (the
// block's first object, then the few objects that start inside the block),
// else from the block cache when it holds t's block.
PR_DEV uint32_t object_trans(const SetupParams& P, const ObjCache* C, uint32_t t, float* trans) {
    if (P.obj_trans) {
        uint32_t o = P.blk_obj[t >> 7];
        while (o + 1 < P.n_objects && P.obj_first[o + 1] <= t) o++;
        const float4* q = reinterpret_cast<const float4*>(P.obj_trans + (size_t)o * 16);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float4 r = __ldg(q + e);
            trans[4 * e] = r.x;
            trans[4 * e + 1] = r.y;
            trans[4 * e + 2] = r.z;
            trans[4 * e + 3] = r.w;
        }
        return o;
    }
    if (C && C->n <= (uint32_t)kBlkObj) {
        uint32_t k = 0;
        while (k + 1 < C->n && C->first[k + 1] <= t) k++;
#pragma unroll
        for (int e = 0; e < 16; e++) trans[e] = C->trans[k][e];
        return C->o0 + k;
    }
    const uint32_t o = find_object(P.obj_first, P.n_objects, t);
    mulm(P.pv, P.obj_model + o * 16, trans);
    return o;
}

// Triangle.IsValid of triangle t (from the flags the scene upload computed).
PR_DEV bool tri_valid_of(const SetupParams& P, uint32_t t, const V4* p) {
    if (P.tri_flags) return (P.tri_flags[t] & kTriValid) != 0;
    return tri_is_valid(p[0], p[1], p[2]);
}

// The transform and the culls of transform_main (screen positions, -1/W,
// the object); false when a cull drops the triangle.
PR_DEV bool transform_main_geom(const SetupParams& P, const ObjCache* C, uint32_t t, SubVtx* v, float* recipw,
                                uint32_t* obj, bool* contained) {
    V4 p[3];
#pragma unroll
    for (int k = 0; k < 3; k++) p[k] = ld4(P.pos[t * 3 + k]);
    if (!tri_valid_of(P, t, p)) return false;
    float trans[16];
    const uint32_t o = object_trans(P, C, t, trans);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const V4 cp = mulv(trans, p[k]);
        recipw[k] = P.perspective ? __fdiv_rn(-1.0f, cp.w) : 1.0f;
        v[k].pos = pos4(viewport_apply(P, cp));
    }
    // cullBackFace (render/cull.go:26-28)
    if (cross_z(__fsub_rn(v[1].pos.x, v[0].pos.x), __fsub_rn(v[1].pos.y, v[0].pos.y), __fsub_rn(v[2].pos.x, v[0].pos.x),
                __fsub_rn(v[2].pos.y, v[0].pos.y)) < 0.0f)
        return false;
    const Box vp = {0.0f, 0.0f, -1.0f, ext_w(P), ext_h(P), 1.0f};
    if (!box_intersect(vp, box3(v[0].pos, v[1].pos, v[2].pos))) return false;
    *contained = box_contains(vp, v[0].pos) && box_contains(vp, v[1].pos) && box_contains(vp, v[2].pos);
    *obj = o;
    return true;
}

// The per-vertex attributes of surviving triangle t of object o (the normal
// matrix Apply does not influence the culls).
PR_DEV void vertex_attrs(const SetupParams& P, uint32_t t, uint32_t o, SubVtx* v, int* matid) {
    const float* nm = P.obj_normal + o * 16;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        v[k].nor = apply4_outline(ld4(P.nor[t * 3 + k]), nm);
        const float2 uv = P.uv[t * 3 + k];
        v[k].u = uv.x;
        v[k].v = uv.y;
        v[k].col = pack_col(P.col[t * 3 + k]);
    }
    int m = P.mat[t];
    if (m >= 0) m += P.obj_matbase[o];
    *matid = m;
}

PR_DEV bool transform_main(const SetupParams& P, const ObjCache* C, uint32_t t, SubVtx* v, float* recipw, int* matid,
                           bool* contained) {
    uint32_t o;
    if (!transform_main_geom(P, C, t, v, recipw, &o, contained)) return false;
    vertex_attrs(P, t, o, v, matid);
    return true;
}

// cpuForwardPass + draw for triangles fully inside the viewport
// (render/raster.go:257-269, 380-436); clipped ones go to clip_kernel.
PR_DEV void setup_main_one(const SetupParams& P, const ObjCache* C, uint32_t t, uint32_t* clip_list) {
    SubVtx v[3];
    float recipw[3];
    int matid = -1;
    bool contained = false;
    uint32_t obj = 0;
    const bool ok = t < P.n_tris && transform_main_geom(P, C, t, v, recipw, &obj, &contained);
    if (ok && !P.defer_attr) vertex_attrs(P, t, obj, v, &matid);
    if (ok && P.tri_scr) {
        float4* s = reinterpret_cast<float4*>(P.tri_scr + 12 * (size_t)t);
        s[0] = make_float4(v[0].pos.x, v[0].pos.y, recipw[0], v[1].pos.x);
        s[1] = make_float4(v[1].pos.y, recipw[1], v[2].pos.x, v[2].pos.y);
        s[2] = make_float4(recipw[2], 0.0f, 0.0f, 0.0f);
    }
    __syncwarp();
    const bool emit = ok && contained, clip = ok && !contained;
    uint32_t tot;
    const uint32_t ci = warp_reserve(&P.cnt->n_clipped, clip ? 1u : 0u, &tot);
    if (clip) clip_list[ci] = t;
    uint32_t ridx = warp_reserve(&P.cnt->n_rec, emit ? 1u : 0u, &tot);
    uint32_t area = 0;
    if (emit) {
        if (ridx >= P.cap_rec) {
            atomicOr(&P.cnt->overflow, 1u);
            atomicMax(&P.cnt->need_rec, ridx + 1);
        } else {
            P.first_rec[t] = ridx;
            area = write_sub(P, ridx, t * 8u, v, recipw, matid);
        }
    }
    emit_tasks_warp(P, &ridx, &area, 1);
}
// 8 blocks per SM (64 registers, a few spilled on rare paths): more warps to
// hide the per-triangle loads and stores measured faster than 80 registers at 6.
__global__ void __launch_bounds__(128, 8) setup_main_kernel(const __grid_constant__ SetupParams P, uint32_t* clip_list) {
    __shared__ ObjCache C;
    if (!P.obj_trans) obj_cache_fill(P, blockIdx.x * blockDim.x, C);  // uniform
    setup_main_one(P, &C, blockIdx.x * blockDim.x + threadIdx.x, clip_list);
}

// clipTriangle (render/clipping.go:70-157) for the listed triangles: fan
// sub-triangles with seq = tri*8 + i, drawn with the parent's recipw.
// j: this thread's entry of the clip list; the whole warp calls (warp
// reservations), with entries past the list's length idle.
PR_DEV void clip_one(const SetupParams& P, const uint32_t* clip_list, uint32_t j, uint32_t n) {
    SubVtx v[3];
    float recipw[3];
    int matid = -1;
    bool contained = false;
    uint32_t t = 0;
    int nc = 0;
    V4 clips[10];
    if (j < n) {
        t = clip_list[j];
        transform_main(P, nullptr, t, v, recipw, &matid, &contained);
        V4 in3[3] = {v[0].pos, v[1].pos, v[2].pos};
        nc = sutherland_hodgman(in3, ext_w(P), ext_h(P), clips);
        if (nc < 0) {
            atomicOr(&P.cnt->overflow, 4u);
            nc = 0;
        }
    }
    __syncwarp();
    const uint32_t nsub = nc > 2 ? (uint32_t)(nc - 2) : 0u;
    uint32_t tot;
    Counters* crec = P.cnt_rec ? P.cnt_rec : P.cnt;
    const uint32_t base = warp_reserve(&crec->n_rec, nsub, &tot);
    uint32_t ridxs[8], areas[8];
    int nw = 0;
    if (nsub > 0) {
        if (base + nsub > P.cap_rec) {
            atomicOr(&P.cnt->overflow, 1u);
            atomicMax(&P.cnt->need_rec, base + nsub);
        } else {
            P.first_rec[t] = base;
            const float psabc = sabc_of(v[0].pos.x, v[0].pos.y, v[1].pos.x, v[1].pos.y, v[2].pos.x, v[2].pos.y);
            SubVtx s[3];
            s[0] = clip_vertex(clips[0], v, psabc);
            for (int i = 2; i < nc; i++) {
                s[1] = clip_vertex(clips[i - 1], v, psabc);
                s[2] = clip_vertex(clips[i], v, psabc);
                ridxs[nw] = base + (uint32_t)(i - 2);
                areas[nw] = write_sub(P, ridxs[nw], t * 8u + (uint32_t)(i - 2), s, recipw, matid);
                nw++;
            }
        }
    }
    emit_tasks_warp(P, ridxs, areas, nw);
}

// clip_one with the work spread over a group of kClipLanes lanes per listed
// triangle. Lane k < 3 transforms vertex k (screen position, -1/W, normal);
// the group clips the triangle with one polygon vertex per lane
// (sutherland_hodgman_group); lane q re-interpolates polygon vertex q with
// its world position; lane `sub` assembles and writes fan sub-triangle sub.
// Each value is the one clip_one computes, from the same inputs in the same
// order; a warp just issues each per-vertex step once instead of once per
// vertex (a frame's few clipped triangles are a serial chain, often on cold
// instruction caches). The group's lanes reserve their records in lane
// order, so its sub-triangles keep consecutive records from first_rec[t].
struct ClipGroupSm {
    V4 pos[3], nor[3];
    float recipw[3];
    V4 ring[2][10];  // the clipper's polygons
    SubVtx cv[9];    // the polygon's re-interpolated vertices
    V4 mw[9];        // and their world positions
};
PR_DEV void clip_one_group(const SetupParams& P, const uint32_t* clip_list, uint32_t j, uint32_t n, uint32_t sub,
                           ClipGroupSm& G) {
    SubVtx v[3];
    float recipw[3];
    int matid = -1;
    uint32_t t = 0;
    if (j < n) {
        t = clip_list[j];
        // the listed triangle passed transform_main_geom's culls in setup
        const uint32_t k = min(sub, 2u);
        float trans[16];
        const uint32_t o = object_trans(P, nullptr, t, trans);
        const V4 cp = mulv(trans, ld4(P.pos[t * 3 + k]));
        const float rw = P.perspective ? __fdiv_rn(-1.0f, cp.w) : 1.0f;
        const V4 sp = pos4(viewport_apply(P, cp));
        const V4 nn = apply4_outline(ld4(P.nor[t * 3 + k]), P.obj_normal + o * 16);
        if (sub < 3u) {
            G.pos[k] = sp;
            G.nor[k] = nn;
            G.recipw[k] = rw;
        }
        int m = P.mat[t];
        if (m >= 0) m += P.obj_matbase[o];
        matid = m;
    }
    __syncwarp();
    V4 pv = {0.0f, 0.0f, 0.0f, 0.0f};  // this lane's polygon vertex
    if (j < n) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            v[k].pos = G.pos[k];
            v[k].nor = G.nor[k];
            recipw[k] = G.recipw[k];
            const float2 uv = P.uv[t * 3 + k];
            v[k].u = uv.x;
            v[k].v = uv.y;
            v[k].col = pack_col(P.col[t * 3 + k]);
        }
        pv = v[min(sub, 2u)].pos;
    }
    int nc = sutherland_hodgman_group(&pv, j < n ? 3 : 0, ext_w(P), ext_h(P), sub, G.ring);
    if (nc < 0) {
        if (sub == 0u) atomicOr(&P.cnt->overflow, 4u);
        nc = 0;
    }
    const bool attrs = P.arec && !P.defer_attr;
    if ((int)sub < nc && nc > 2) {
        const float psabc = sabc_of(v[0].pos.x, v[0].pos.y, v[1].pos.x, v[1].pos.y, v[2].pos.x, v[2].pos.y);
        const SubVtx cv = clip_vertex(pv, v, psabc);
        G.cv[sub] = cv;
        if (attrs) G.mw[sub] = world_of(P, cv.pos);
    }
    __syncwarp();
    const bool mine = (int)sub < nc - 2;
    uint32_t tot;
    Counters* crec = P.cnt_rec ? P.cnt_rec : P.cnt;
    uint32_t ridx = warp_reserve(&crec->n_rec, mine ? 1u : 0u, &tot);
    uint32_t area = 0;
    int nw = 0;
    if (mine) {
        if (ridx >= P.cap_rec) {
            atomicOr(&P.cnt->overflow, 1u);
            atomicMax(&P.cnt->need_rec, ridx + 1u);
        } else {
            if (sub == 0) P.first_rec[t] = ridx;
            const SubVtx s3[3] = {G.cv[0], G.cv[sub + 1], G.cv[sub + 2]};
            const V4 mw[3] = {G.mw[0], G.mw[sub + 1], G.mw[sub + 2]};
            area = write_sub(P, ridx, t * 8u + sub, s3, recipw, matid, attrs ? mw : nullptr);
            nw = 1;
        }
    }
    emit_tasks_warp(P, &ridx, &area, nw);
}
__global__ void __launch_bounds__(128) clip_kernel(const __grid_constant__ SetupParams P, const uint32_t* clip_list) {
    const uint32_t n = (P.cnt_rec ? P.cnt_rec : P.cnt)->n_clipped;
    constexpr uint32_t kPerBlock = 128 / kClipLanes;
    __shared__ ClipGroupSm s_g[kPerBlock];
    // grid-stride over the list (uniform per block, so every warp calls clip_one_group whole)
    for (uint32_t b = blockIdx.x * kPerBlock; b < n; b += gridDim.x * kPerBlock) {
        clip_one_group(P, clip_list, b + threadIdx.x / kClipLanes, n, threadIdx.x % kClipLanes,
                       s_g[threadIdx.x / kClipLanes]);
        __syncwarp();  // the group's scratch is free for its next entry
    }
}

// passShadows / drawDepth for one input triangle (render/shadow.go:137-192)
PR_DEV void setup_shadow_one(const SetupParams& P, const ObjCache* C, uint32_t t) {
    bool ok = false;
    SubVtx v[3];
    if (t < P.n_tris) {
        V4 p[3];
#pragma unroll
        for (int k = 0; k < 3; k++) p[k] = ld4(P.pos[t * 3 + k]);
        if (tri_valid_of(P, t, p)) {
            float trans[16];
            object_trans(P, C, t, trans);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                v[k].pos = pos4(viewport_apply(P, mulv(trans, p[k])));
                v[k].nor = {0, 0, 0, 0};
                v[k].u = v[k].v = 0;
                v[k].col = 0;
            }
            // cullBackFace (render/cull.go:26-28): culled iff cross.Z < 0
            ok = !(cross_z(__fsub_rn(v[1].pos.x, v[0].pos.x), __fsub_rn(v[1].pos.y, v[0].pos.y),
                           __fsub_rn(v[2].pos.x, v[0].pos.x), __fsub_rn(v[2].pos.y, v[0].pos.y)) < 0.0f);
            // cullViewFrustum (render/cull.go:15-23): NewAABB((W,H,1),(0,0,0),(0,0,-1))
            if (ok) {
                const Box vp = box3(V4{ext_w(P), ext_h(P), 1.0f, 1.0f}, V4{0, 0, 0, 1}, V4{0, 0, -1.0f, 1});
                ok = box_intersect(vp, box3(v[0].pos, v[1].pos, v[2].pos));
            }
        }
    }
    __syncwarp();
    uint32_t area = 0;
    if (ok) {
        float rw[3] = {1, 1, 1};
        area = write_sub(P, t, t, v, rw, -1);
    }
    uint32_t ridx = t;
    emit_tasks_warp(P, &ridx, &area, ok ? 1 : 0);
}
// 9 blocks per SM (56 registers): more warps than at 62 registers and 8.
__global__ void __launch_bounds__(128, 9) setup_shadow_kernel(const __grid_constant__ SetupParams P) {
    __shared__ ObjCache C;
    if (!P.obj_trans) obj_cache_fill(P, blockIdx.x * blockDim.x, C);  // uniform
    setup_shadow_one(P, &C, blockIdx.x * blockDim.x + threadIdx.x);
}

// Proj·View·Model per (pass, object), the product obj_cache_fill forms.
__global__ void obj_trans_kernel(const __grid_constant__ PassMats pm, int n_pass, const float* obj_model,
                                 uint32_t n_objects, float* out) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n_pass * n_objects * 16) return;
    const size_t po = e >> 4;
    const int pass = (int)(po / n_objects);
    const size_t o = po - (size_t)pass * n_objects;
    const uint32_t i = (uint32_t)(e >> 2) & 3u, j = (uint32_t)e & 3u;
    const float* m = pm.pv[pass] + i * 4;
    const float* q = obj_model + o * 16;
    out[e] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], q[j]), __fmul_rn(m[1], q[4 + j])), __fmul_rn(m[2], q[8 + j])),
                       __fmul_rn(m[3], q[12 + j]));
}

// ---------------------------------------------------------------- raster

constexpr int kRasterWarps = 8;

// One record of a warp's task batch in shared memory, laid out for 16-byte
// loads, with the per-triangle terms of the coverage test precomputed.
struct __align__(16) SmRec {
    float4 ab;  // A.x, A.y, B.x, B.y (screen vertices)
    float4 e0;  // (B-A).x, (B-A).y, (C-A).x, (C-A).y
    float4 e1;  // (C-B).x, (C-B).y, RN(1/Sabc) (0: no early reject), Sabc
    float4 zs;  // A.z, B.z, C.z, seq (bits)
    uint4 bb;   // bbox x0, bbox y0 + the task's first row, bbox width bw, ceil(2^32 / bw) (0 for bw = 1)
};

// A warp's raster scratch: its 32 records, the prefix of their pixel counts,
// and a ring of pixels that passed the early reject. The exact test runs
// only once 32 of them are queued, on all lanes, instead of on the lanes
// whose pixel happened to survive.
struct RasterWarpSm {
    SmRec rec[32];
    int start[32];    // first warp pixel of each task
    uint32_t tq[32];  // the task's first bbox index minus start (mod 2^32)
    uint32_t q[64];   // (slot << 27) | bbox index t (t < 2^17)
    uint32_t zk[32];  // early depth test: key of a bound on the record's depths (kNoEarlyZ: none)
};

// Early depth test. Visibility keeps the largest key per texel or pixel, so
// a fragment whose key cannot exceed the value already there changes
// nothing (values only grow during a pass). For a triangle with finite
// vertex depths Zi, a covered pixel (every computed barycentric b >=
// -Epsilon) gets z = RN(RN(RN(b0 Z0) + RN(b1 Z1)) + RN(b2 Z2)) with
// |sum b - 1| <= eta = (dA + 3 dS) / |Sabc| + 3u (1.06) (the sub-areas' and
// Sabc's rounding, as in tighten_box, and the divisions'), so z <= max Zi +
// M (eta + 6 Epsilon + 8u), M = max |Zi|, while eta <= 0.05 (b <= 1.06). The
// raster skips, before the exact test, every pixel whose current value is
// at least that bound's key (a stale read is only smaller: still sound).
constexpr uint32_t kNoEarlyZ = 0xFFFFFFFFu;  // no depth key reaches it (NaN depths take the NaN path)
PR_DEV uint32_t early_z_key(float ax, float ay, float bx, float by, float cx, float cy, float sabc, float4 zs) {
    const float z0 = zs.x, z1 = zs.y, z2 = zs.z;
    if (!(isfinite(z0) && isfinite(z1) && isfinite(z2) && isfinite(sabc) && sabc != 0.0f)) return kNoEarlyZ;
    const float mnx = fminf(fminf(ax, bx), cx), mxx = fmaxf(fmaxf(ax, bx), cx);
    const float mny = fminf(fminf(ay, by), cy), mxy = fmaxf(fmaxf(ay, by), cy);
    const float E = __fadd_ru(__fsub_ru(mxx, mnx), __fsub_ru(mxy, mny)), U = __fadd_ru(E, 4.0f);
    const float k6u = 3.6e-7f;  // >= 6 * 2^-24
    const float dS = __fmul_ru(__fmul_ru(k6u, E), U), dA = __fmul_ru(__fmul_ru(k6u, E), E);
    const float eta = __fdiv_ru(__fadd_ru(dA, __fmul_ru(3.0f, dS)), fabsf(sabc));
    if (!(eta <= 0.05f)) return kNoEarlyZ;
    const float M = fmaxf(fmaxf(fabsf(z0), fabsf(z1)), fabsf(z2));
    // 3u (1.06) + 6 Epsilon + 8u < 1.3e-6
    const float zb = __fadd_ru(fmaxf(fmaxf(z0, z1), z2), __fmul_ru(M, __fadd_ru(eta, 1.5e-6f)));
    return isfinite(zb) ? fkey(zb) : kNoEarlyZ;
}

// bbox index t of a record's pixel -> (px, py). t < 2^17 and bw <= 2^14, so
// t * bw < 2^32 and the multiply-high quotient is exact.
PR_DEV void rec_pixel(const uint4& bb, uint32_t t, int* px, int* py) {
    const uint32_t q = bb.w ? __umulhi(t, bb.w) : t;  // ceil(2^32 / 1) does not fit: one column, row t
    *px = (int)(bb.x + (t - q * bb.z));
    *py = (int)(bb.y + q);
}

// Conservative early reject (pixel certainly outside): the single-rounding
// estimate differs from the reference's double rounding by at most one ulp,
// so a margin of 2^-20 relative decides only pixels that are certainly out.
PR_DEV bool pixel_rejected(const SmRec& r, int px, int py) {
    const float fx = __fadd_rn(small_u2f((uint32_t)px), 0.5f), fy = __fadd_rn(small_u2f((uint32_t)py), 0.5f);
    const float4 ab = r.ab, e0 = r.e0, e1 = r.e1;
    const float apx = __fsub_rn(fx, ab.x), apy = __fsub_rn(fy, ab.y);
    const float bpx = __fsub_rn(fx, ab.z), bpy = __fsub_rn(fy, ab.w);
    const float inv = e1.z;
    const float w0 = __fmul_rn(__fmaf_rn(e1.x, bpy, -__fmul_rn(e1.y, bpx)), inv);
    const float w1 = __fmul_rn(__fmaf_rn(apx, e0.w, -__fmul_rn(apy, e0.z)), inv);
    const float w2 = __fmul_rn(__fmaf_rn(e0.x, apy, -__fmul_rn(e0.y, apx)), inv);
    const float shrink = 0.99999904632568359375f;  // 1 - 2^-20
    return __fmul_rn(w0, shrink) < -kEps || __fmul_rn(w1, shrink) < -kEps || __fmul_rn(w2, shrink) < -kEps;
}

// Coverage and depth of one pixel against one record (drawClipped's
// Barycoord / inside / z lines, render/raster.go:487-496).
PR_DEV bool pixel_depth(const SmRec& r, int px, int py, float* zout) {
    const float fx = __fadd_rn(small_u2f((uint32_t)px), 0.5f), fy = __fadd_rn(small_u2f((uint32_t)py), 0.5f);
    const float4 ab = r.ab, e0 = r.e0, e1 = r.e1;
    const float apx = __fsub_rn(fx, ab.x), apy = __fsub_rn(fy, ab.y);
    const float bpx = __fsub_rn(fx, ab.z), bpy = __fsub_rn(fy, ab.w);
    const float sabc = e1.w;
    const float sabp = cross_z(e0.x, e0.y, apx, apy);
    const float sapc = cross_z(apx, apy, e0.z, e0.w);
    const float sbcp = cross_z(e1.x, e1.y, bpx, bpy);
    const float b0 = __fdiv_rn(sbcp, sabc), b1 = __fdiv_rn(sapc, sabc), b2 = __fdiv_rn(sabp, sabc);
    if (b0 < -kEps || b1 < -kEps || b2 < -kEps) return false;
    const float4 zs = r.zs;
    *zout = __fadd_rn(__fadd_rn(__fmul_rn(b0, zs.x), __fmul_rn(b1, zs.y)), __fmul_rn(b2, zs.z));
    return true;
}

// The exact test and the depth write of one queued pixel.
PR_DEV void raster_pixel(const RasterParams& P, const RasterWarpSm& S, uint32_t ent) {
    const SmRec& r = S.rec[ent >> 27];
    int px, py;
    rec_pixel(r.bb, ent & 0x7FFFFFFu, &px, &py);
    float z;
    if (!pixel_depth(r, px, py, &z)) return;
    const uint32_t seq = __float_as_uint(r.zs.w);
    const bool zn = isnan(z);
    if (P.mode == kMain) {
        size_t i = (size_t)(P.H - 1 - py) * P.W + px;
        if (zn) {
            atomicMin(&P.nanseq[i], seq);
            atomicExch(&P.cnt_w->nan_flag, 1u);
            atomicAdd(&P.cnt_w->n_nan, 1u);
        } else {
            unsigned long long key = ((unsigned long long)fkey(z) << 32) | (unsigned long long)(0xFFFFFFFFu - seq);
            atomicMax(&P.keys[i], key);
        }
    } else if (P.mode == kMainFixup) {
        size_t i = (size_t)(P.H - 1 - py) * P.W + px;
        if (!zn) {
            uint32_t ns = P.nanseq[i];
            if (ns != kNone && seq < ns) P.beaten[i] = 1u;
        }
    } else if (P.mode == kShadow) {
        size_t i = (size_t)px + (size_t)py * P.W;
        if (zn) {
            if (P.lastnan) atomicMax(&P.lastnan[i], seq + 1u);
            atomicExch(&P.cnt_w->nan_flag, 1u);
            atomicAdd(&P.cnt_w->n_nan, 1u);
        } else {
            atomicMax(&P.smap[i], fkey(z));
        }
    } else {  // kShadowFixup
        size_t i = (size_t)px + (size_t)py * P.W;
        uint32_t ln = P.lastnan[i];
        if (!zn && ln != 0u && seq + 1u > ln) atomicMax(&P.smap[i], fkey(z));
    }
}

// Tasks [base, base + 32) of one pass, one per lane, pixels spread over the
// warp by a prefix scan of their counts.
PR_DEV void raster_warp(const RasterParams& P, const uint2* tasks, uint32_t base, uint32_t n_tasks, RasterWarpSm& S,
                        bool early_z) {
    const int lane = threadIdx.x & 31;
    uint32_t ti = base + lane;
    int cnt = 0;
    uint32_t qx0 = 0;
    if (ti < n_tasks) {
        uint2 tk = tasks[ti];
        const float4* rp = reinterpret_cast<const float4*>(P.rrec + tk.x);
        const float4 q0 = rp[0], q1 = rp[1], q2 = rp[2], q3 = rp[3];
        // record: A.xyz, B.xyz, C.xyz, Sabc, packed bbox x and y ranges, seq
        const float ax = q0.x, ay = q0.y, bx = q0.w, by = q1.x, cx = q1.z, cy = q1.w, sabc = q2.y;
        const uint32_t bxr = __float_as_uint(q2.z), byr = __float_as_uint(q2.w);
        const uint32_t x0 = bxr & 0xffffu, x1 = bxr >> 16, y0 = byr & 0xffffu, y1 = byr >> 16;
        SmRec& s = S.rec[lane];
        s.ab = make_float4(ax, ay, bx, by);
        s.e0 = make_float4(__fsub_rn(bx, ax), __fsub_rn(by, ay), __fsub_rn(cx, ax), __fsub_rn(cy, ay));
        const float as = fabsf(sabc);
        const float inv = (as >= 1e-30f && as <= 1e30f) ? __frcp_rn(sabc) : 0.0f;
        s.e1 = make_float4(__fsub_rn(cx, bx), __fsub_rn(cy, by), inv, sabc);
        s.zs = make_float4(q0.z, q1.y, q2.x, q3.x);
        S.zk[lane] = (early_z && (P.mode == kMain || P.mode == kShadow)) ? early_z_key(ax, ay, bx, by, cx, cy, sabc, s.zs)
                                                                          : kNoEarlyZ;
        if (x0 <= x1 && y0 <= y1) {
            const uint32_t bw = x1 - x0 + 1, area = bw * (y1 - y0 + 1);
            const uint32_t k0 = tk.y << P.task_shift;
            if (k0 < area) cnt = (int)min(area - k0, 1u << P.task_shift);
            const uint32_t qy0 = k0 / bw;  // one division per task
            qx0 = k0 - qy0 * bw;
            s.bb = make_uint4(x0, y0 + qy0, bw, bw > 1u ? 0xFFFFFFFFu / bw + 1u : 0u);
        }
    }
    int incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    S.start[lane] = incl - cnt;
    S.tq[lane] = qx0 - (uint32_t)(incl - cnt);
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    uint32_t head = 0, tail = 0;  // warp-uniform ring positions
    for (int g0 = 0; g0 < total; g0 += 32) {
        const int g = g0 + lane;
        bool keep = false;
        uint32_t ent = 0;
        if (g < total) {
            int j = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (S.start[j + step] <= g) j += step;
            const SmRec& r = S.rec[j];
            const uint32_t t = S.tq[j] + (uint32_t)g;
            int px, py;
            rec_pixel(r.bb, t, &px, &py);
            keep = !pixel_rejected(r, px, py);
            const uint32_t zk = S.zk[j];
            if (keep && zk != kNoEarlyZ) {
                if (P.mode == kShadow)
                    keep = __ldcg(P.smap + ((size_t)px + (size_t)py * P.W)) < zk;
                else
                    keep = __ldcg(P.keys + ((size_t)(P.H - 1 - py) * P.W + px)) <
                           (((unsigned long long)zk << 32) | 0xFFFFFFFFull);
            }
            ent = ((uint32_t)j << 27) | t;
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) S.q[(tail + __popc(m & lt)) & 63u] = ent;
        tail += __popc(m);
        if (tail - head >= 32u) {
            __syncwarp();
            raster_pixel(P, S, S.q[(head + lane) & 63u]);
            head += 32u;
            __syncwarp();
        }
    }
    __syncwarp();
    if ((uint32_t)lane < tail - head) raster_pixel(P, S, S.q[(head + lane) & 63u]);
    __syncwarp();
}

constexpr uint32_t kSpreadShare = 33;  // lists with fewer tasks per warp than this (and than grab) are spread
__global__ void __launch_bounds__(kRasterWarps * 32, 6) raster_kernel(const __grid_constant__ RasterParams P) {
    __shared__ RasterWarpSm s_w[kRasterWarps];
    const Counters* c = P.cnt;
    if (P.mode == kMainFixup || P.mode == kShadowFixup) {
        if (P.cnt_w->nan_flag == 0) return;  // flags of every list of the pass meet in cnt_w
    }
    const uint32_t n_tasks = c->n_tasks;
    if (c->overflow) return;
    const int warp = threadIdx.x >> 5;
    if (P.take) {
        // Dynamic: a task's cost is its bbox chunk, and consecutive tasks of
        // one object tend to be alike, so a static stride leaves a tail.
        // P.grab tasks per atomic (one counter serves every warp of the
        // pass): four 32-task batches on long lists, two on shorter ones,
        // where larger grabs would leave warps without work
        // The early depth test pays on passes with many fragments per pixel;
        // on short lists its extra read only lengthens each warp's chain.
        // A list of fewer than kSpreadShare (and fewer than grab) tasks per
        // warp (a small frame: a few thousand tasks, mostly from one or two
        // large triangles; a 2048^2 shadow pass) is spread
        // over every warp instead, down to one task each, by warp index: the
        // pass then lasts one or two small batches rather than grab tasks in
        // a few warps, and no warp waits on the counter. Its batches being
        // small, a block that becomes resident late adds little.
        auto drain = [&](const uint2* tasks, uint32_t* take, uint32_t n) {
            const uint32_t nw = gridDim.x * kRasterWarps;
            const uint32_t grab = P.grab ? P.grab : (n < nw * 256u ? 64u : 128u);
            const bool early_z = n >= nw * 32u;
            if (n / nw < min(grab, kSpreadShare)) {
                // spread: batches of max(n / nw, 1) tasks by warp index, at most two per warp
                const uint32_t g = max(n / nw, 1u);
                for (uint32_t base = (blockIdx.x * kRasterWarps + (uint32_t)warp) * g; base < n; base += nw * g)
                    raster_warp(P, tasks, base, min(base + g, n), s_w[warp], early_z);  // g <= 32
                return;
            }
            for (;;) {
                uint32_t base = 0;
                if ((threadIdx.x & 31) == 0) base = atomicAdd(take, grab);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base >= n) break;
                const uint32_t end = min(base + grab, n);
                for (uint32_t b = base; b < end; b += 32u) raster_warp(P, tasks, b, end, s_w[warp], early_z);
            }
        };
        drain(P.tasks, P.take, n_tasks);
        if (P.tasks2 && !P.cnt2->overflow) drain(P.tasks2, P.take2, P.cnt2->n_tasks);
        return;
    }
    const uint32_t gw = blockIdx.x * kRasterWarps + warp, nw = gridDim.x * kRasterWarps;
    for (uint32_t base = gw * 32u; base < n_tasks; base += nw * 32u)
        raster_warp(P, P.tasks, base, n_tasks, s_w[warp], n_tasks >= nw * 32u);
}

PR_DEV void resolve_one(int W, int H, const unsigned long long* keys, const uint32_t* nanseq, const uint32_t* beaten,
                        const Counters* cnt, uint32_t* win, float* depth_ao, size_t i) {
    if (i >= (size_t)W * H) return;
    unsigned long long key = keys[i];
    uint32_t w = kNone;
    float d = -1.0f;
    if (cnt->nan_flag && nanseq[i] != kNone && beaten[i] == 0u) {
        w = nanseq[i];
        d = __uint_as_float(0x7fc00000u);
    } else if (key != 0ull) {
        w = 0xFFFFFFFFu - (uint32_t)(key & 0xFFFFFFFFull);
        d = fkey_decode((uint32_t)(key >> 32));
    }
    win[i] = w;
    depth_ao[i] = d;
}

// Resolve (resolve_one) that also lists the winners' deferred attribute
// records (the first pixel to find its record pending, 1 -> 2, appends it)
// and, with ao_list, the frame's AO pixels: every covered pixel whose winning
// triangle's material has AO (tri_flags kTriAO; AmbientOcclusionShade's own
// condition, material/ao.go:22), appended tile by tile (32 x 8 blocks, warps
// in order) for the march's locality. One atomic per block and list.
__global__ void __launch_bounds__(256) resolve_listing_kernel(int W, int H, const unsigned long long* keys,
                                                              uint32_t* nanseq, uint32_t* beaten,
                                                              Counters* cnt, uint32_t* win, float* depth_ao,
                                                              const uint32_t* first_rec, uint32_t* attr_state,
                                                              uint32_t* vis, const uint8_t* tri_flags,
                                                              uint32_t* ao_list) {
    const int x = blockIdx.x * 32 + threadIdx.x, r = blockIdx.y * 8 + threadIdx.y;
    const int lane = threadIdx.x, warp = threadIdx.y;
    bool want = false, ao = false;
    uint32_t ridx = 0;
    const size_t i = (size_t)r * W + x;
    if (x < W && r < H) {
        resolve_one(W, H, keys, nanseq, beaten, cnt, win, depth_ao, i);
        // the NaN bookkeeping back to its rest state (resolve reads it last)
        if (cnt->nan_flag && nanseq[i] != kNone) {
            nanseq[i] = kNone;
            beaten[i] = 0u;
        }
        const uint32_t w = win[i];
        if (w != kNone) {
            ridx = first_rec[w >> 3] + (w & 7u);
            // most pixels find their record listed already: a plain read first
            want = attr_state[ridx] == 1u && atomicCAS(&attr_state[ridx], 1u, 2u) == 1u;
            ao = ao_list && (tri_flags[w >> 3] & kTriAO) != 0;
        }
    }
    __shared__ uint32_t s_cnt[2][8];
    __shared__ uint32_t s_base[2];
    const unsigned m = __ballot_sync(0xffffffffu, want), ma = __ballot_sync(0xffffffffu, ao);
    if (lane == 0) {
        s_cnt[0][warp] = (uint32_t)__popc(m);
        s_cnt[1][warp] = (uint32_t)__popc(ma);
    }
    __syncthreads();
    if (warp == 0 && lane < 2) {
        uint32_t tot = 0;
        for (int q = 0; q < 8; q++) tot += s_cnt[lane][q];
        s_base[lane] = tot ? atomicAdd(lane ? &cnt->n_ao : &cnt->n_vis, tot) : 0u;
    }
    __syncthreads();
    const uint32_t below = (1u << lane) - 1u;
    if (want) {
        uint32_t o = s_base[0] + (uint32_t)__popc(m & below);
        for (int q = 0; q < warp; q++) o += s_cnt[0][q];
        vis[o] = ridx;
    }
    if (ao) {
        uint32_t o = s_base[1] + (uint32_t)__popc(ma & below);
        for (int q = 0; q < warp; q++) o += s_cnt[1][q];
        ao_list[o] = (uint32_t)i;
    }
}

// The deferred attribute records of the listed records: everything comes
// back from the raster record (screen positions, -1/W, the triangle in seq)
// and the scene, by the same functions the setup uses, so the bits are
// those an eager setup writes. Three lanes per record, one per vertex (ten
// records per warp), and the face normal from the three world positions
// gathered by shuffles.
__global__ void __launch_bounds__(128) attr_kernel(const __grid_constant__ SetupParams P, const uint32_t* vis) {
    __shared__ __align__(16) float s_rec[4][10][36];  // each warp's ten records, stored whole
    const uint32_t n = P.cnt->n_vis;
    const int lane = threadIdx.x & 31, r = lane / 3, k = lane - 3 * r, warp = threadIdx.x >> 5;
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = wid * 10u; base < n; base += nw * 10u) {
        const uint32_t j = base + (uint32_t)r;
        const bool act = lane < 30 && j < n;
        V4 m = {0.0f, 0.0f, 0.0f, 0.0f};
        uint32_t ridx = 0, t = 0, o = 0;
        if (act) {
            ridx = vis[j];
            const float* R = reinterpret_cast<const float*>(P.rrec + ridx);
            t = __float_as_uint(R[12]) >> 3;
            o = P.blk_obj[t >> 7];
            while (o + 1 < P.n_objects && P.obj_first[o + 1] <= t) o++;
            const V4 pos = {R[3 * k], R[3 * k + 1], R[3 * k + 2], 1.0f};
            const V4 nor = apply4_outline(ld4(P.nor[t * 3 + k]), P.obj_normal + o * 16);
            const float2 uv = P.uv[t * 3 + k];
            m = apply4_outline(apply4_outline(apply4_outline(pos, P.viewport_inv), P.proj_inv), P.view_inv);  // render/raster.go:467-469
            float* A = s_rec[warp][r];
            A[k] = R[13 + k];  // recipw
            A[3 + 3 * k] = nor.x;
            A[4 + 3 * k] = nor.y;
            A[5 + 3 * k] = nor.z;
            A[12 + 2 * k] = uv.x;
            A[13 + 2 * k] = uv.y;
            A[18 + k] = __uint_as_float(pack_col(P.col[t * 3 + k]));
            A[21 + 3 * k] = m.x;
            A[22 + 3 * k] = m.y;
            A[23 + 3 * k] = m.z;
        }
        const float m1x = __shfl_down_sync(0xffffffffu, m.x, 1), m1y = __shfl_down_sync(0xffffffffu, m.y, 1),
                    m1z = __shfl_down_sync(0xffffffffu, m.z, 1);
        const float m2x = __shfl_down_sync(0xffffffffu, m.x, 2), m2y = __shfl_down_sync(0xffffffffu, m.y, 2),
                    m2z = __shfl_down_sync(0xffffffffu, m.z, 2);
        if (act && k == 0) {
            const V4 m1 = {m1x, m1y, m1z, 0.0f}, m2 = {m2x, m2y, m2z, 0.0f};
            const V4 fn = unit4(cross4(sub4(m1, m), sub4(m2, m)));  // render/raster.go:479
            float* A = s_rec[warp][r];
            A[30] = fn.x;
            A[31] = fn.y;
            A[32] = fn.z;
            A[33] = fn.w;
            int matid = P.mat[t];
            if (matid >= 0) matid += P.obj_matbase[o];
            A[34] = __int_as_float(matid);
            A[35] = 0.0f;
        }
        __syncwarp();
        // the warp's records out as whole 16-byte words: 9 per record
        const uint32_t nr = min(10u, n - base);
        for (uint32_t e = (uint32_t)lane; e < nr * 9u; e += 32u) {
            const uint32_t rr = e / 9u, w4 = e - rr * 9u;
            reinterpret_cast<float4*>(P.arec + vis[base + rr])[w4] = reinterpret_cast<const float4*>(s_rec[warp][rr])[w4];
        }
        __syncwarp();
    }
}

// Shadow NaN fix-up: pixels that saw a NaN-depth fragment restart from NaN
// (key 0) and take the maximum over the fragments drawn after the last one.
// (A small persistent grid: with no NaN fragment, the usual case, every block
// reads the flag and leaves.)
__global__ void shadow_fixup_reset_kernel(size_t n, const uint32_t* lastnan, uint32_t* smap, const Counters* cnt) {
    if (cnt->nan_flag == 0) return;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (lastnan[i] != 0u) smap[i] = 0u;
}

// After a pass that saw a NaN-depth fragment, put its NaN bookkeeping back to
// the state a pass starts from (a[] = va, b[] = vb); untouched otherwise, as
// only NaN fragments write it.
__global__ void nan_cleanup_kernel(size_t n, uint32_t* a, uint32_t va, uint32_t* b, uint32_t vb, const Counters* cnt) {
    if (cnt->nan_flag == 0) return;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        a[i] = va;
        if (b) b[i] = vb;
    }
}

__global__ void decode_shadow_kernel(const uint32_t* smap, float* out, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = fkey_decode(smap[i]);
}

// ---------------------------------------------------------------- shade

// Go math.Pow(0.5, n) for an integer 0 <= n <= 16 is exactly 2^-n.
PR_DEV float pow_half(int n) { return __uint_as_float((uint32_t)(127 - n) << 23); }

// The differentiation G-buffer of one covered pixel: triangle, material,
// flags, fixed factor (shadow now, AO multiplied in later), the screen
// barycentric weights of the pixel centre in the input triangle (for a
// material-less pixel: its perspective-correct weights), alpha, world
// position and face normal.
PR_DEV void diff_gbuffer_pixel(const ShadeParams& P, size_t i, uint32_t seq, int matid, const pr_material* mat,
                               float shadow_w, uint32_t alpha, V4 wp, V4 fn, float fx, float fy) {
    const uint32_t t = seq >> 3;
    const float4* S = reinterpret_cast<const float4*>(P.tri_scr + 12 * (size_t)t);
    const float4 s0 = S[0], s1 = S[1], s2 = S[2];
    const float x0 = s0.x, y0 = s0.y, w0 = s0.z, x1 = s0.w, y1 = s1.x, w1 = s1.y, x2 = s1.z, y2 = s1.w, w2 = s2.x;
    const float den = (y1 - y2) * (x0 - x2) + (x2 - x1) * (y0 - y2);
    float b0 = ((y1 - y2) * (fx - x2) + (x2 - x1) * (fy - y2)) / den;
    float b1 = ((y2 - y0) * (fx - x2) + (x0 - x2) * (fy - y2)) / den;
    float b2 = 1.0f - b0 - b1;
    uint32_t fl;
    if (mat) {
        fl = P.n_lights ? kDgbLit : kDgbConst;
        if (mat->flags & PR_MAT_FLAT_SHADING) fl |= kDgbFlat;
    } else {
        fl = kDgbUnlit;
        const bool persp = (P.flags & PR_FRAME_PERSPECTIVE) != 0;
        const float q0 = persp ? w0 * b0 : b0, q1 = persp ? w1 * b1 : b1, q2 = persp ? w2 * b2 : b2;
        const float inv = 1.0f / (q0 + q1 + q2);
        b0 = q0 * inv;
        b1 = q1 * inv;
        b2 = q2 * inv;
        shadow_w = 1.0f;
    }
    float4* D = P.dgb + 4 * i;
    D[0] = make_float4(__uint_as_float(t), __int_as_float(matid), __uint_as_float(fl), shadow_w);
    D[1] = make_float4(b0, b1, b2, small_u2f(alpha));
    D[2] = make_float4(wp.x, wp.y, wp.z, 1.0f);
    D[3] = make_float4(fn.x, fn.y, fn.z, fn.w);
}

// The shadow test of one light (render/raster.go:339-352, render/shadow.go:230-283):
// ws (ViewportToWorld of the pixel) through the light's view, projection and
// the map viewport, then the map depth 0.03 in front of the pixel's.
__device__ __noinline__ bool shadow_hit_exact(const ShadeParams& P, const LightK& L, V4 ws, size_t plane, int li) {
    const V4 sc = pos4(apply4(apply4(apply4(ws, L.lview), L.lproj), P.shadow_vp));
    const long long lx = go_f2i(sc.x), ly = go_f2i(sc.y);
    const long long idx =
        (long long)((unsigned long long)lx + (unsigned long long)ly * (unsigned long long)(long long)P.SW);
    if (idx > 0 && idx < (long long)plane) {
        const float sz = fkey_decode(P.smaps[plane * li + (size_t)idx]);
        return sc.z < __fsub_rn(sz, 0.03f);
    }
    return false;
}

// Vec4.Apply evaluated with single-rounding FMAs, and a bound on its distance
// from the reference's Apply (FMAs through float64) of the exact input, given
// a bound e on the input's distance (e.w = 0: the bottom row (0, 0, 0, 1)
// passes w through unchanged in both). Per row, both evaluations lie within
// g sum_j |m_ij||input_j| of their exact values (g = gamma_4 = 4u'/(1-4u'),
// u' = 2^-24 (1 + 2^-28) covering the double rounding), so
// |fast - reference| <= sum_j |m_ij| (e_j (1 + g) + 2g |x_j|), all in upward
// rounding (1 + g <= 1.0000005, 2g <= 4.8e-7).
PR_DEV V4 apply4_bounded(V4 x, V4 e, const float* m, V4* eo) {
    const V4 y = {__fmaf_rn(m[0], x.x, __fmaf_rn(m[1], x.y, __fmaf_rn(m[2], x.z, __fmul_rn(m[3], x.w)))),
                  __fmaf_rn(m[4], x.x, __fmaf_rn(m[5], x.y, __fmaf_rn(m[6], x.z, __fmul_rn(m[7], x.w)))),
                  __fmaf_rn(m[8], x.x, __fmaf_rn(m[9], x.y, __fmaf_rn(m[10], x.z, __fmul_rn(m[11], x.w)))),
                  __fmaf_rn(m[12], x.x, __fmaf_rn(m[13], x.y, __fmaf_rn(m[14], x.z, __fmul_rn(m[15], x.w))))};
    const float c1 = 1.0000005f, c2 = 4.8e-7f;
    const float w0 = __fmaf_ru(e.x, c1, __fmul_ru(c2, fabsf(x.x))), w1 = __fmaf_ru(e.y, c1, __fmul_ru(c2, fabsf(x.y)));
    const float w2 = __fmaf_ru(e.z, c1, __fmul_ru(c2, fabsf(x.z))), w3 = __fmul_ru(c2, fabsf(x.w));
    *eo = V4{__fmaf_ru(fabsf(m[0]), w0, __fmaf_ru(fabsf(m[1]), w1, __fmaf_ru(fabsf(m[2]), w2, __fmul_ru(fabsf(m[3]), w3)))),
             __fmaf_ru(fabsf(m[4]), w0, __fmaf_ru(fabsf(m[5]), w1, __fmaf_ru(fabsf(m[6]), w2, __fmul_ru(fabsf(m[7]), w3)))),
             __fmaf_ru(fabsf(m[8]), w0, __fmaf_ru(fabsf(m[9]), w1, __fmaf_ru(fabsf(m[10]), w2, __fmul_ru(fabsf(m[11]), w3)))),
             0.0f};
    return y;
}

// shadow_hit_exact from the single-rounding transform, when its bound
// decides every outcome (both truncated map coordinates and the depth
// compare); false: undecided, the caller runs the exact test. The division
// by w uses the same iw = RN(1/w) in both, so it scales the bound by |iw|
// and adds two roundings (2u |sc| < 2.4e-7 |sc|); 1e-30 covers underflow.
PR_DEV bool shadow_hit_fast(const ShadeParams& P, const LightK& L, V4 ws, size_t plane, int li, bool* hit) {
    V4 e = {0.0f, 0.0f, 0.0f, 0.0f};
    V4 v = apply4_bounded(ws, e, L.lview, &e);
    v = apply4_bounded(v, e, L.lproj, &e);
    v = apply4_bounded(v, e, P.shadow_vp, &e);
    float sx = v.x, sy = v.y, sz = v.z, ia = 1.0f;
    if (!(v.w == 1.0f || v.w == 0.0f)) {  // pos4
        const float iw = __fdiv_rn(1.0f, v.w);
        sx = __fmul_rn(v.x, iw);
        sy = __fmul_rn(v.y, iw);
        sz = __fmul_rn(v.z, iw);
        ia = __fmul_ru(fabsf(iw), 1.0000002f);
    }
    const float dx = __fadd_ru(__fmaf_ru(ia, e.x, __fmul_ru(2.4e-7f, fabsf(sx))), 1e-30f);
    const float dy = __fadd_ru(__fmaf_ru(ia, e.y, __fmul_ru(2.4e-7f, fabsf(sy))), 1e-30f);
    const float dz = __fadd_ru(__fmaf_ru(ia, e.z, __fmul_ru(2.4e-7f, fabsf(sz))), 1e-30f);
    const float xl = __fsub_rd(sx, dx), xh = __fadd_ru(sx, dx);
    const float yl = __fsub_rd(sy, dy), yh = __fadd_ru(sy, dy);
    if (!(fabsf(xl) < 8388608.0f && fabsf(xh) < 8388608.0f && fabsf(yl) < 8388608.0f && fabsf(yh) < 8388608.0f))
        return false;
    const int lx = trunc_small(xl), ly = trunc_small(yl);
    if (lx != trunc_small(xh) || ly != trunc_small(yh)) return false;
    const long long idx = (long long)lx + (long long)ly * (long long)P.SW;
    if (!(idx > 0 && idx < (long long)plane)) {
        *hit = false;
        return true;
    }
    const float thr = __fsub_rn(fkey_decode(P.smaps[plane * li + (size_t)idx]), 0.03f);
    if (__fadd_ru(sz, dz) < thr) {
        *hit = true;
        return true;
    }
    if (__fsub_rd(sz, dz) >= thr) {
        *hit = false;
        return true;
    }
    return false;
}

// Returns true for a pixel that AO still has to finish (its pre-AO colour is
// in rgba; the caller lists it).
// The colour of an image texture at a fragment (Texture.Query at the
// FragmentShader's lod), out of line: the shade kernel's other paths keep
// their registers.
static __device__ __noinline__ uint32_t texture_colour(const prt::TexDesc* td, const uint32_t* texels, float du,
                                                       float dv, float u, float v) {
    return prt::tex_query(*td, texels, prt::tex_lod(*td, du, dv), u, v);
}

// kTex: the scene has image textures (P.mat_tex set); without them the
// texture code is compiled out and the kernel keeps its registers.
template <bool kTex>
PR_DEV bool shade_one(const ShadeParams& P, int x, int r) {
    if (x >= P.W || r >= P.H) return false;
    const int W = P.W, H = P.H;
    const int y = H - 1 - r;
    const size_t i = (size_t)r * W + x;
    const uint32_t seq = P.win[i];
    uint32_t c0, c1, c2, c3;
    bool ao_pending = false;
    if (seq == kNone) {
        c0 = P.background[0]; c1 = P.background[1]; c2 = P.background[2]; c3 = P.background[3];
        if (P.tri_id) P.tri_id[i] = kNone;
        if (P.depth) P.depth[i] = 0.0f;
        if (P.gnor) P.gnor[i] = make_float4(0, 0, 0, 0);
        if (P.gfnor) P.gfnor[i] = make_float4(0, 0, 0, 0);
        if (P.gwpos) P.gwpos[i] = make_float4(0, 0, 0, 0);
        if (P.guvd) P.guvd[i] = make_float4(0, 0, 0, 0);
        if (P.gvcol) P.gvcol[i] = make_uchar4(0, 0, 0, 0);
        if (P.gmat) P.gmat[i] = -1;
        if (P.dgb) {
            float4* D = P.dgb + 4 * i;
            D[0] = make_float4(__uint_as_float(kNone), __int_as_float(-1), 0.0f, 1.0f);
            D[1] = make_float4(0.0f, 0.0f, 0.0f, small_u2f(c3));
            D[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            D[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    } else {
        const uint32_t ridx = P.first_rec[seq >> 3] + (seq & 7u);
        const float4* rp = reinterpret_cast<const float4*>(P.rrec + ridx);
        float4 q0 = rp[0], q1 = rp[1], q2 = rp[2];
        const float X0 = q0.x, Y0 = q0.y, Z0 = q0.z, X1 = q0.w, Y1 = q1.x, Z1 = q1.y, X2 = q1.z, Y2 = q1.w, Z2 = q2.x;
        const float sabc = q2.y;
        const AttrRec& A = P.arec[ridx];
        const float fx = __fadd_rn(small_u2f((uint32_t)x), 0.5f), fy = __fadd_rn(small_u2f((uint32_t)y), 0.5f);
        float bc[3];
        barycoord_s(fx, fy, X0, Y0, X1, Y1, X2, Y2, sabc, bc);
        const float z = __fadd_rn(__fadd_rn(__fmul_rn(bc[0], Z0), __fmul_rn(bc[1], Z1)), __fmul_rn(bc[2], Z2));
        const float rw0 = A.recipw[0], rw1 = A.recipw[1], rw2 = A.recipw[2];
        const float wc1 = __fmul_rn(rw0, bc[0]), wc2 = __fmul_rn(rw1, bc[1]), wc3 = __fmul_rn(rw2, bc[2]);
        const bool persp = (P.flags & PR_FRAME_PERSPECTIVE) != 0;
        const float norm = persp ? __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(wc1, wc2), wc3)) : 1.0f;
        auto wsum = [&](float a, float b, float c, float w1, float w2, float w3) {
            return __fadd_rn(__fadd_rn(__fmul_rn(w1, a), __fmul_rn(w2, b)), __fmul_rn(w3, c));
        };
        const float uvX = __fmul_rn(wsum(A.uv[0], A.uv[2], A.uv[4], wc1, wc2, wc3), norm);
        const float uvY = __fmul_rn(wsum(A.uv[1], A.uv[3], A.uv[5], wc1, wc2, wc3), norm);
        const int matid = A.matid;
        // a mipmapped image texture needs the derivatives for its lod
        bool need_lod = false;
        if (kTex && matid >= 0 && (uint32_t)matid < P.n_mats) {
            const int t = P.mat_tex[matid];
            need_lod = t >= 0 && P.tex[t].use_mipmap;
        }
        float du = 0.0f, dv = 0.0f;
        if (matid >= 0 && (P.guvd || need_lod)) {  // the UV derivatives feed that G-buffer and the lod
            float bx3[3], by3[3];
            barycoord_s(__fadd_rn(fx, 1.0f), fy, X0, Y0, X1, Y1, X2, Y2, sabc, bx3);
            float wc1x = __fmul_rn(rw0, bx3[0]), wc2x = __fmul_rn(rw1, bx3[1]), wc3x = __fmul_rn(rw2, bx3[2]);
            float normx = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(wc1x, wc2x), wc3x));
            barycoord_s(fx, __fadd_rn(fy, 1.0f), X0, Y0, X1, Y1, X2, Y2, sabc, by3);
            float wc1y = __fmul_rn(rw0, by3[0]), wc2y = __fmul_rn(rw1, by3[1]), wc3y = __fmul_rn(rw2, by3[2]);
            float normy = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(wc1y, wc2y), wc3y));
            float uvdU = __fmul_rn(wsum(A.uv[0], A.uv[2], A.uv[4], wc1x, wc2x, wc3x), normx);
            float uvdX = __fmul_rn(wsum(A.uv[1], A.uv[3], A.uv[5], wc1x, wc2x, wc3x), normx);
            float uvdV = __fmul_rn(wsum(A.uv[0], A.uv[2], A.uv[4], wc1y, wc2y, wc3y), normy);
            float uvdY = __fmul_rn(wsum(A.uv[1], A.uv[3], A.uv[5], wc1y, wc2y, wc3y), normy);
            float a = __fsub_rn(uvdU, uvX), b = __fsub_rn(uvdX, uvY);
            du = __fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b));
            float c = __fsub_rn(uvdV, uvX), d = __fsub_rn(uvdY, uvY);
            dv = __fadd_rn(__fmul_rn(c, c), __fmul_rn(d, d));
        }
        const V4 n = unit4(V4{wsum(A.nor[0], A.nor[3], A.nor[6], bc[0], bc[1], bc[2]),
                              wsum(A.nor[1], A.nor[4], A.nor[7], bc[0], bc[1], bc[2]),
                              wsum(A.nor[2], A.nor[5], A.nor[8], bc[0], bc[1], bc[2]), 0.0f});
        const V4 wp = {wsum(A.m[0], A.m[3], A.m[6], bc[0], bc[1], bc[2]), wsum(A.m[1], A.m[4], A.m[7], bc[0], bc[1], bc[2]),
                       wsum(A.m[2], A.m[5], A.m[8], bc[0], bc[1], bc[2]), 1.0f};
        const V4 fn = {A.fn[0], A.fn[1], A.fn[2], A.fn[3]};
        uint32_t vc[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            float s = __fmul_rn(wsum(col_ch(A.col[0], k), col_ch(A.col[1], k), col_ch(A.col[2], k), wc1, wc2, wc3), norm);
            vc[k] = go_f2u8(pclamp(s, 0.0f, 255.0f));
        }
        if (P.tri_id) P.tri_id[i] = seq >> 3;
        if (P.depth) P.depth[i] = z;
        if (P.gnor) P.gnor[i] = make_float4(n.x, n.y, n.z, n.w);
        if (P.gfnor) P.gfnor[i] = make_float4(fn.x, fn.y, fn.z, fn.w);
        if (P.gwpos) P.gwpos[i] = make_float4(wp.x, wp.y, wp.z, wp.w);
        if (P.guvd) P.guvd[i] = make_float4(uvX, uvY, du, dv);
        if (P.gvcol) P.gvcol[i] = make_uchar4(vc[0], vc[1], vc[2], vc[3]);
        if (P.gmat) P.gmat[i] = matid;

        c0 = vc[0]; c1 = vc[1]; c2 = vc[2]; c3 = vc[3];
        float shadow_w = 1.0f;
        const pr_material* mat = (matid >= 0 && (uint32_t)matid < P.n_mats) ? &P.mats[matid] : nullptr;
        if (mat) {
            // FragmentShader (shader/blinn_cpu.go:24-106): the texture colour
            // Query(lod, U, 1-V); a uniform texture gives its texel at any lod
            uint32_t t0 = mat->texture[0], t1 = mat->texture[1], t2 = mat->texture[2], t3 = mat->texture[3];
            const int tix = kTex ? P.mat_tex[matid] : -1;  // the material's image texture, if any
            if (tix >= 0) {
                const uint32_t tc = texture_colour(P.tex + tix, P.texels, du, dv, uvX, __fsub_rn(1.0f, uvY));
                t0 = tc & 0xffu;
                t1 = (tc >> 8) & 0xffu;
                t2 = (tc >> 16) & 0xffu;
                t3 = tc >> 24;
            }
            if (P.n_lights == 0) {
                c0 = t0; c1 = t1; c2 = t2; c3 = t3;
            } else {
                const float cr = small_u2f(t0), cg = small_u2f(t1), cb = small_u2f(t2);
                float LaR = 0, LaG = 0, LaB = 0;
                for (int e = 0; e < P.n_ambient; e++) {
                    LaR = __fadd_rn(LaR, __fmul_rn(P.ambient[e], cr));
                    LaG = __fadd_rn(LaG, __fmul_rn(P.ambient[e], cg));
                    LaB = __fadd_rn(LaB, __fmul_rn(P.ambient[e], cb));
                }
                float LdR = 0, LdG = 0, LdB = 0, LsR = 0, LsG = 0, LsB = 0;
                const V4 nn = (mat->flags & PR_MAT_FLAT_SHADING) ? fn : n;
                const V4 cam = {P.cam[0], P.cam[1], P.cam[2], 1.0f};
                const V4 Vv = unit4(sub4(cam, wp));  // the same for every light
                for (int li = 0; li < P.n_lights; li++) {
                    const LightK& L = P.lights[li];
                    V4 Lv;
                    float I;
                    if (L.type == PR_LIGHT_POINT) {
                        const V4 Ldir = sub4(V4{L.pos[0], L.pos[1], L.pos[2], 1.0f}, wp);
                        // Ldir.Unit() and Ldir.Len() share one length
                        const float ln = len4(Ldir);
                        const float inv = __fdiv_rn(1.0f, ln);
                        Lv = V4{__fmul_rn(Ldir.x, inv), __fmul_rn(Ldir.y, inv), __fmul_rn(Ldir.z, inv), __fmul_rn(Ldir.w, inv)};
                        I = __fdiv_rn(L.intensity, ln);
                    } else {
                        Lv = V4{-L.dir[0], -L.dir[1], -L.dir[2], 0.0f};
                        I = L.intensity;
                    }
                    V4 Hv = unit4(add4(Lv, Vv));
                    float Ld = pclamp(dot4(nn, Lv), 0.0f, 1.0f);
                    float Ls = go_pow_f32(pclamp(dot4(nn, Hv), 0.0f, 1.0f), mat->shininess);
                    LdR = __fadd_rn(LdR, __fmul_rn(__fmul_rn(Ld, cr), I));
                    LdG = __fadd_rn(LdG, __fmul_rn(__fmul_rn(Ld, cg), I));
                    LdB = __fadd_rn(LdB, __fmul_rn(__fmul_rn(Ld, cb), I));
                    LsR = __fadd_rn(LsR, __fmul_rn(__fmul_rn(Ls, L.color[0]), I));
                    LsG = __fadd_rn(LsG, __fmul_rn(__fmul_rn(Ls, L.color[1]), I));
                    LsB = __fadd_rn(LsB, __fmul_rn(__fmul_rn(Ls, L.color[2]), I));
                }
                auto fin = [&](float La, float Ld, float Ls, uint8_t kd, uint8_t ks) {
                    float v = __fadd_rn(__fadd_rn(La, __fdiv_rn(__fmul_rn(small_u2f(kd), Ld), 255.0f)),
                                        __fdiv_rn(__fmul_rn(small_u2f(ks), Ls), 255.0f));
                    return go_f2u8(pclamp(pround(v), 0.0f, 255.0f));
                };
                c0 = fin(LaR, LdR, LsR, mat->diffuse[0], mat->specular[0]);
                c1 = fin(LaG, LdG, LsG, mat->diffuse[1], mat->specular[1]);
                c2 = fin(LaB, LdB, LsB, mat->diffuse[2], mat->specular[2]);
                c3 = t3;
            }
            // Shadows (render/raster.go:339-352, render/shadow.go:230-283)
            if ((P.flags & PR_FRAME_SHADOWMAP) && (mat->flags & PR_MAT_RECEIVE_SHADOW)) {
                int occl = 0;
                const size_t plane = (size_t)P.SW * P.SH;
                // ViewportToWorld of the pixel, the same for every light
                const V4 ws = apply4(V4{small_u2f((uint32_t)x), small_u2f((uint32_t)y), z, 1.0f}, P.s2w);
                for (int li = 0; li < P.n_lights; li++) {
                    const LightK& L = P.lights[li];
                    if (!L.cast) {
                        occl++;
                        continue;
                    }
                    bool hit = false;
                    if (!(L.sfast && shadow_hit_fast(P, L, ws, plane, li, &hit))) hit = shadow_hit_exact(P, L, ws, plane, li);
                    occl += hit ? 1 : 0;
                }
                float w = pow_half(occl);
                shadow_w = w;
                c0 = go_f2u8(__fmul_rn(small_u2f(c0), w));
                c1 = go_f2u8(__fmul_rn(small_u2f(c1), w));
                c2 = go_f2u8(__fmul_rn(small_u2f(c2), w));
            }
            // AmbientOcclusionShade (material/ao.go:20-73) runs in ao_kernel
            // on a compacted list of these pixels.
            ao_pending = (mat->flags & PR_MAT_AO) && P.rgba && P.ao_list;
        }
        if (P.dgb) diff_gbuffer_pixel(P, i, seq, matid, mat, shadow_w, c3, wp, fn, fx, fy);
    }
    if (ao_pending) {
        P.rgba[i] = make_uchar4(c0, c1, c2, c3);  // pre-AO, pre-gamma colour
        return true;
    }
    if (P.flags & PR_FRAME_GAMMA) {
        c0 = P.gamma[c0];
        c1 = P.gamma[c1];
        c2 = P.gamma[c2];
    }
    if (P.rgba) P.rgba[i] = make_uchar4(c0, c1, c2, c3);
    return false;
}

// Block-wide append of the AO pixels of a 32 x 8 tile (every thread of the
// 256-thread block calls): one atomic per tile, so the list runs tile by
// tile and an AO block marches a compact patch whose taps overlap.
PR_DEV void ao_append_tile(const ShadeParams& P, bool pending, uint32_t i) {
    __shared__ uint32_t s_cnt[8];
    __shared__ uint32_t s_base;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x, warp = tid >> 5, lane = tid & 31;
    const unsigned m = __ballot_sync(0xffffffffu, pending);
    if (lane == 0) s_cnt[warp] = (uint32_t)__popc(m);
    __syncthreads();
    if (tid == 0) {
        uint32_t tot = 0;
        for (int w = 0; w < 8; w++) tot += s_cnt[w];
        s_base = tot ? atomicAdd(&P.cnt_w->n_ao, tot) : 0u;
    }
    __syncthreads();
    if (pending) {
        uint32_t o = s_base + (uint32_t)__popc(m & ((1u << lane) - 1u));
        for (int w = 0; w < warp; w++) o += s_cnt[w];
        P.ao_list[o] = i;
    }
}
template <bool kTex>
// 4 blocks per SM (64 registers, a few spilled): 32 warps to hide the
// record, attribute and shadow-map loads measured faster than 80 registers at 3.
__global__ void __launch_bounds__(256, 4) shade_kernel(const __grid_constant__ ShadeParams P) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y * blockDim.y + threadIdx.y;
    const bool pending = shade_one<kTex>(P, x, r);
    if (P.ao_list && !P.ao_listed) ao_append_tile(P, pending, (uint32_t)r * (uint32_t)P.W + (uint32_t)x);
}

// ---------------------------------------------------------------- AO

// The 8 march directions (material/ao.go:28): cos/sin of the float32 angle.
__constant__ float c_ao_dir[2][8];

constexpr int kAoTaps = 100;     // t = 0 .. 99 (material/ao.go:44)
constexpr int kAoTable = 100;    // tap offsets for t = 2 .. 101 (t >= 100: padding, offset 0)
constexpr float kAoSkip = 1.0f - 0x1p-20f;
constexpr int kAoThreads = 256;

// distance of material/ao.go:52, p.Sub(cur).Len() with z = w = 0
PR_DEV float ao_distance(float pxf, float pyf, float cx, float cy) {
    const float ddx = __fsub_rn(pxf, cx), ddy = __fsub_rn(pyf, cy);
    return __fsqrt_rn(fma64f(ddx, ddx, __fmul_rn(ddy, ddy)));
}

// The exact ratio elevation/distance of tap t >= 2 (distance >= 1.998).
__device__ __noinline__ float ao_exact_ratio(int t, float el, float pxf, float pyf, float dX, float dY) {
    const float tf = small_u2f((uint32_t)t);
    const float cx = __fadd_rn(pxf, __fmul_rn(dX, tf)), cy = __fadd_rn(pyf, __fmul_rn(dY, tf));
    return __fdiv_rn(el, ao_distance(pxf, pyf, cx, cy));
}

// One tap evaluated from its float coordinates, as the reference does:
// cur = p + dir*t, int(cur) (in [0, W) for the taps the caller passes), the
// distance check and the ratio. A tap that cannot raise best past the lower
// bound lb (elev <= lb (1 - 2^-20) (t - 0.0101), using dist >= t - 0.002)
// needs neither its distance nor its division. Returns false for a NaN
// elevation at dist >= 1.
PR_DEV bool ao_tap_exact(int t, float pxf, float pyf, float dX, float dY, int W, int H, const float* depth,
                         float z, float lb, float& best) {
    const float tf = small_u2f((uint32_t)t);
    const float cx = __fadd_rn(pxf, __fmul_rn(dX, tf)), cy = __fadd_rn(pyf, __fmul_rn(dY, tf));
    const uint32_t ix = __float_as_uint(__fadd_rz(fmaxf(cx, 0.0f), 8388608.0f)) - 0x4B000000u;
    const uint32_t iy = __float_as_uint(__fadd_rz(fmaxf(cy, 0.0f), 8388608.0f)) - 0x4B000000u;
    const float el = __fsub_rn(__ldg(depth + ((size_t)(H - 1 - (int)iy) * W + ix)), z);
    if (el <= __fmul_rn(__fmul_rd(lb, kAoSkip), __fsub_rd(tf, 0.0101f))) return true;
    const float d = ao_distance(pxf, pyf, cx, cy);
    if (d < 1.0f) return true;
    if (isnan(el)) return false;
    best = fmaxf(best, __fdiv_rn(el, d));
    return true;
}

// The elevation of fast-path tap t again (settling a pending tap reloads it
// instead of carrying it).
PR_DEV float ao_tap_elev(const int (*s_off)[kAoTable], int k, int t, const float* p0, const float* pA, int tstar, float z,
                         bool tiny) {
    const float* q = (tiny && t < tstar) ? pA : p0;
    return __fsub_rn(__ldg(q + s_off[k][t - 2]), z);
}

// maxElevationAngle's march for taps 2 .. 101 in groups of four, from shared
// tables of index offsets and of bounds on 1/dist (see ao_kernel): the exact
// ratio RN(elev/dist) of a tap lies in [RD(elev rlo), RU(elev rhi)]. A tap
// whose upper bound does not exceed lb cannot raise the maximum; the others
// are candidates, of which one is held pending by its interval. Exact ratios
// are computed only when a new candidate's interval overlaps the pending one
// and, once, for the final pending tap. best is exact throughout and lb <= the
// largest exact ratio seen so far.
template <bool TINY>
PR_DEV bool ao_fast_groups(int n_groups, const int (*s_off)[kAoTable], const float (*s_rlo)[kAoTable],
                           const float (*s_rhi)[kAoTable], int k, const float* p0, const float* pA, int tstar, float z,
                           float pxf, float pyf, float dX, float dY, float& best) {
    float lb = best;
    int pt = 0;
    float phi = 0.0f;
    bool nan_seen = false;
#pragma unroll 2
    for (int g = 0; g < n_groups; g++) {
        const int t0 = 4 * g + 2;
        const int4 o = *reinterpret_cast<const int4*>(&s_off[k][4 * g]);
        const float4 rh = *reinterpret_cast<const float4*>(&s_rhi[k][4 * g]);
        const float* q0 = (TINY && t0 < tstar) ? pA : p0;
        const float* q1 = (TINY && t0 + 1 < tstar) ? pA : p0;
        const float* q2 = (TINY && t0 + 2 < tstar) ? pA : p0;
        const float* q3 = (TINY && t0 + 3 < tstar) ? pA : p0;
        float el[4], hi[4];
        el[0] = __fsub_rn(__ldg(q0 + o.x), z);
        el[1] = __fsub_rn(__ldg(q1 + o.y), z);
        el[2] = __fsub_rn(__ldg(q2 + o.z), z);
        el[3] = __fsub_rn(__ldg(q3 + o.w), z);
        hi[0] = __fmul_ru(el[0], rh.x);
        hi[1] = __fmul_ru(el[1], rh.y);
        hi[2] = __fmul_ru(el[2], rh.z);
        hi[3] = __fmul_ru(el[3], rh.w);
        const bool c0 = !(hi[0] <= lb), c1 = !(hi[1] <= lb), c2 = !(hi[2] <= lb), c3 = !(hi[3] <= lb);
        if (c0 | c1 | c2 | c3) {
            const float4 rl = *reinterpret_cast<const float4*>(&s_rlo[k][4 * g]);
            const float lo[4] = {rl.x, rl.y, rl.z, rl.w};
            const bool cu[4] = {c0, c1, c2, c3};
            // Branch-free: each candidate becomes the pending tap; a pending
            // tap it overlaps is recorded and settled after the group (rare).
            int st[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                nan_seen |= isnan(el[u]);
                const bool take = cu[u] & !isnan(el[u]);
                const float rlo = __fmul_rd(el[u], lo[u]);
                const bool ov = take & (pt != 0) & !(rlo >= phi);
                st[u] = ov ? pt : 0;
                pt = take ? t0 + u : pt;
                phi = take ? hi[u] : phi;
                lb = take ? fmaxf(lb, rlo) : lb;
            }
            if (nan_seen) return false;
            if ((st[0] | st[1] | st[2] | st[3]) != 0) {
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (st[u]) best = fmaxf(best, ao_exact_ratio(st[u], ao_tap_elev(s_off, k, st[u], p0, pA, tstar, z,
                                                                                     TINY),
                                                               pxf, pyf, dX, dY));
                lb = fmaxf(lb, best);
            }
        }
    }
    if (pt != 0) best = fmaxf(best, ao_exact_ratio(pt, ao_tap_elev(s_off, k, pt, p0, pA, tstar, z, TINY), pxf, pyf, dX, dY));
    return true;
}

// The exact ratios of the taps of group g (taps 4g+2 .. 4g+5) whose upper
// bound exceeds lb; returns their maximum (0 if none). Each lane loops over
// its own such taps only.
template <bool TINY>
__device__ __noinline__ float ao_settle_group(const int (*s_off)[kAoTable], const float (*s_rhi)[kAoTable], int k, int g,
                                              const float* p0, const float* pA, int tstar, float z, float pxf, float pyf,
                                              float dX, float dY, float lb) {
    const int t0 = 4 * g + 2;
    float el[4];
    unsigned m = 0;
#pragma unroll
    for (int u = 0; u < 4; u++) {
        el[u] = ao_tap_elev(s_off, k, t0 + u, p0, pA, tstar, z, TINY);
        if (__fmul_ru(el[u], s_rhi[k][4 * g + u]) > lb) m |= 1u << u;
    }
    float r = 0.0f;
    while (m) {
        const int u = __ffs(m) - 1;
        m &= m - 1u;
        const float e = u == 0 ? el[0] : (u == 1 ? el[1] : (u == 2 ? el[2] : el[3]));
        r = fmaxf(r, ao_exact_ratio(t0 + u, e, pxf, pyf, dX, dY));
    }
    return r;
}

// The march of ao_fast_groups for frames without NaN depths, bookkept per
// unit of two groups of four taps (eight taps; a last odd group alone): a
// unit is a candidate when the largest upper bound of its taps exceeds lb;
// it then raises lb by the largest lower bound of its taps and becomes the
// pending unit (bounded above by that largest upper bound phi). A pending
// unit is settled (its taps above lb evaluated exactly, group by group) only
// when a later candidate's lower bound does not clear phi, and at the end.
// Every tap above the final lb is thus evaluated exactly, and best is the
// exact maximum, whatever the unit's size; eight taps per unit halve the
// candidate steps a warp issues (some lane of a warp is a candidate in most
// units). UNROLL: the unit loop unrolled by two (the single-view kernel, at
// 64 registers; the batched kernel keeps one unit at a time).
template <bool TINY, bool UNROLL>
PR_DEV void ao_fast_groups_nf(int n_groups, const int (*s_off)[kAoTable], const float (*s_rlo)[kAoTable],
                              const float (*s_rhi)[kAoTable], int k, const float* p0, const float* pA, int tstar,
                              float z, float pxf, float pyf, float dX, float dY, float& best) {
    float lb = best;
    int pg = -1, pn = 0;  // pending unit: first group, group count
    float phi = 0.0f;
    // the elevations of group g's taps and the largest upper bound of their ratios
    auto group_hi = [&](int g, float& gh, float e[4]) {
        const int t0 = 4 * g + 2;
        const int4 o = *reinterpret_cast<const int4*>(&s_off[k][4 * g]);
        const float4 rh = *reinterpret_cast<const float4*>(&s_rhi[k][4 * g]);
        const float* q0 = (TINY && t0 < tstar) ? pA : p0;
        const float* q1 = (TINY && t0 + 1 < tstar) ? pA : p0;
        const float* q2 = (TINY && t0 + 2 < tstar) ? pA : p0;
        const float* q3 = (TINY && t0 + 3 < tstar) ? pA : p0;
        e[0] = __fsub_rn(__ldg(q0 + o.x), z);
        e[1] = __fsub_rn(__ldg(q1 + o.y), z);
        e[2] = __fsub_rn(__ldg(q2 + o.z), z);
        e[3] = __fsub_rn(__ldg(q3 + o.w), z);
        gh = fmaxf(fmaxf(__fmul_ru(e[0], rh.x), __fmul_ru(e[1], rh.y)), fmaxf(__fmul_ru(e[2], rh.z), __fmul_ru(e[3], rh.w)));
    };
    auto group_lo = [&](int g, const float e[4]) {
        const float4 rl = *reinterpret_cast<const float4*>(&s_rlo[k][4 * g]);
        return fmaxf(fmaxf(__fmul_rd(e[0], rl.x), __fmul_rd(e[1], rl.y)), fmaxf(__fmul_rd(e[2], rl.z), __fmul_rd(e[3], rl.w)));
    };
    auto settle = [&]() {
        for (int q = 0; q < pn; q++)
            best = fmaxf(best, ao_settle_group<TINY>(s_off, s_rhi, k, pg + q, p0, pA, tstar, z, pxf, pyf, dX, dY, lb));
        lb = fmaxf(lb, best);
    };
    int g = 0;
#pragma unroll(UNROLL ? 2 : 1)
    for (; g + 1 < n_groups; g += 2) {
        float ea[4], eb[4], ha, hb;
        group_hi(g, ha, ea);
        group_hi(g + 1, hb, eb);
        const float gh = fmaxf(ha, hb);
        if (gh > lb) {
            const float gl = fmaxf(group_lo(g, ea), group_lo(g + 1, eb));
            lb = fmaxf(lb, gl);
            if (pg >= 0 && gl < phi) settle();
            pg = g;
            pn = 2;
            phi = gh;
        }
    }
    if (g < n_groups) {  // the last group alone
        float e[4], gh;
        group_hi(g, gh, e);
        if (gh > lb) {
            const float gl = group_lo(g, e);
            lb = fmaxf(lb, gl);
            if (pg >= 0 && gl < phi) settle();
            pg = g;
            pn = 1;
            phi = gh;
        }
    }
    if (pg >= 0) settle();
}

// AmbientOcclusionShade (material/ao.go:20-73) for the pixels the shade
// kernel listed, one thread per pixel. Per direction, maxangle is the Max
// over taps of float32(Atan(elev/dist)); Atan and the rounding to float32 are
// monotone, so it is float32(Atan(best)) with best the largest ratio, and
// only positive ratios can exceed the initial 0. A NaN ratio (at a tap not
// skipped for dist < 1) makes the direction, and so the pixel, NaN.
//
// Tap positions. cur = p + float32(dir*t) (dir.Scale(t,t,1,1) then Add) and
// Go's int(cur) is in [0, W) exactly when -1 < cur < W; cur moves
// monotonically in t, so the first tap outside the buffer (where the
// reference returns) bounds the march, and is found by binary search unless
// tap 99 is inside. For x >= 0 and a = float32(dX t):
//  * a "regular" component (a an integer, or at least 2^-10 below the next
//    integer for every t <= 99, which holds for all 8 directions) has
//    int(RN(x + a)) = x + floor(a) for coordinates below 16384, since
//    RN(x + a) cannot round up to the next integer;
//  * a tiny negative component (-1 < a < 0: the cos of float32(Pi/2) and the
//    sin of float32(Pi)) has int(RN(x - |a|)) = x while |a| is at most half
//    the gap below x, else x - 1; |a| grows with t, so the switch happens at
//    one tap t*, found by binary search.
// So while cur >= 0, the depth index of tap t is the pixel's index plus a
// per-(direction, t) offset from a table, plus a correction before t* for a
// tiny component. Taps with cur < 0 (int truncates toward zero there) and
// the last taps that do not fill a group of four take the float path.
// Tap 1 always takes it: its distance may fall below 1 (diagonals).
// The tap tables of a W x H frame (every thread of the block calls).
PR_DEV void ao_tables(const AoParams& P, int (*s_off)[kAoTable], float (*s_rlo)[kAoTable], float (*s_rhi)[kAoTable]) {
    const int W = P.W;
    for (int e = threadIdx.x; e < 8 * kAoTable; e += blockDim.x) {
        const int k = e / kAoTable, q = e - k * kAoTable, t = q + 2;
        int o = 0;
        float rlo = 0.0f, rhi = 0.0f;
        if (t < kAoTaps && k < P.n_dirs) {
            const float tf = small_u2f((uint32_t)t);
            const float ax = __fmul_rn(c_ao_dir[0][k], tf), ay = __fmul_rn(c_ao_dir[1][k], tf);
            o = (int)floorf(ax) - (int)floorf(ay) * W;
            // |dist - |(ax, ay)|| <= sqrt(2) (h + 2^-18) + 2.5e-7 |(ax, ay)|: h bounds the rounding of
            // cur = RN(p + a), 2^-18 that of p - cur, the rest the float32 steps of both distances
            const float d0 = __fsqrt_rn(__fmaf_rn(ax, ax, __fmul_rn(ay, ay)));
            const float dl = __fadd_ru(__fmul_ru(1.5f, __fadd_ru(P.ao_half_ulp, 4e-6f)), __fmul_ru(d0, 4e-7f));
            rlo = __frcp_rd(__fadd_ru(d0, dl));
            rhi = __frcp_ru(__fsub_rd(d0, dl));
        }
        s_off[k][q] = o;
        s_rlo[k][q] = rlo;
        s_rhi[k][q] = rhi;
    }
}

PR_DEV void ao_finish(const AoParams& P, uint32_t i, float T);

// One pixel of the AO list: its total T, then (kApply) the colour scaling,
// or (!kApply) T stored for ao_apply_kernel.
template <bool kApply>
PR_DEV void ao_one(const AoParams& P, uint32_t j, const int (*s_off)[kAoTable], const float (*s_rlo)[kAoTable],
                   const float (*s_rhi)[kAoTable]) {
    const int W = P.W, H = P.H;
    const float fW = (float)W, fH = (float)H;
    const uint32_t i = P.list[j];
    const int r = (int)(i / (uint32_t)W);
    const int x = (int)i - r * W;
    const int y = H - 1 - r;
    const float* p0 = P.depth + i;
    const float z = *p0;
    const float pxf = small_u2f((uint32_t)x), pyf = small_u2f((uint32_t)y);
    // no NaN-depth fragment reached this frame's depth buffer (the raster flags every one)
    const bool nan_free = P.cnt->nan_flag == 0u;
    float total = 0.0f;
    bool nanpix = false;
    for (int k = 0; k < P.n_dirs; k++) {
        const float dX = c_ao_dir[0][k], dY = c_ao_dir[1][k];
        int t_end = kAoTaps, t_fast = kAoTaps;
        {
            const float cx = __fadd_rn(pxf, __fmul_rn(dX, 99.0f)), cy = __fadd_rn(pyf, __fmul_rn(dY, 99.0f));
            if (!(cx >= 0.0f && cx < fW && cy >= 0.0f && cy < fH)) {
                // first tap outside (-1, W) x (-1, H), then first tap with cur < 0
                int lo = 1, hi = kAoTaps;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    const float tf = small_u2f((uint32_t)mid);
                    const float mx = __fadd_rn(pxf, __fmul_rn(dX, tf)), my = __fadd_rn(pyf, __fmul_rn(dY, tf));
                    if (mx > -1.0f && mx < fW && my > -1.0f && my < fH)
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                t_end = lo;
                lo = 1;
                hi = t_end;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    const float tf = small_u2f((uint32_t)mid);
                    const float mx = __fadd_rn(pxf, __fmul_rn(dX, tf)), my = __fadd_rn(pyf, __fmul_rn(dY, tf));
                    if (mx >= 0.0f && my >= 0.0f)
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                t_fast = lo;
            }
        }
        // the padding taps 100, 101 read the pixel itself: elev 0 needs a finite depth
        if (!P.dir_fast[k] || !isfinite(z)) t_fast = 1;
        float best = 0.0f;
        bool ok = true;
        if (t_end > 1) ok = ao_tap_exact(1, pxf, pyf, dX, dY, W, H, P.depth, z, 0.0f, best);
        int t = 2;
        if (ok && t_fast > 2) {
            const int n_groups = t_fast == kAoTaps ? kAoTable / 4 : (t_fast - 2) >> 2;
            const int tiny = P.dir_tiny[k];
            if (tiny) {
                // t*: first tap with |a| above half the gap below the coordinate
                const float cf = fabsf(tiny == 1 ? dX : dY);
                const uint32_t vb = __float_as_uint(tiny == 1 ? pxf : pyf);
                const float h = __uint_as_float(((vb >> 23) - ((vb & 0x7fffffu) ? 24u : 25u)) << 23);
                int lo = 1, hi = kAoTaps;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (__fmul_rn(cf, small_u2f((uint32_t)mid)) > h)
                        hi = mid;
                    else
                        lo = mid + 1;
                }
                const float* pA = p0 + (tiny == 1 ? 1 : -W);
                if (nan_free)
                    ao_fast_groups_nf<true, !kApply>(n_groups, s_off, s_rlo, s_rhi, k, p0, pA, lo, z, pxf, pyf, dX, dY,
                                                     best);
                else
                    ok = ao_fast_groups<true>(n_groups, s_off, s_rlo, s_rhi, k, p0, pA, lo, z, pxf, pyf, dX, dY, best);
            } else if (nan_free) {
                ao_fast_groups_nf<false, !kApply>(n_groups, s_off, s_rlo, s_rhi, k, p0, p0, 0, z, pxf, pyf, dX, dY, best);
            } else {
                ok = ao_fast_groups<false>(n_groups, s_off, s_rlo, s_rhi, k, p0, p0, 0, z, pxf, pyf, dX, dY, best);
            }
            t = 2 + 4 * n_groups;
        }
        for (; ok && t < t_end; t++) ok = ao_tap_exact(t, pxf, pyf, dX, dY, W, H, P.depth, z, best, best);
        if (!ok) {
            nanpix = true;
            break;
        }
        const float ma = best > 0.0f ? atan_f32(best) : 0.0f;
        total = __fadd_rn(total, __fsub_rn(1.57079632679489661923f, ma));  // HalfPi - angle
    }
    const float T = nanpix ? __uint_as_float(0x7fc00000u) : __fdiv_rn(total, 12.5663706143591729539f);
    if (kApply)
        ao_finish(P, i, T);
    else
        P.T[j] = T;
}

// material/ao.go:34-37 for pixel i with total T: the colour the shade kernel
// left (pre-AO, pre-gamma) times float32(Pow(T, 10000)), then gamma.
PR_DEV void ao_finish(const AoParams& P, uint32_t i, float T) {
    const uchar4 c = P.rgba[i];
    if (P.dgb) {
        // float32(Pow(T, 10000)) as a fixed factor of the differentiable radiance (0 for NaN, as the
        // reference's uint8(NaN) darkens the pixel)
        const float fa = isnan(T) ? 0.0f : (T == 1.0f ? 1.0f : powf(T, 10000.0f));
        P.dgb[4 * i].w *= fa;
    }
    uint3 o = ao_scale(T, c.x, c.y, c.z);
    if (P.gamma_on) {
        o.x = P.gamma[o.x];
        o.y = P.gamma[o.y];
        o.z = P.gamma[o.z];
    }
    P.rgba[i] = make_uchar4(o.x, o.y, o.z, c.w);
}

// 4 blocks per SM (up to 64 registers): the march's eight-tap units, two
// at a time, keep sixteen depth loads in flight per thread without spills.
template <bool kApply>
__global__ void __launch_bounds__(kAoThreads, 4) ao_kernel(const __grid_constant__ AoParams P) {
    __shared__ __align__(16) int s_off[8][kAoTable];
    __shared__ __align__(16) float s_rlo[8][kAoTable];
    __shared__ __align__(16) float s_rhi[8][kAoTable];
    const uint32_t n = P.cnt->n_ao;
    if (blockIdx.x * blockDim.x >= n) return;  // whole block: no pixel of the list
    ao_tables(P, s_off, s_rlo, s_rhi);
    __syncthreads();
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        ao_one<kApply>(P, j, s_off, s_rlo, s_rhi);
}

// The colour scaling of every listed pixel from its stored total.
__global__ void ao_apply_kernel(const __grid_constant__ AoParams P) {
    const uint32_t n = P.cnt->n_ao;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        ao_finish(P, P.list[j], P.T[j]);
}

// Triangle.IsValid (geometry/primitive/triangle.go:63-80) of every input
// triangle, once per scene upload: it depends on model-space positions only.
__global__ void tri_flags_kernel(const float4* pos, uint32_t n, uint8_t* flags, const int32_t* mat,
                                 const uint32_t* obj_first, const uint32_t* blk_obj, const int32_t* obj_matbase,
                                 uint32_t n_objects, const pr_material* mats, uint32_t n_mats) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    uint8_t f = tri_is_valid(ld4(pos[3 * t]), ld4(pos[3 * t + 1]), ld4(pos[3 * t + 2])) ? kTriValid : 0;
    // the flat material of the triangle's fragments (MaterialID plus its geometry's base) has AO
    int m = mat[t];
    if (m >= 0) {
        uint32_t o = blk_obj[t >> 7];
        while (o + 1 < n_objects && obj_first[o + 1] <= t) o++;
        m += obj_matbase[o];
        if (m >= 0 && (uint32_t)m < n_mats && (mats[m].flags & PR_MAT_AO)) f |= kTriAO;
    }
    flags[t] = f;
}

// ---------------------------------------------------------------- batches

// The job owning launch block (or item) b: the largest j with start[j] <= b.
PR_DEV int job_of(const uint32_t* start, int n_jobs, uint32_t b) {
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(128) setup_shadow_batch_kernel(const SetupParams* jobs, const uint32_t* blk, int n_jobs) {
    __shared__ ObjCache C;
    const int j = job_of(blk, n_jobs, blockIdx.x);
    const uint32_t t0 = (blockIdx.x - blk[j]) * blockDim.x;
    obj_cache_fill(jobs[j], t0, C);
    setup_shadow_one(jobs[j], &C, t0 + threadIdx.x);
}
__global__ void __launch_bounds__(128) setup_main_batch_kernel(const SetupParams* jobs, const uint32_t* blk, int n_jobs) {
    __shared__ ObjCache C;
    const int j = job_of(blk, n_jobs, blockIdx.x);
    const uint32_t t0 = (blockIdx.x - blk[j]) * blockDim.x;
    obj_cache_fill(jobs[j], t0, C);
    setup_main_one(jobs[j], &C, t0 + threadIdx.x, jobs[j].clip_list);
}
__global__ void __launch_bounds__(128) clip_batch_kernel(const SetupParams* jobs, const uint32_t* blk, int n_jobs) {
    const int j = job_of(blk, n_jobs, blockIdx.x);
    const SetupParams& P = jobs[j];
    const uint32_t n = P.cnt->n_clipped;
    const uint32_t b0 = (blockIdx.x - blk[j]) * blockDim.x;
    if (b0 >= n) return;  // whole block idle
    clip_one(P, P.clip_list, b0 + threadIdx.x, n);
}

// items[j] = warp batches before pass j (one block; a chained scan in
// chunks of its 1024 threads).
__global__ void __launch_bounds__(1024) batch_scan_kernel(const RasterParams* jobs, int n_jobs, uint32_t* items,
                                                          uint32_t* queue, int fixup) {
    __shared__ uint32_t s[1024];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) {
        carry = 0;
        *queue = 0;
    }
    __syncthreads();
    for (int base = 0; base < n_jobs; base += blockDim.x) {
        const int j = base + threadIdx.x;
        uint32_t v = 0;
        if (j < n_jobs) {
            const Counters* c = jobs[j].cnt;
            const bool run = !c->overflow && (!fixup || c->nan_flag);
            v = run ? (c->n_tasks + 31u) >> 5 : 0u;
        }
        s[threadIdx.x] = v;
        __syncthreads();
        for (int d = 1; d < (int)blockDim.x; d <<= 1) {
            const uint32_t t = threadIdx.x >= (unsigned)d ? s[threadIdx.x - d] : 0u;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (j < n_jobs) items[j] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += s[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) items[n_jobs] = carry;
}

// Persistent raster over every pass of a batch: each warp takes the next
// (pass, warp batch) item from the global queue.
__global__ void __launch_bounds__(kRasterWarps * 32, 6) raster_batch_kernel(const RasterParams* jobs, const uint32_t* items,
                                                                         int n_jobs, uint32_t* queue) {
    __shared__ RasterWarpSm s_w[kRasterWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t total = items[n_jobs];
    for (;;) {
        uint32_t it = 0;
        if (lane == 0) it = atomicAdd(queue, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= total) break;
        const int j = job_of(items, n_jobs, it);
        const RasterParams& P = jobs[j];
        raster_warp(P, P.tasks, (it - items[j]) * 32u, P.cnt->n_tasks, s_w[warp], true);
    }
}

__global__ void resolve_batch_kernel(const ResolveParams* jobs, const uint32_t* blk, int n_jobs) {
    const int j = job_of(blk, n_jobs, blockIdx.x);
    const ResolveParams& R = jobs[j];
    resolve_one(R.W, R.H, R.keys, R.nanseq, R.beaten, R.cnt, R.win, R.depth_ao,
                (size_t)(blockIdx.x - blk[j]) * blockDim.x + threadIdx.x);
}

// 256-thread blocks as 32 x 8 pixel tiles, row-major over each view's tiles.
__global__ void __launch_bounds__(256) shade_batch_kernel(const ShadeParams* views, const uint32_t* blk, int n_views) {
    const int v = job_of(blk, n_views, blockIdx.x);
    const ShadeParams& P = views[v];
    const uint32_t b = blockIdx.x - blk[v], tiles_x = (uint32_t)(P.W + 31) / 32u;
    const uint32_t ty = b / tiles_x, tx = b - ty * tiles_x;
    const int x = (int)(tx * 32u + (threadIdx.x & 31u)), r = (int)(ty * 8u + (threadIdx.x >> 5));
    const bool pending = shade_one<false>(P, x, r);  // batches carry no image textures
    if (P.ao_list) ao_append_tile(P, pending, (uint32_t)r * (uint32_t)P.W + (uint32_t)x);
}

// Persistent AO over every view's list, in chunks of one block taken from
// per-view counters; tap tables rebuilt when the frame size changes.
__global__ void __launch_bounds__(kAoThreads) ao_batch_kernel(const AoParams* views, int n_views,
                                                                uint32_t* chunk_ctr) {
    __shared__ __align__(16) int s_off[8][kAoTable];
    __shared__ __align__(16) float s_rlo[8][kAoTable];
    __shared__ __align__(16) float s_rhi[8][kAoTable];
    __shared__ uint32_t s_chunk;
    int tab_w = -1, tab_dirs = -1;
    float tab_h = -1.0f;
    for (int v = 0; v < n_views; v++) {
        const AoParams& P = views[v];
        const uint32_t n = P.cnt->n_ao;
        if (n == 0) continue;
        if (P.W != tab_w || P.ao_half_ulp != tab_h || P.n_dirs != tab_dirs) {
            __syncthreads();
            ao_tables(P, s_off, s_rlo, s_rhi);
            __syncthreads();
            tab_w = P.W;
            tab_h = P.ao_half_ulp;
            tab_dirs = P.n_dirs;
        }
        for (;;) {
            if (threadIdx.x == 0) s_chunk = atomicAdd(&chunk_ctr[v], 1u);
            __syncthreads();
            const uint32_t c = s_chunk;
            __syncthreads();
            if (c * blockDim.x >= n) break;
            const uint32_t j = c * blockDim.x + threadIdx.x;
            if (j < n) ao_one<true>(P, j, s_off, s_rlo, s_rhi);
        }
    }
}

__global__ void pow_probe_kernel(const float* x, const float* y, float* fast, float* ref, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fast[i] = go_pow_f32(x[i], y[i]);
    ref[i] = __double2float_rn(go_pow((double)x[i], (double)y[i]));
}

__global__ void ao_probe_kernel(const float* x, float* atan_fast, float* atan_ref, const float* T, const uchar4* col,
                                uchar4* o_fast, uchar4* o_ref, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atan_fast[i] = atan_f32(x[i]);
    atan_ref[i] = __double2float_rn(go_atan((double)x[i]));
    const uchar4 c = col[i];
    const uint3 a = ao_scale(T[i], c.x, c.y, c.z);
    o_fast[i] = make_uchar4(a.x, a.y, a.z, c.w);
    const float P = __double2float_rn(go_pow((double)T[i], 10000.0));
    o_ref[i] = make_uchar4(go_f2u8(__fmul_rn(P, small_u2f(c.x))), go_f2u8(__fmul_rn(P, small_u2f(c.y))),
                           go_f2u8(__fmul_rn(P, small_u2f(c.z))), c.w);
}

__global__ void fma_probe_kernel(const float* a, const float* b, const float* c, float* out, float* out_ref, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = fma64f(a[i], b[i], c[i]);
    out_ref[i] = fma64f_slow(a[i], b[i], c[i]);
}

int check(cudaError_t e) { return e == cudaSuccess ? 0 : (int)e; }

}  // namespace

int launch_setup_main_only(const SetupParams& p, uint32_t* clip_list, void* stream) {
    if (p.n_tris == 0) return 0;
    setup_main_kernel<<<(p.n_tris + 127) / 128, 128, 0, (cudaStream_t)stream>>>(p, clip_list);
    return check(cudaGetLastError());
}
int launch_resolve_listing(int W, int H, const unsigned long long* keys, uint32_t* nanseq, uint32_t* beaten,
                           Counters* cnt, uint32_t* win, float* depth_ao, const uint32_t* first_rec,
                           uint32_t* attr_state, uint32_t* vis, const uint8_t* tri_flags, uint32_t* ao_list,
                           void* stream) {
    if (W <= 0 || H <= 0) return 0;
    const dim3 blk(32, 8), grd((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8));
    resolve_listing_kernel<<<grd, blk, 0, (cudaStream_t)stream>>>(W, H, keys, nanseq, beaten, cnt, win, depth_ao,
                                                                 first_rec, attr_state, vis, tri_flags, ao_list);
    return check(cudaGetLastError());
}
int launch_attr(const SetupParams& p, const uint32_t* vis, void* stream) {
    attr_kernel<<<(unsigned)sm_count() * 8u, 128, 0, (cudaStream_t)stream>>>(p, vis);
    return check(cudaGetLastError());
}
int launch_obj_trans(const PassMats& pm, int n_pass, const float* obj_model, uint32_t n_objects, float* out,
                     void* stream) {
    const size_t n = (size_t)n_pass * n_objects * 16;
    if (n == 0) return 0;
    obj_trans_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(pm, n_pass, obj_model, n_objects, out);
    return check(cudaGetLastError());
}
int launch_clip(const SetupParams& p, const uint32_t* clip_list, void* stream) {
    if (p.n_tris == 0) return 0;
    // the list's length is known only on the device: a few blocks per SM stride over it
    const unsigned nb = std::min((p.n_tris + 15) / 16, (unsigned)sm_count() * 4u);
    clip_kernel<<<nb, 128, 0, (cudaStream_t)stream>>>(p, clip_list);
    return check(cudaGetLastError());
}
int launch_setup_shadow(const SetupParams& p, void* stream) {
    if (p.n_tris == 0) return 0;
    unsigned nb = (p.n_tris + 127) / 128;
    setup_shadow_kernel<<<nb, 128, 0, (cudaStream_t)stream>>>(p);
    return check(cudaGetLastError());
}
int launch_raster(const RasterParams& p, int n_blocks, void* stream) {
    raster_kernel<<<n_blocks, kRasterWarps * 32, 0, (cudaStream_t)stream>>>(p);
    return check(cudaGetLastError());
}
int launch_shadow_fixup_reset(int W, int H, const uint32_t* lastnan, uint32_t* smap, const Counters* cnt,
                              void* stream) {
    size_t n = (size_t)W * H;
    const unsigned nb = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)sm_count() * 8);
    shadow_fixup_reset_kernel<<<std::max(nb, 1u), 256, 0, (cudaStream_t)stream>>>(n, lastnan, smap, cnt);
    return check(cudaGetLastError());
}
int launch_nan_cleanup(size_t n, uint32_t* a, uint32_t va, uint32_t* b, uint32_t vb, const Counters* cnt,
                       void* stream) {
    const unsigned nb = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)sm_count() * 8);
    nan_cleanup_kernel<<<std::max(nb, 1u), 256, 0, (cudaStream_t)stream>>>(n, a, va, b, vb, cnt);
    return check(cudaGetLastError());
}
int launch_shade(const ShadeParams& p, void* stream) {
    dim3 blk(32, 8);
    dim3 grd((p.W + 31) / 32, (p.H + 7) / 8);
    if (p.mat_tex)
        shade_kernel<true><<<grd, blk, 0, (cudaStream_t)stream>>>(p);
    else
        shade_kernel<false><<<grd, blk, 0, (cudaStream_t)stream>>>(p);
    return check(cudaGetLastError());
}
int launch_tri_flags(const float4* pos, uint32_t n, uint8_t* flags, const int32_t* mat, const uint32_t* obj_first,
                     const uint32_t* blk_obj, const int32_t* obj_matbase, uint32_t n_objects, const pr_material* mats,
                     uint32_t n_mats, void* stream) {
    if (n == 0) return 0;
    tri_flags_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(pos, n, flags, mat, obj_first, blk_obj,
                                                                          obj_matbase, n_objects, mats, n_mats);
    return check(cudaGetLastError());
}
int launch_setup_shadow_batch(const SetupParams* jobs, const uint32_t* blk, int n_jobs, uint32_t n_blocks, void* stream) {
    if (n_blocks == 0) return 0;
    setup_shadow_batch_kernel<<<n_blocks, 128, 0, (cudaStream_t)stream>>>(jobs, blk, n_jobs);
    return check(cudaGetLastError());
}
int launch_setup_main_batch(const SetupParams* jobs, const uint32_t* blk, int n_jobs, uint32_t n_blocks, void* stream) {
    if (n_blocks == 0) return 0;
    setup_main_batch_kernel<<<n_blocks, 128, 0, (cudaStream_t)stream>>>(jobs, blk, n_jobs);
    return check(cudaGetLastError());
}
int launch_clip_batch(const SetupParams* jobs, const uint32_t* blk, int n_jobs, uint32_t n_blocks, void* stream) {
    if (n_blocks == 0) return 0;
    clip_batch_kernel<<<n_blocks, 128, 0, (cudaStream_t)stream>>>(jobs, blk, n_jobs);
    return check(cudaGetLastError());
}
int launch_batch_scan(const RasterParams* jobs, int n_jobs, uint32_t* items, uint32_t* queue, int fixup, void* stream) {
    batch_scan_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(jobs, n_jobs, items, queue, fixup);
    return check(cudaGetLastError());
}
int launch_raster_batch(const RasterParams* jobs, const uint32_t* items, int n_jobs, uint32_t* queue, int n_blocks,
                        void* stream) {
    raster_batch_kernel<<<n_blocks, kRasterWarps * 32, 0, (cudaStream_t)stream>>>(jobs, items, n_jobs, queue);
    return check(cudaGetLastError());
}
int launch_resolve_batch(const ResolveParams* jobs, const uint32_t* blk, int n_jobs, uint32_t n_blocks, void* stream) {
    if (n_blocks == 0) return 0;
    resolve_batch_kernel<<<n_blocks, 256, 0, (cudaStream_t)stream>>>(jobs, blk, n_jobs);
    return check(cudaGetLastError());
}
int launch_shade_batch(const ShadeParams* views, const uint32_t* blk, int n_views, uint32_t n_blocks, void* stream) {
    if (n_blocks == 0) return 0;
    shade_batch_kernel<<<n_blocks, 256, 0, (cudaStream_t)stream>>>(views, blk, n_views);
    return check(cudaGetLastError());
}
int launch_ao_batch(const AoParams* views, int n_views, uint32_t* chunk_ctr, int n_blocks, void* stream) {
    ao_batch_kernel<<<n_blocks, kAoThreads, 0, (cudaStream_t)stream>>>(views, n_views, chunk_ctr);
    return check(cudaGetLastError());
}
// ---------------------------------------------------------------- MSAA resize

constexpr int kMaxMsaa = 16;

// createWeights8 (internal/imageutil/resize.go:161-181) for output index y:
// the linear kernel's taps as int16 (x256, truncated) and the first input
// index, in the reference's float32 order. len <= 2 * kMaxMsaa.
PR_DEV int resize_taps(int y, float scale, float factor, int len, int16_t* coeff) {
    float interp = __fsub_rn(__fmul_rn(scale, __fadd_rn((float)y, 0.5f)), 0.5f);
    const int start = (int)interp - len / 2 + 1;  // int(interpX) truncates
    interp = __fsub_rn(interp, (float)start);
    for (int i = 0; i < len; i++) {
        const float in = fabsf(__fmul_rn(__fsub_rn(interp, (float)i), factor));
        const float k = in <= 1.0f ? __fsub_rn(1.0f, in) : 0.0f;  // linear()
        coeff[i] = (int16_t)(int)__fmul_rn(k, 256.0f);
    }
    return start;
}

// resizeRGBA's edge rule (resize.go:98-105): inside [0, max) as is, at or
// past max -> max, negative -> 0.
PR_DEV int resize_clamp(int i, int max) { return (unsigned)i < (unsigned)max ? i : (i >= max ? max : 0); }

PR_DEV uint8_t resize_div(int32_t acc, int32_t sum) {
    const int32_t v = sum != 0 ? acc / sum : 0;
    return (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
}

// imageutil.Resize's two passes for one output pixel: the horizontal pass
// (into the reference's transposed uint8 temporary) for every input row the
// vertical taps reach, then the vertical pass over those values.
__global__ void msaa_resize_kernel(const uchar4* __restrict__ in, int in_w, int in_h, uchar4* __restrict__ out, int w,
                                   int h) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    // calcFactors, then createWeights8's filterLength and filterFactor
    const float sx = __fdiv_rn((float)in_w, (float)w), sy = __fdiv_rn((float)in_h, (float)h);
    const int lx = min(2 * max((int)ceilf(sx), 1), 2 * kMaxMsaa), ly = min(2 * max((int)ceilf(sy), 1), 2 * kMaxMsaa);
    const float fx = fminf(__fdiv_rn(1.0f, sx), 1.0f), fy = fminf(__fdiv_rn(1.0f, sy), 1.0f);
    int16_t cx[2 * kMaxMsaa], cy[2 * kMaxMsaa];
    const int x0 = resize_taps(x, sx, fx, lx, cx);
    const int y0 = resize_taps(y, sy, fy, ly, cy);
    int32_t acc[4] = {0, 0, 0, 0}, sum_y = 0;
    for (int j = 0; j < ly; j++) {
        if (cy[j] == 0) continue;
        const uchar4* row = in + (size_t)resize_clamp(y0 + j, in_h - 1) * in_w;
        int32_t t[4] = {0, 0, 0, 0}, sum_x = 0;
        for (int i = 0; i < lx; i++) {
            if (cx[i] == 0) continue;
            const uchar4 p = row[resize_clamp(x0 + i, in_w - 1)];
            t[0] += cx[i] * (int32_t)p.x;
            t[1] += cx[i] * (int32_t)p.y;
            t[2] += cx[i] * (int32_t)p.z;
            t[3] += cx[i] * (int32_t)p.w;
            sum_x += cx[i];
        }
        for (int k = 0; k < 4; k++) acc[k] += cy[j] * (int32_t)resize_div(t[k], sum_x);
        sum_y += cy[j];
    }
    out[(size_t)y * w + x] = make_uchar4(resize_div(acc[0], sum_y), resize_div(acc[1], sum_y), resize_div(acc[2], sum_y),
                                         resize_div(acc[3], sum_y));
}

int launch_msaa_resize(const uchar4* in, int in_w, int in_h, uchar4* out, int w, int h, void* stream) {
    if (w <= 0 || h <= 0 || in_w < w || in_h < h || in_w > w * kMaxMsaa || in_h > h * kMaxMsaa) return -1;
    const dim3 block(32, 8), grid((unsigned)((w + 31) / 32), (unsigned)((h + 7) / 8));
    msaa_resize_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(in, in_w, in_h, out, w, h);
    return check(cudaGetLastError());
}

int launch_ao_T(const AoParams& p, void* stream) {
    // One pixel per thread for the largest possible list (every pixel): the
    // block scheduler balances the uneven per-pixel work; blocks past the
    // list's length exit at once.
    const size_t n = (size_t)p.W * p.H;
    if (n == 0) return 0;
    ao_kernel<false><<<(unsigned)((n + kAoThreads - 1) / kAoThreads), kAoThreads, 0, (cudaStream_t)stream>>>(p);
    return check(cudaGetLastError());
}
int launch_ao_apply(const AoParams& p, int n_blocks, void* stream) {
    ao_apply_kernel<<<n_blocks, 256, 0, (cudaStream_t)stream>>>(p);
    return check(cudaGetLastError());
}
int set_ao_tables(const float* cosv, const float* sinv, int n, void* stream) {
    float d[2][8] = {};
    for (int k = 0; k < n && k < 8; k++) {
        d[0][k] = cosv[k];
        d[1][k] = sinv[k];
    }
    cudaError_t e = cudaMemcpyToSymbolAsync(c_ao_dir, d, sizeof(d), 0, cudaMemcpyHostToDevice, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    return check(e);
}
int launch_decode_shadow(const uint32_t* smap, float* out, size_t n, void* stream) {
    if (n == 0) return 0;
    decode_shadow_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(smap, out, n);
    return check(cudaGetLastError());
}
int launch_pow_probe(const float* x, const float* y, float* fast, float* ref, int n, void* stream) {
    if (n <= 0) return 0;
    pow_probe_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(x, y, fast, ref, n);
    return check(cudaGetLastError());
}
int launch_ao_probe(const float* x, float* atan_fast, float* atan_ref, const float* T, const void* col, void* o_fast,
                    void* o_ref, int n, void* stream) {
    if (n <= 0) return 0;
    ao_probe_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(x, atan_fast, atan_ref, T, (const uchar4*)col,
                                                                        (uchar4*)o_fast, (uchar4*)o_ref, n);
    return check(cudaGetLastError());
}
int launch_fma_probe(const float* a, const float* b, const float* c, float* out, float* out_ref, int n, void* stream) {
    if (n <= 0) return 0;
    fma_probe_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(a, b, c, out, out_ref, n);
    return check(cudaGetLastError());
}
int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace prk

namespace prk {

// ===========================================================================
// Allocation-free depth-map raster (pr_depth_map_noalloc).
//
// For callers that must not allocate device memory themselves: a host whose
// device memory is entirely owned by another allocator (a framework's fixed
// caching pool), or a frame loop that cannot afford cudaMalloc/cudaFree
// (cudaFree synchronises the whole device). It runs the shadow-map raster
// (setup_shadow_kernel + raster_kernel, the drawDepth pass) with every byte
// of scratch carved from the fixed array below, which each GPU that loads the
// library keeps until the process exits.
//
// Calls share the array: two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on it and corrupt each other's
// results. Each call clears the parts that must start at zero.
// ===========================================================================

namespace {

constexpr uint32_t kNoAllocMaxTris = 65536;
constexpr uint32_t kNoAllocMaxObjects = 256;
constexpr uint32_t kNoAllocMaxTexels = 1u << 20;  // e.g. 1024 x 1024
constexpr uint32_t kNoAllocMaxTasks = 4u * kNoAllocMaxTris;
constexpr uint32_t kNoAllocTaskShift = 10;  // 1024-pixel tasks: the fixed task table covers large triangles

constexpr size_t kNaCounters = 0;                                   // Counters
constexpr size_t kNaObjFirst = 256;                                 // u32 [max_objects + 1]
constexpr size_t kNaObjModel = kNaObjFirst + 4096;                  // f32 [max_objects][16]
constexpr size_t kNaRecords = kNaObjModel + kNoAllocMaxObjects * 64; // RasterRec [max_tris]
constexpr size_t kNaTasks = kNaRecords + (size_t)kNoAllocMaxTris * sizeof(RasterRec);
constexpr size_t kNaKeys = kNaTasks + (size_t)kNoAllocMaxTasks * sizeof(uint2);
constexpr size_t kNaLastNan = kNaKeys + (size_t)kNoAllocMaxTexels * 4;
constexpr size_t kNaBytes = kNaLastNan + (size_t)kNoAllocMaxTexels * 4;
static_assert(kNaBytes <= (16u << 20), "scratch layout exceeds 16 MiB");

static __device__ __align__(256) unsigned char g_noalloc_scratch[16u << 20];

__global__ void encode_map_kernel(const float* depth, uint32_t* keys, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float d = depth[i];
    keys[i] = isnan(d) ? 0u : fkey(d);  // key 0 stands for NaN (below every value)
}

// Back into the caller's map: a texel whose key the raster changed takes the
// decoded key; the others keep their bits, so a -0 or a NaN payload that no
// fragment replaced stays as it was, as in the reference's map.
__global__ void decode_changed_kernel(const uint32_t* keys, float* depth, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float d = depth[i];
    const uint32_t k0 = isnan(d) ? 0u : fkey(d), k = keys[i];
    if (k != k0) depth[i] = fkey_decode(k);
}

std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {};

}  // namespace

}  // namespace prk

extern "C" int pr_depth_map_noalloc(const pr_depth_map_desc* d) {
    using namespace prk;
    auto err = [](int code, const char* msg) { return set_last_error(code, msg); };
    if (!d) return err(PR_ERR_INVALID_ARG, "pr_depth_map_noalloc: desc is NULL");
    if (d->size < sizeof(pr_depth_map_desc)) return err(PR_ERR_INVALID_ARG, "pr_depth_map_noalloc: desc->size too small");
    if (d->n_tris > kNoAllocMaxTris)
        return err(PR_ERR_INVALID_ARG, "pr_depth_map_noalloc: n_tris exceeds PR_NOALLOC_MAX_TRIS (65536)");
    if (d->n_objects > kNoAllocMaxObjects)
        return err(PR_ERR_INVALID_ARG, "pr_depth_map_noalloc: n_objects exceeds PR_NOALLOC_MAX_OBJECTS (256)");
    if (d->width <= 0 || d->height <= 0 || (uint64_t)d->width * (uint64_t)d->height > kNoAllocMaxTexels)
        return err(PR_ERR_INVALID_ARG, "pr_depth_map_noalloc: width*height must be in 1..PR_NOALLOC_MAX_TEXELS (1048576)");
    if (!d->depth || (d->n_tris > 0 && (!d->pos || d->n_objects == 0)) || (d->n_objects > 0 && !d->objects))
        return err(PR_ERR_INVALID_ARG, "pr_depth_map_noalloc: NULL input or output pointer");
    uint64_t expect = 0;
    for (uint32_t o = 0; o < d->n_objects; o++) {
        if (d->objects[o].first_tri != expect)
            return err(PR_ERR_INVALID_ARG, "pr_depth_map_noalloc: objects must tile the triangles in order");
        expect += d->objects[o].n_tris;
        if (expect > d->n_tris)
            return err(PR_ERR_INVALID_ARG, "pr_depth_map_noalloc: objects do not cover n_tris");
    }
    if (expect != d->n_tris) return err(PR_ERR_INVALID_ARG, "pr_depth_map_noalloc: objects do not cover n_tris");

    // Once per device, with that device current: the device address of the
    // scratch array (its host-side name is not a device address).
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return err(PR_ERR_NO_DEVICE, "pr_depth_map_noalloc: no current CUDA device");
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return err(PR_ERR_CUDA, "pr_depth_map_noalloc: cudaGetSymbolAddress failed");
            g_noalloc_addr[dev] = p;
        }
        base = (unsigned char*)g_noalloc_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)d->stream;
    (void)cudaGetLastError();  // a failure of an earlier runtime call is not this call's
    Counters* cnt = (Counters*)(base + kNaCounters);
    uint32_t* obj_first = (uint32_t*)(base + kNaObjFirst);
    float* obj_model = (float*)(base + kNaObjModel);
    RasterRec* rrec = (RasterRec*)(base + kNaRecords);
    uint2* tasks = (uint2*)(base + kNaTasks);
    uint32_t* keys = (uint32_t*)(base + kNaKeys);
    uint32_t* lastnan = (uint32_t*)(base + kNaLastNan);
    const size_t n = (size_t)d->width * d->height;

    // object tables (host -> the scratch array)
    uint32_t first[kNoAllocMaxObjects + 1];
    float model[kNoAllocMaxObjects * 16];
    for (uint32_t o = 0; o < d->n_objects; o++) {
        first[o] = d->objects[o].first_tri;
        std::memcpy(model + o * 16, d->objects[o].model, 64);
    }
    first[d->n_objects] = d->n_tris;
    cudaError_t e = cudaSuccess;
    if (d->n_objects > 0) {
        e = cudaMemcpyAsync(obj_first, first, (d->n_objects + 1) * 4, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(obj_model, model, d->n_objects * 64, cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(Counters), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(lastnan, 0, n * 4, st);
    if (e != cudaSuccess) return err(PR_ERR_CUDA, "pr_depth_map_noalloc: scratch initialisation failed");
    encode_map_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d->depth, keys, n);

    SetupParams sp{};
    sp.pos = (const float4*)d->pos;
    sp.obj_first = obj_first;
    sp.obj_model = obj_model;
    sp.n_tris = d->n_tris;
    sp.n_objects = d->n_objects;
    sp.W = d->width;
    sp.H = d->height;
    sp.perspective = 0;
    prh::M4 pv = prh::mulm(prh::M4{{d->proj[0], d->proj[1], d->proj[2], d->proj[3], d->proj[4], d->proj[5], d->proj[6],
                                     d->proj[7], d->proj[8], d->proj[9], d->proj[10], d->proj[11], d->proj[12],
                                     d->proj[13], d->proj[14], d->proj[15]}},
                           prh::M4{{d->view[0], d->view[1], d->view[2], d->view[3], d->view[4], d->view[5], d->view[6],
                                     d->view[7], d->view[8], d->view[9], d->view[10], d->view[11], d->view[12],
                                     d->view[13], d->view[14], d->view[15]}});
    prh::M4 vp = prh::viewport((float)d->width, (float)d->height);
    std::memcpy(sp.pv, pv.m, 64);
    std::memcpy(sp.viewport, vp.m, 64);
    sp.rrec = rrec;
    sp.cap_rec = kNoAllocMaxTris;
    sp.tasks = tasks;
    sp.cap_tasks = kNoAllocMaxTasks;
    sp.cnt = cnt;
    sp.task_shift = kNoAllocTaskShift;
    int rc = launch_setup_shadow(sp, st);
    RasterParams rp{};
    rp.task_shift = kNoAllocTaskShift;
    rp.rrec = rrec;
    rp.tasks = tasks;
    rp.cnt = cnt;
    rp.cnt_w = cnt;
    rp.W = d->width;
    rp.H = d->height;
    rp.mode = kShadow;
    rp.smap = keys;
    rp.lastnan = lastnan;
    rp.take = &cnt->take[0];
    if (!rc) rc = launch_raster(rp, sm_count() * 8, st);
    if (!rc) rc = launch_shadow_fixup_reset(d->width, d->height, lastnan, keys, cnt, st);
    rp.mode = kShadowFixup;
    rp.take = &cnt->take[1];
    if (!rc) rc = launch_raster(rp, sm_count() * 8, st);
    if (rc) return err(PR_ERR_CUDA, "pr_depth_map_noalloc: kernel launch failed");
    Counters h{};
    e = cudaMemcpyAsync(&h, cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return err(PR_ERR_CUDA, "pr_depth_map_noalloc: execution failed");
    if (h.overflow)
        return err(PR_ERR_OVERFLOW, "pr_depth_map_noalloc: more raster tasks than PR_NOALLOC_MAX_TASKS (262144); "
                                    "the depth map was left unchanged");
    decode_changed_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(keys, d->depth, n);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return err(PR_ERR_CUDA, "pr_depth_map_noalloc: decode failed");
    return PR_OK;
}
