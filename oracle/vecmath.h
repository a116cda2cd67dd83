// vecmath.h — CPU restatement of polyred's float32 vector/matrix package
// (math/vec2.go, math/vec3.go, math/vec4.go, math/mat4.go, math/interpolate.go)
// and of the primitives the render path uses (geometry/primitive/box.go,
// geometry/primitive/triangle.go, camera/*.go).
//
// TEST INFRASTRUCTURE (oracle): never linked into the product.
#pragma once

#include "gomath.h"

namespace orc {

using gomath::fma32;

struct V2 { float x, y; };
struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };

// ---- Vec4 (math/vec4.go) ----
inline V4 sub4(V4 v, V4 u) { return {v.x - u.x, v.y - u.y, v.z - u.z, v.w - u.w}; }   // :56-58
inline V4 add4(V4 v, V4 u) { return {v.x + u.x, v.y + u.y, v.z + u.z, v.w + u.w}; }   // :51-53
inline V4 scale4(V4 v, float x, float y, float z, float w) { return {v.x * x, v.y * y, v.z * z, v.w * w}; }
// Dot: FMA(v.X,u.X, FMA(v.Y,u.Y, FMA(v.Z,u.Z, v.W*u.W)))   :89-93
inline float dot4(V4 v, V4 u) { return fma32(v.x, u.x, fma32(v.y, u.y, fma32(v.z, u.z, v.w * u.w))); }
// Len: Sqrt(Dot) in float64 -> float32                         :95-98
inline float len4(V4 v) { return (float)std::sqrt((double)dot4(v, v)); }
// Unit: n := 1.0 / Len; scale all four components             :100-104
inline V4 unit4(V4 v) {
    float n = 1.0f / len4(v);
    return {v.x * n, v.y * n, v.z * n, v.w * n};
}
// Apply (M * v) with FMA-through-float64 rows                  :108-117
struct M4 {
    float m[16];  // row-major X00 X01 X02 X03 X10 ...
    float operator()(int i, int j) const { return m[i * 4 + j]; }
};
inline V4 apply4(V4 v, const M4& M) {
    const float* m = M.m;
    float x = fma32(m[0], v.x, fma32(m[1], v.y, fma32(m[2], v.z, m[3] * v.w)));
    float y = fma32(m[4], v.x, fma32(m[5], v.y, fma32(m[6], v.z, m[7] * v.w)));
    float z = fma32(m[8], v.x, fma32(m[9], v.y, fma32(m[10], v.z, m[11] * v.w)));
    float w = fma32(m[12], v.x, fma32(m[13], v.y, fma32(m[14], v.z, m[15] * v.w)));
    return {x, y, z, w};
}
// Cross (w = 0)                                                :130-138
inline V4 cross4(V4 v, V4 u) {
    float x = fma32(v.y, u.z, -v.z * u.y);
    float y = fma32(v.z, u.x, -v.x * u.z);
    float z = fma32(v.x, u.y, -v.y * u.x);
    return {x, y, z, 0};
}
// Pos: divide by W unless W is 0 or 1                           :140-147
inline V4 pos4(V4 v) {
    if (v.w == 1 || v.w == 0) return {v.x, v.y, v.z, 1};
    float invW = 1.0f / v.w;
    return {v.x * invW, v.y * invW, v.z * invW, 1};
}
inline V3 to3(V4 v) { return {v.x, v.y, v.z}; }
inline V2 to2(V4 v) { return {v.x, v.y}; }

// ---- Vec3 (math/vec3.go) ----
inline V3 sub3(V3 v, V3 u) { return {v.x - u.x, v.y - u.y, v.z - u.z}; }
inline V3 add3(V3 v, V3 u) { return {v.x + u.x, v.y + u.y, v.z + u.z}; }
inline float dot3(V3 v, V3 u) { return fma32(v.x, u.x, fma32(v.y, u.y, v.z * u.z)); }  // :78-82
inline float len3(V3 v) { return (float)std::sqrt((double)dot3(v, v)); }
inline V3 unit3(V3 v) {
    float n = 1.0f / len3(v);
    return {v.x * n, v.y * n, v.z * n};
}
inline V3 cross3(V3 v, V3 u) {  // :111-119
    float x = fma32(v.y, u.z, -v.z * u.y);
    float y = fma32(v.z, u.x, -v.x * u.z);
    float z = fma32(v.x, u.y, -v.y * u.x);
    return {x, y, z};
}
// Cross(...).Z only: the component Barycoord and cullBackFace use.
inline float cross_z(float vx, float vy, float ux, float uy) { return fma32(vx, uy, -vy * ux); }

// ---- Mat4 (math/mat4.go) ----
inline M4 mulm(const M4& A, const M4& B) {  // :201-220, plain float32 sums left to right
    const float* m = A.m;
    const float* n = B.m;
    M4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            r.m[i * 4 + j] = m[i * 4 + 0] * n[0 * 4 + j] + m[i * 4 + 1] * n[1 * 4 + j] +
                             m[i * 4 + 2] * n[2 * 4 + j] + m[i * 4 + 3] * n[3 * 4 + j];
    return r;
}
inline V4 mulv(const M4& M, V4 v) {  // :224-230
    const float* m = M.m;
    return {m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * v.w,
            m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * v.w,
            m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * v.w,
            m[12] * v.x + m[13] * v.y + m[14] * v.z + m[15] * v.w};
}
inline M4 transpose(const M4& A) {
    M4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.m[i * 4 + j] = A.m[j * 4 + i];
    return r;
}
// Det: the 24-term expansion in the reference's order (:233-246).
inline float det(const M4& M) {
#define X(i, j) M.m[(i) * 4 + (j)]
    return X(0,0)*X(1,1)*X(2,2)*X(3,3) - X(0,0)*X(1,1)*X(2,3)*X(3,2) +
           X(0,0)*X(1,2)*X(2,3)*X(3,1) - X(0,0)*X(1,2)*X(2,1)*X(3,3) +
           X(0,0)*X(1,3)*X(2,1)*X(3,2) - X(0,0)*X(1,3)*X(2,2)*X(3,1) -
           X(0,1)*X(1,2)*X(2,3)*X(3,0) + X(0,1)*X(1,2)*X(2,0)*X(3,3) -
           X(0,1)*X(1,3)*X(2,0)*X(3,2) + X(0,1)*X(1,3)*X(2,2)*X(3,0) -
           X(0,1)*X(1,0)*X(2,2)*X(3,3) + X(0,1)*X(1,0)*X(2,3)*X(3,2) +
           X(0,2)*X(1,3)*X(2,0)*X(3,1) - X(0,2)*X(1,3)*X(2,1)*X(3,0) +
           X(0,2)*X(1,0)*X(2,1)*X(3,3) - X(0,2)*X(1,0)*X(2,3)*X(3,1) +
           X(0,2)*X(1,1)*X(2,3)*X(3,0) - X(0,2)*X(1,1)*X(2,0)*X(3,3) -
           X(0,3)*X(1,0)*X(2,1)*X(3,2) + X(0,3)*X(1,0)*X(2,2)*X(3,1) -
           X(0,3)*X(1,1)*X(2,2)*X(3,0) + X(0,3)*X(1,1)*X(2,0)*X(3,2) -
           X(0,3)*X(1,2)*X(2,0)*X(3,1) + X(0,3)*X(1,2)*X(2,1)*X(3,0);
#undef X
}
// Inv: adjugate / det with dinv := 1/d (:259-283). Returns false on d == 0
// (the reference panics).
inline bool inv(const M4& M, M4* out) {
    float d = det(M);
    if (d == 0) return false;
    float dinv = 1 / d;
#define m(i, j) M.m[(i) * 4 + (j)]
    M4 n;
    n.m[0]  = dinv * (m(1,2)*m(2,3)*m(3,1) - m(1,3)*m(2,2)*m(3,1) + m(1,3)*m(2,1)*m(3,2) - m(1,1)*m(2,3)*m(3,2) - m(1,2)*m(2,1)*m(3,3) + m(1,1)*m(2,2)*m(3,3));
    n.m[1]  = dinv * (m(0,3)*m(2,2)*m(3,1) - m(0,2)*m(2,3)*m(3,1) - m(0,3)*m(2,1)*m(3,2) + m(0,1)*m(2,3)*m(3,2) + m(0,2)*m(2,1)*m(3,3) - m(0,1)*m(2,2)*m(3,3));
    n.m[2]  = dinv * (m(0,2)*m(1,3)*m(3,1) - m(0,3)*m(1,2)*m(3,1) + m(0,3)*m(1,1)*m(3,2) - m(0,1)*m(1,3)*m(3,2) - m(0,2)*m(1,1)*m(3,3) + m(0,1)*m(1,2)*m(3,3));
    n.m[3]  = dinv * (m(0,3)*m(1,2)*m(2,1) - m(0,2)*m(1,3)*m(2,1) - m(0,3)*m(1,1)*m(2,2) + m(0,1)*m(1,3)*m(2,2) + m(0,2)*m(1,1)*m(2,3) - m(0,1)*m(1,2)*m(2,3));
    n.m[4]  = dinv * (m(1,3)*m(2,2)*m(3,0) - m(1,2)*m(2,3)*m(3,0) - m(1,3)*m(2,0)*m(3,2) + m(1,0)*m(2,3)*m(3,2) + m(1,2)*m(2,0)*m(3,3) - m(1,0)*m(2,2)*m(3,3));
    n.m[5]  = dinv * (m(0,2)*m(2,3)*m(3,0) - m(0,3)*m(2,2)*m(3,0) + m(0,3)*m(2,0)*m(3,2) - m(0,0)*m(2,3)*m(3,2) - m(0,2)*m(2,0)*m(3,3) + m(0,0)*m(2,2)*m(3,3));
    n.m[6]  = dinv * (m(0,3)*m(1,2)*m(3,0) - m(0,2)*m(1,3)*m(3,0) - m(0,3)*m(1,0)*m(3,2) + m(0,0)*m(1,3)*m(3,2) + m(0,2)*m(1,0)*m(3,3) - m(0,0)*m(1,2)*m(3,3));
    n.m[7]  = dinv * (m(0,2)*m(1,3)*m(2,0) - m(0,3)*m(1,2)*m(2,0) + m(0,3)*m(1,0)*m(2,2) - m(0,0)*m(1,3)*m(2,2) - m(0,2)*m(1,0)*m(2,3) + m(0,0)*m(1,2)*m(2,3));
    n.m[8]  = dinv * (m(1,1)*m(2,3)*m(3,0) - m(1,3)*m(2,1)*m(3,0) + m(1,3)*m(2,0)*m(3,1) - m(1,0)*m(2,3)*m(3,1) - m(1,1)*m(2,0)*m(3,3) + m(1,0)*m(2,1)*m(3,3));
    n.m[9]  = dinv * (m(0,3)*m(2,1)*m(3,0) - m(0,1)*m(2,3)*m(3,0) - m(0,3)*m(2,0)*m(3,1) + m(0,0)*m(2,3)*m(3,1) + m(0,1)*m(2,0)*m(3,3) - m(0,0)*m(2,1)*m(3,3));
    n.m[10] = dinv * (m(0,1)*m(1,3)*m(3,0) - m(0,3)*m(1,1)*m(3,0) + m(0,3)*m(1,0)*m(3,1) - m(0,0)*m(1,3)*m(3,1) - m(0,1)*m(1,0)*m(3,3) + m(0,0)*m(1,1)*m(3,3));
    n.m[11] = dinv * (m(0,3)*m(1,1)*m(2,0) - m(0,1)*m(1,3)*m(2,0) - m(0,3)*m(1,0)*m(2,1) + m(0,0)*m(1,3)*m(2,1) + m(0,1)*m(1,0)*m(2,3) - m(0,0)*m(1,1)*m(2,3));
    n.m[12] = dinv * (m(1,2)*m(2,1)*m(3,0) - m(1,1)*m(2,2)*m(3,0) - m(1,2)*m(2,0)*m(3,1) + m(1,0)*m(2,2)*m(3,1) + m(1,1)*m(2,0)*m(3,2) - m(1,0)*m(2,1)*m(3,2));
    n.m[13] = dinv * (m(0,1)*m(2,2)*m(3,0) - m(0,2)*m(2,1)*m(3,0) + m(0,2)*m(2,0)*m(3,1) - m(0,0)*m(2,2)*m(3,1) - m(0,1)*m(2,0)*m(3,2) + m(0,0)*m(2,1)*m(3,2));
    n.m[14] = dinv * (m(0,2)*m(1,1)*m(3,0) - m(0,1)*m(1,2)*m(3,0) - m(0,2)*m(1,0)*m(3,1) + m(0,0)*m(1,2)*m(3,1) + m(0,1)*m(1,0)*m(3,2) - m(0,0)*m(1,1)*m(3,2));
    n.m[15] = dinv * (m(0,1)*m(1,2)*m(2,0) - m(0,2)*m(1,1)*m(2,0) + m(0,2)*m(1,0)*m(2,1) - m(0,0)*m(1,2)*m(2,1) - m(0,1)*m(1,0)*m(2,2) + m(0,0)*m(1,1)*m(2,2));
#undef m
    *out = n;
    return true;
}

// math.ViewportMatrix (math/math.go:270-277)
inline M4 viewport(float w, float h) {
    return M4{{w / 2, 0, 0, w / 2, 0, h / 2, 0, h / 2, 0, 0, 1, 0, 0, 0, 0, 1}};
}

// math.Barycoord (math/interpolate.go:66-78)
inline void barycoord(V2 p, V2 t1, V2 t2, V2 t3, float out[3]) {
    float apx = p.x - t1.x, apy = p.y - t1.y;
    float abx = t2.x - t1.x, aby = t2.y - t1.y;
    float acx = t3.x - t1.x, acy = t3.y - t1.y;
    float bcx = t3.x - t2.x, bcy = t3.y - t2.y;
    float bpx = p.x - t2.x, bpy = p.y - t2.y;
    float Sabc = cross_z(abx, aby, acx, acy);
    float Sabp = cross_z(abx, aby, apx, apy);
    float Sapc = cross_z(apx, apy, acx, acy);
    float Sbcp = cross_z(bcx, bcy, bpx, bpy);
    out[0] = Sbcp / Sabc;
    out[1] = Sapc / Sabc;
    out[2] = Sabp / Sabc;
}

// ---- AABB (geometry/primitive/box.go) ----
struct AABB { V3 mn, mx; };
inline AABB new_aabb(const V3* vs, int n) {  // :15-27
    AABB a{{FLT_MAX, FLT_MAX, FLT_MAX}, {-FLT_MAX, -FLT_MAX, -FLT_MAX}};
    for (int i = 0; i < n; i++) {
        a.mn.x = gomath::pmin(a.mn.x, vs[i].x);
        a.mn.y = gomath::pmin(a.mn.y, vs[i].y);
        a.mn.z = gomath::pmin(a.mn.z, vs[i].z);
        a.mx.x = gomath::pmax(a.mx.x, vs[i].x);
        a.mx.y = gomath::pmax(a.mx.y, vs[i].y);
        a.mx.z = gomath::pmax(a.mx.z, vs[i].z);
    }
    return a;
}
// Intersect, including the reference's Z-vs-Max.Y comparison (:32-41).
inline bool aabb_intersect(const AABB& a, const AABB& b) {
    float minX = gomath::pmax(a.mn.x, b.mn.x);
    float minY = gomath::pmax(a.mn.y, b.mn.y);
    float minZ = gomath::pmax(a.mn.z, b.mn.z);
    float maxX = gomath::pmin(a.mx.x, b.mx.x);
    float maxY = gomath::pmin(a.mx.y, b.mx.y);
    float maxZ = gomath::pmin(a.mx.y, b.mx.z);
    return minX <= maxX && minY <= maxY && minZ <= maxZ;
}
// ApproxEq / ApproxLess (math/math.go:41-49): Abs through float64.
inline bool approx_eq(float a, float b, float eps) { return (float)std::fabs((double)(a - b)) <= eps; }
inline bool approx_less(float a, float b, float eps) {
    return a < b && (float)std::fabs((double)(a - b)) > eps;
}
inline bool aabb_contains(const AABB& a, const V3* vs, int n) {  // :61-75
    const float eps = 1e-7f;
    auto le = [&](float v1, float v2) { return approx_eq(v1, v2, eps) || approx_less(v1, v2, eps); };
    auto lev = [&](V3 v1, V3 v2) { return le(v1.x, v2.x) && le(v1.y, v2.y) && le(v1.z, v2.z); };
    for (int i = 0; i < n; i++)
        if (!(lev(a.mn, vs[i]) && lev(vs[i], a.mx))) return false;
    return true;
}

// Vec4.IsZero (math/vec4.go:63-67)
inline bool is_zero4(V4 v) {
    return approx_eq(v.x, 0, 1e-7f) && approx_eq(v.y, 0, 1e-7f) && approx_eq(v.z, 0, 1e-7f);
}
// Triangle.IsValid (geometry/primitive/triangle.go:63-80)
inline bool tri_is_valid(V4 p1, V4 p2, V4 p3) {
    V4 p1p2 = sub4(p2, p1);
    V4 p1p3 = sub4(p3, p1);
    if (is_zero4(p1p2)) return false;
    if (is_zero4(p1p3)) return false;
    float d = dot4(p1p2, p1p3) / (len4(p1p2) * len4(p1p3));
    return !approx_eq(d, 1, 1e-7f) && !approx_eq(d, -1, 1e-7f);
}

// ---- camera (camera/camera.go:42-53, perspective.go:100-111, orthographic.go:106-119) ----
inline M4 view_matrix(V3 pos, V3 target, V3 up) {
    V3 l = unit3(sub3(target, pos));
    V3 lxu = unit3(cross3(l, up));
    V3 u = unit3(cross3(lxu, l));
    return M4{{lxu.x, lxu.y, lxu.z, -dot3(lxu, pos),
               u.x, u.y, u.z, -dot3(u, pos),
               -l.x, -l.y, -l.z, dot3(l, pos),
               0, 0, 0, 1}};
}
inline M4 perspective_matrix(float fov_deg, float aspect, float n, float f) {
    const float pi = 3.14159265358979323846f;
    float fov = (fov_deg * pi) / 180;
    float t = (float)std::tan((double)(fov / 2));
    return M4{{-1 / (aspect * t), 0, 0, 0,
               0, -1 / t, 0, 0,
               0, 0, (n + f) / (n - f), (2 * n * f) / (n - f),
               0, 0, 1, 0}};
}
inline M4 ortho_matrix(float l, float r, float b, float t, float n, float f) {
    return M4{{2 / (r - l), 0, 0, (l + r) / (l - r),
               0, 2 / (t - b), 0, (b + t) / (b - t),
               0, 0, 2 / (n - f), (f + n) / (f - n),
               0, 0, 0, 1}};
}

}  // namespace orc
