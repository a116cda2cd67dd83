// pr_hostmath.cpp — see pr_hostmath.h. Compiled with -ffp-contract=off.
#include "pr_hostmath.h"

#include <cmath>
#include <cstring>

namespace prh {
namespace {

// Go math.FMA[float32]: one float64 FMA rounded to float32 (math/math.go:265-267).
inline float fma32(float x, float y, float z) { return (float)std::fma((double)x, (double)y, (double)z); }

struct V3 {
    float x, y, z;
};
inline V3 sub3(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float dot3(V3 a, V3 b) { return fma32(a.x, b.x, fma32(a.y, b.y, a.z * b.z)); }
inline V3 unit3(V3 a) {
    float n = 1.0f / (float)std::sqrt((double)dot3(a, a));
    return {a.x * n, a.y * n, a.z * n};
}
inline V3 cross3(V3 v, V3 u) {
    return {fma32(v.y, u.z, -v.z * u.y), fma32(v.z, u.x, -v.x * u.z), fma32(v.x, u.y, -v.y * u.x)};
}

struct V4 {
    float x, y, z, w;
};
inline V4 apply4(V4 v, const M4& M) {
    const float* m = M.m;
    return {fma32(m[0], v.x, fma32(m[1], v.y, fma32(m[2], v.z, m[3] * v.w))),
            fma32(m[4], v.x, fma32(m[5], v.y, fma32(m[6], v.z, m[7] * v.w))),
            fma32(m[8], v.x, fma32(m[9], v.y, fma32(m[10], v.z, m[11] * v.w))),
            fma32(m[12], v.x, fma32(m[13], v.y, fma32(m[14], v.z, m[15] * v.w)))};
}
inline V4 pos4(V4 v) {
    if (v.w == 1 || v.w == 0) return {v.x, v.y, v.z, 1};
    float iw = 1.0f / v.w;
    return {v.x * iw, v.y * iw, v.z * iw, 1};
}

// Go math.Min/Max special cases (+-Inf win over NaN; NaN propagates).
inline double gmin(double x, double y) {
    if (std::isinf(x) && x < 0) return x;
    if (std::isinf(y) && y < 0) return y;
    if (std::isnan(x) || std::isnan(y)) return NAN;
    if (x == 0 && x == y) return std::signbit(x) ? x : y;
    return x < y ? x : y;
}
inline double gmax(double x, double y) {
    if (std::isinf(x) && x > 0) return x;
    if (std::isinf(y) && y > 0) return y;
    if (std::isnan(x) || std::isnan(y)) return NAN;
    if (x == 0 && x == y) return std::signbit(x) ? y : x;
    return x > y ? x : y;
}

}  // namespace

M4 mulm(const M4& a, const M4& b) {
    M4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            r.m[i * 4 + j] = a.m[i * 4 + 0] * b.m[0 * 4 + j] + a.m[i * 4 + 1] * b.m[1 * 4 + j] +
                             a.m[i * 4 + 2] * b.m[2 * 4 + j] + a.m[i * 4 + 3] * b.m[3 * 4 + j];
    return r;
}

M4 transpose(const M4& a) {
    M4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.m[i * 4 + j] = a.m[j * 4 + i];
    return r;
}

bool inv(const M4& M, M4* out) {
    const float* q = M.m;
    auto e = [q](int i, int j) { return q[i * 4 + j]; };
    // Determinant: 24 products summed left to right in the order of
    // math/mat4.go:233-246.
    float d = e(0,0)*e(1,1)*e(2,2)*e(3,3) - e(0,0)*e(1,1)*e(2,3)*e(3,2) +
              e(0,0)*e(1,2)*e(2,3)*e(3,1) - e(0,0)*e(1,2)*e(2,1)*e(3,3) +
              e(0,0)*e(1,3)*e(2,1)*e(3,2) - e(0,0)*e(1,3)*e(2,2)*e(3,1) -
              e(0,1)*e(1,2)*e(2,3)*e(3,0) + e(0,1)*e(1,2)*e(2,0)*e(3,3) -
              e(0,1)*e(1,3)*e(2,0)*e(3,2) + e(0,1)*e(1,3)*e(2,2)*e(3,0) -
              e(0,1)*e(1,0)*e(2,2)*e(3,3) + e(0,1)*e(1,0)*e(2,3)*e(3,2) +
              e(0,2)*e(1,3)*e(2,0)*e(3,1) - e(0,2)*e(1,3)*e(2,1)*e(3,0) +
              e(0,2)*e(1,0)*e(2,1)*e(3,3) - e(0,2)*e(1,0)*e(2,3)*e(3,1) +
              e(0,2)*e(1,1)*e(2,3)*e(3,0) - e(0,2)*e(1,1)*e(2,0)*e(3,3) -
              e(0,3)*e(1,0)*e(2,1)*e(3,2) + e(0,3)*e(1,0)*e(2,2)*e(3,1) -
              e(0,3)*e(1,1)*e(2,2)*e(3,0) + e(0,3)*e(1,1)*e(2,0)*e(3,2) -
              e(0,3)*e(1,2)*e(2,0)*e(3,1) + e(0,3)*e(1,2)*e(2,1)*e(3,0);
    if (d == 0) return false;
    float di = 1 / d;
    float* n = out->m;
    // Cofactors in the order of math/mat4.go:266-281.
    n[0]  = di * (e(1,2)*e(2,3)*e(3,1) - e(1,3)*e(2,2)*e(3,1) + e(1,3)*e(2,1)*e(3,2) - e(1,1)*e(2,3)*e(3,2) - e(1,2)*e(2,1)*e(3,3) + e(1,1)*e(2,2)*e(3,3));
    n[1]  = di * (e(0,3)*e(2,2)*e(3,1) - e(0,2)*e(2,3)*e(3,1) - e(0,3)*e(2,1)*e(3,2) + e(0,1)*e(2,3)*e(3,2) + e(0,2)*e(2,1)*e(3,3) - e(0,1)*e(2,2)*e(3,3));
    n[2]  = di * (e(0,2)*e(1,3)*e(3,1) - e(0,3)*e(1,2)*e(3,1) + e(0,3)*e(1,1)*e(3,2) - e(0,1)*e(1,3)*e(3,2) - e(0,2)*e(1,1)*e(3,3) + e(0,1)*e(1,2)*e(3,3));
    n[3]  = di * (e(0,3)*e(1,2)*e(2,1) - e(0,2)*e(1,3)*e(2,1) - e(0,3)*e(1,1)*e(2,2) + e(0,1)*e(1,3)*e(2,2) + e(0,2)*e(1,1)*e(2,3) - e(0,1)*e(1,2)*e(2,3));
    n[4]  = di * (e(1,3)*e(2,2)*e(3,0) - e(1,2)*e(2,3)*e(3,0) - e(1,3)*e(2,0)*e(3,2) + e(1,0)*e(2,3)*e(3,2) + e(1,2)*e(2,0)*e(3,3) - e(1,0)*e(2,2)*e(3,3));
    n[5]  = di * (e(0,2)*e(2,3)*e(3,0) - e(0,3)*e(2,2)*e(3,0) + e(0,3)*e(2,0)*e(3,2) - e(0,0)*e(2,3)*e(3,2) - e(0,2)*e(2,0)*e(3,3) + e(0,0)*e(2,2)*e(3,3));
    n[6]  = di * (e(0,3)*e(1,2)*e(3,0) - e(0,2)*e(1,3)*e(3,0) - e(0,3)*e(1,0)*e(3,2) + e(0,0)*e(1,3)*e(3,2) + e(0,2)*e(1,0)*e(3,3) - e(0,0)*e(1,2)*e(3,3));
    n[7]  = di * (e(0,2)*e(1,3)*e(2,0) - e(0,3)*e(1,2)*e(2,0) + e(0,3)*e(1,0)*e(2,2) - e(0,0)*e(1,3)*e(2,2) - e(0,2)*e(1,0)*e(2,3) + e(0,0)*e(1,2)*e(2,3));
    n[8]  = di * (e(1,1)*e(2,3)*e(3,0) - e(1,3)*e(2,1)*e(3,0) + e(1,3)*e(2,0)*e(3,1) - e(1,0)*e(2,3)*e(3,1) - e(1,1)*e(2,0)*e(3,3) + e(1,0)*e(2,1)*e(3,3));
    n[9]  = di * (e(0,3)*e(2,1)*e(3,0) - e(0,1)*e(2,3)*e(3,0) - e(0,3)*e(2,0)*e(3,1) + e(0,0)*e(2,3)*e(3,1) + e(0,1)*e(2,0)*e(3,3) - e(0,0)*e(2,1)*e(3,3));
    n[10] = di * (e(0,1)*e(1,3)*e(3,0) - e(0,3)*e(1,1)*e(3,0) + e(0,3)*e(1,0)*e(3,1) - e(0,0)*e(1,3)*e(3,1) - e(0,1)*e(1,0)*e(3,3) + e(0,0)*e(1,1)*e(3,3));
    n[11] = di * (e(0,3)*e(1,1)*e(2,0) - e(0,1)*e(1,3)*e(2,0) - e(0,3)*e(1,0)*e(2,1) + e(0,0)*e(1,3)*e(2,1) + e(0,1)*e(1,0)*e(2,3) - e(0,0)*e(1,1)*e(2,3));
    n[12] = di * (e(1,2)*e(2,1)*e(3,0) - e(1,1)*e(2,2)*e(3,0) - e(1,2)*e(2,0)*e(3,1) + e(1,0)*e(2,2)*e(3,1) + e(1,1)*e(2,0)*e(3,2) - e(1,0)*e(2,1)*e(3,2));
    n[13] = di * (e(0,1)*e(2,2)*e(3,0) - e(0,2)*e(2,1)*e(3,0) + e(0,2)*e(2,0)*e(3,1) - e(0,0)*e(2,2)*e(3,1) - e(0,1)*e(2,0)*e(3,2) + e(0,0)*e(2,1)*e(3,2));
    n[14] = di * (e(0,2)*e(1,1)*e(3,0) - e(0,1)*e(1,2)*e(3,0) - e(0,2)*e(1,0)*e(3,1) + e(0,0)*e(1,2)*e(3,1) + e(0,1)*e(1,0)*e(3,2) - e(0,0)*e(1,1)*e(3,2));
    n[15] = di * (e(0,1)*e(1,2)*e(2,0) - e(0,2)*e(1,1)*e(2,0) + e(0,2)*e(1,0)*e(2,1) - e(0,0)*e(1,2)*e(2,1) - e(0,1)*e(1,0)*e(2,2) + e(0,0)*e(1,1)*e(2,2));
    return true;
}

M4 viewport(float w, float h) { return M4{{w / 2, 0, 0, w / 2, 0, h / 2, 0, h / 2, 0, 0, 1, 0, 0, 0, 0, 1}}; }

M4 view_matrix(const float pos[3], const float target[3], const float up[3]) {
    V3 p{pos[0], pos[1], pos[2]}, t{target[0], target[1], target[2]}, u0{up[0], up[1], up[2]};
    V3 l = unit3(sub3(t, p));
    V3 lxu = unit3(cross3(l, u0));
    V3 u = unit3(cross3(lxu, l));
    return M4{{lxu.x, lxu.y, lxu.z, -dot3(lxu, p), u.x, u.y, u.z, -dot3(u, p), -l.x, -l.y, -l.z, dot3(l, p), 0, 0, 0, 1}};
}

M4 perspective(float fov_deg, float aspect, float n, float f) {
    const float pi = 3.14159265358979323846f;  // math.Pi as float32
    float fov = (fov_deg * pi) / 180;
    float t = (float)std::tan((double)(fov / 2));
    return M4{{-1 / (aspect * t), 0, 0, 0, 0, -1 / t, 0, 0, 0, 0, (n + f) / (n - f), (2 * n * f) / (n - f), 0, 0, 1, 0}};
}

M4 ortho(float l, float r, float b, float t, float n, float f) {
    return M4{{2 / (r - l), 0, 0, (l + r) / (l - r), 0, 2 / (t - b), 0, (b + t) / (b - t), 0, 0, 2 / (n - f),
               (f + n) / (f - n), 0, 0, 0, 1}};
}

bool shadow_camera(const float light_pos[3], const float center[3], const M4& cam_view, const M4& cam_proj,
                   M4* out_view, M4* out_proj) {
    const float up[3] = {0, 1, 0};
    M4 lv = view_matrix(light_pos, center, up);
    M4 vi, pi;
    if (!inv(cam_view, &vi) || !inv(cam_proj, &pi)) return false;
    M4 tm = mulm(mulm(lv, vi), pi);
    // The eight NDC corners in the order of render/shadow.go:47-54.
    const float cs[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {-1, 1, 1}, {-1, -1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, -1}};
    const float fmax32 = 3.40282346638528859812e38f;  // math.MaxFloat32
    float fmnx = fmax32, fmny = fmax32, fmnz = fmax32, fmxx = -fmax32, fmxy = -fmax32, fmxz = -fmax32;
    for (int i = 0; i < 8; i++) {
        V4 v = pos4(apply4(V4{cs[i][0], cs[i][1], cs[i][2], 1}, tm));
        // NewAABB: polyred Min/Max fold through float64 (math/math.go:245-261)
        fmnx = (float)gmin(gmin(1.7976931348623157e308, fmnx), v.x);
        fmny = (float)gmin(gmin(1.7976931348623157e308, fmny), v.y);
        fmnz = (float)gmin(gmin(1.7976931348623157e308, fmnz), v.z);
        fmxx = (float)gmax(gmax(-1.7976931348623157e308, fmxx), v.x);
        fmxy = (float)gmax(gmax(-1.7976931348623157e308, fmxy), v.y);
        fmxz = (float)gmax(gmax(-1.7976931348623157e308, fmxz), v.z);
    }
    *out_view = lv;
    *out_proj = ortho(fmnx, fmxx, fmny, fmxy, fmxz, fmnz - 2);
    return true;
}

void gamma_table(uint8_t out[256]) {
    // lin2sRGBLUT (color/srgb.go:66-75): 1.055*Pow(v, 1/2.4) - 0.055 above the
    // knee; Go's Pow of a fractional exponent below 0.5 is Exp(y*Log(x)).
    double lut[1025];
    for (int i = 0; i < 1024; i++) {
        double v = (double)i / 1024;
        if (v <= 0.0031308)
            lut[i] = v * 12.92;
        else if (v == 0)
            lut[i] = 0;
        else
            lut[i] = 1.055 * std::exp((5.0 / 12.0) * std::log(v)) - 0.055;
    }
    lut[1024] = lut[1023];
    for (int c = 0; c < 256; c++) {
        float v = (float)c / 255.0f;
        float s;
        if (v <= 0) {
            s = 0;
        } else if (v == 1) {
            s = 1;
        } else {
            float i = v * 1024.0f;
            int ifl = (int)i & 1023;
            float v0 = (float)lut[ifl], v1 = (float)lut[ifl + 1];
            i -= (float)ifl;
            s = v0 * (1.0f - i) + v1 * i;
        }
        float q = s * 255.0f + 0.5f;
        out[c] = (uint8_t)((uint32_t)(int32_t)q & 0xffu);
    }
}

// Go math.Pow (math/pow.go) for finite x > 0 and y > 0, the cases the
// sRGB tables use: Exp(yf*Log(x)) for the fractional part, repeated squaring
// of Frexp's mantissa for the integer part, Ldexp at the end.
double go_pow_pos(double x, double y) {
    if (y == 0 || x == 1) return 1;
    if (y == 1) return x;
    if (y == 0.5) return std::sqrt(x);
    double yi;
    double yf = std::modf(y, &yi);
    double a1 = 1.0;
    long long ae = 0;
    if (yf != 0) {
        if (yf > 0.5) {
            yf -= 1;
            yi += 1;
        }
        a1 = std::exp(yf * std::log(x));
    }
    int xe_i;
    double x1 = std::frexp(x, &xe_i);
    long long xe = xe_i;
    for (long long i = (long long)yi; i != 0; i >>= 1) {
        if (xe < -(1 << 12) || (1 << 12) < xe) {
            ae += xe;
            break;
        }
        if ((i & 1) == 1) {
            a1 *= x1;
            ae += xe;
        }
        x1 *= x1;
        xe <<= 1;
        if (x1 < .5) {
            x1 += x1;
            xe--;
        }
    }
    if (ae > 4096) ae = 4096;
    if (ae < -4096) ae = -4096;
    return std::ldexp(a1, (int)ae);
}

void srgb_decode_table(uint8_t out[256]) {
    // sRGB2linLUT (color/srgb.go:60-75): v/12.92 below the knee, else
    // Pow((v+0.055)/1.055, 2.4), in float64 at i/1024
    double lut[1025];
    for (int i = 0; i < 1024; i++) {
        double v = (double)i / 1024;
        lut[i] = v <= 0.04045 ? v / 12.92 : go_pow_pos((v + 0.055) / 1.055, 2.4);
    }
    lut[1024] = lut[1023];
    // LoadImage's byte map (internal/imageutil/image.go:75-101):
    // uint8(FromsRGB2Linear(float32(b)/0xff)*0xff + 0.5) in float32
    for (int c = 0; c < 256; c++) {
        float v = (float)c / 255.0f;
        float s;
        if (v <= 0) {
            s = 0;
        } else if (v >= 1) {
            s = 1;
        } else {
            float i = v * 1024.0f;
            int ifl = (int)i & 1023;
            float v0 = (float)lut[ifl], v1 = (float)lut[ifl + 1];
            i -= (float)ifl;
            s = v0 * (1.0f - i) + v1 * i;
        }
        float q = s * 255.0f + 0.5f;
        out[c] = (uint8_t)((uint32_t)(int32_t)q & 0xffu);
    }
}

void ao_directions(float cosv[8], float sinv[8], int* n) {
    const float limit = (float)(6.28318530717958647692 - 1e-4);  // TwoPi - 1e-4 as float32
    const float step = 0.785398163397448309616f;                  // Pi/4 as float32
    int k = 0;
    for (float a = 0; a < limit && k < 8; a += step) {
        cosv[k] = (float)std::cos((double)a);
        sinv[k] = (float)std::sin((double)a);
        k++;
    }
    *n = k;
}

float ao_classify(const float cosv[8], const float sinv[8], int n, int W, int H, int8_t fast[8], int8_t tiny[8]) {
    // Tap coordinates RN(x + a) stay below M = max(W, H) + 100 < 2^(E+1), where
    // half an ulp is at most 2^(E-24). A component whose a = RN(c t) is, for
    // every t <= 99, an integer or more than that below the next integer never
    // rounds up across an integer: int(RN(x + a)) = x + floor(a) for x >= 0.
    const int M = (W > H ? W : H) + 100;
    int E = 0;
    while ((2 << E) <= M) E++;
    const float h = std::ldexp(1.0f, E - 24);
    for (int k = 0; k < 8; k++) {
        fast[k] = 0;
        tiny[k] = 0;
        if (k >= n) continue;
        const float comp[2] = {cosv[k], sinv[k]};
        bool ok = true;
        int nt = 0;
        for (int a = 0; a < 2; a++) {
            const float c = comp[a];
            if (c < 0.0f && -c * 99.0f < 1.0f) {  // every a_t in (-1, 0)
                tiny[k] = (int8_t)(a + 1);
                nt++;
                continue;
            }
            for (int t = 1; t < 100; t++) {
                const float at = c * (float)t;
                if (at != std::floor(at) && std::ceil(at) - at <= h) ok = false;
            }
        }
        if (nt > 1) ok = false;
        fast[k] = ok ? 1 : 0;
        if (!ok) tiny[k] = 0;
    }
    return h;
}

}  // namespace prh
