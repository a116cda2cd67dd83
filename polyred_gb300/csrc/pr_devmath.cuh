// pr_devmath.cuh — device arithmetic with the reference's exact float32
// semantics. The translation unit is compiled with -fmad=false so that every
// plain a*b+c below stays two IEEE roundings (Go amd64 never fuses); fused
// operations are spelled out with __fmaf_rn.
#pragma once

#include <cstdint>

#define PR_DEV __device__ __forceinline__

namespace prd {

// ---------------------------------------------------------------------------
// float32(fma(float64(a), float64(b), float64(c))): Go's math.FMA[float32]
// (math/math.go:265-267), used by Vec4.Dot/Apply/Cross and Barycoord.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the common case is
// decided in FP32. Let s = a*b + c (exact) and r1 = fmaf(a, b, c) = RN32(s).
//
// (1) The double rounding RN32(RN64(s)) differs from r1 only if RN64(s) is a
//     float32 rounding midpoint m with s != m (a float32 midpoint is a float64
//     number, so RN64 cannot carry s across one). The tie then goes to the
//     neighbour of m with an even significand, while r1 is the neighbour on
//     s's side: a difference needs r1 odd, so that m is r1 +- ulp(r1)/2 and
//     |s - r1| >= ulp(r1)/2 - ulp64(m)/2 >= T (1 - 2^-29), T = ulp(r1)/2.
// (2) The residual e = s - r1 is estimated in FP32: p = RN(ab) and
//     q = ab - p (exact by FMA); (sg, tau) = TwoSum(p, c) (Knuth), so
//     ab + c = sg + tau + q; d = sg - r1 is exact (if tau = 0, r1 = RN(sg + q)
//     with |sg| >= |q| or sg = 0, the Fast2Sum case; if tau != 0, the sum
//     p + c is inexact, so |sg| >= 2^22 ulp(p) >= 2^23 |q| and r1 is within a
//     factor 2 of sg, the Sterbenz case). e' = RN(RN(d + tau) + q) then
//     differs from e by at most 2^-24 (|d + tau| + |e'|) <= 6 * 2^-24 T, the
//     first rounding being exact when tau = 0 (|q| <= 4T when tau != 0).
// (3) Hence |e'| < T (1 - 2^-20) proves r1 is the reference result. The test
//     is an integer compare of bit patterns (T is a power of two; 16 float
//     steps below it are 2^-20 T) and requires r1's exponent field >= 25, so
//     that T and every partial result above are normal enough; an even r1
//     also settles it by (1). What is left (an odd r1 within 2^-20 of a
//     midpoint, tiny or infinite results, NaN) goes to the FP64 unit: on
//     random and pixel-grid data about 1 call in 5 million.
// (Checked against the FP64 expression on 4.8e8 inputs, 6e7 of them true
// double-rounding hazards, with no difference.)
// ---------------------------------------------------------------------------
// Kept out of line: if the compiler predicated this into the fast path, the
// FP64 pipe (2 lanes/clk/SM on GB300) would be occupied on every call.
static __device__ __noinline__ float fma64f_slow(float a, float b, float c) {
    return __double2float_rn(__fma_rn((double)a, (double)b, (double)c));
}

// The certified FP32 result; sets *bad when (3) does not settle it. Callers
// evaluate whole chains this way and redo the chain on the FP64 unit when any
// step is unsettled, so the common path has no call and no per-step branch.
PR_DEV float fma64f_try(float a, float b, float c, bool& bad) {
    const float r1 = __fmaf_rn(a, b, c);
    // a zero first factor (a matrix entry, usually warp-uniform): s = c + (+-0)
    // rounds to c in both precisions; a zero addend (the w terms of direction
    // vectors, usually warp-uniform): the product of two floats is exact in
    // float64, so s = ab + (+-0) is rounded once, to r1, with the same sign
    // of zero
    if (a == 0.0f || c == 0.0f) return r1;
    const float p = __fmul_rn(a, b);
    const float q = __fmaf_rn(a, b, -p);
    const float sg = __fadd_rn(p, c);
    const float bb = __fsub_rn(sg, p);
    const float tau = __fadd_rn(__fsub_rn(p, __fsub_rn(sg, bb)), __fsub_rn(c, bb));
    const float e = __fadd_rn(__fadd_rn(__fsub_rn(sg, r1), tau), q);
    const uint32_t rb = __float_as_uint(r1);
    const int thr = (int)(rb & 0x7f800000u) - ((24 << 23) + 16);
    const bool ok = (int)(__float_as_uint(e) & 0x7fffffffu) < thr ||
                    ((rb & 1u) == 0u && (rb & 0x7f800000u) != 0x7f800000u);
    bad |= !ok;
    return r1;
}

PR_DEV float fma64f(float a, float b, float c) {
    bool bad = false;
    const float r = fma64f_try(a, b, c, bad);
    return __builtin_expect(bad, 0) ? fma64f_slow(a, b, c) : r;
}

// ---- Go conversions and polyred scalar helpers --------------------------

// GB300 executes int<->float conversion instructions on its FP64 pipe (2
// lanes/clk/SM), so the common cases below use exact FP32/integer bit tricks.

// (float)v for 0 <= v < 2^23: 2^23 + v is exact in float32.
PR_DEV float small_u2f(uint32_t v) { return __fsub_rn(__uint_as_float(0x4B000000u | v), 8388608.0f); }

// Truncation toward zero for |v| < 2^23: adding 2^23 with round-toward-zero
// drops the fraction of |v| exactly.
PR_DEV int trunc_small(float v) {
    const float a = fabsf(v);
    const int k = (int)(__float_as_uint(__fadd_rz(a, 8388608.0f)) - 0x4B000000u);
    return v < 0.0f ? -k : k;
}

// Go int(float32) on amd64 (CVTTSS2SQ): NaN / out of range -> INT64_MIN.
PR_DEV long long go_f2i(float x) {
    if (fabsf(x) < 8388608.0f) return (long long)trunc_small(x);
    if (!(x < 9.2233720368547758e18f && x >= -9.2233720368547758e18f)) return (long long)0x8000000000000000ull;
    return (long long)x;
}
// Go uint8(float32) on amd64: via int32 (CVTTSS2SL), low byte.
PR_DEV uint32_t go_f2u8(float x) {
    if (fabsf(x) < 8388608.0f) return (uint32_t)trunc_small(x) & 0xffu;
    if (!(x < 2147483648.0f && x >= -2147483648.0f)) return 0u;
    return ((uint32_t)(int)x) & 0xffu;
}
// polyred math.Round: half away from zero (roundf is exact).
PR_DEV float pround(float x) { return roundf(x); }
PR_DEV float pclamp(float n, float lo, float hi) {
    if (n < lo) return lo;
    if (n > hi) return hi;
    return n;
}
// Go math.Max / math.Min special cases on float32 arguments.
PR_DEV float pmax(float x, float y) {
    if (__float_as_uint(x) == 0x7f800000u || __float_as_uint(y) == 0x7f800000u) return __uint_as_float(0x7f800000u);
    if (isnan(x) || isnan(y)) return __uint_as_float(0x7fc00000u);
    if (x == 0.0f && y == 0.0f) return signbit(x) ? y : x;
    return x > y ? x : y;
}
PR_DEV float pmin(float x, float y) {
    if (__float_as_uint(x) == 0xff800000u || __float_as_uint(y) == 0xff800000u) return __uint_as_float(0xff800000u);
    if (isnan(x) || isnan(y)) return __uint_as_float(0x7fc00000u);
    if (x == 0.0f && y == 0.0f) return signbit(x) ? x : y;
    return x < y ? x : y;
}

// ---- vectors (math/vec4.go) ----------------------------------------------
struct V4 { float x, y, z, w; };

PR_DEV V4 sub4(V4 v, V4 u) { return {__fsub_rn(v.x, u.x), __fsub_rn(v.y, u.y), __fsub_rn(v.z, u.z), __fsub_rn(v.w, u.w)}; }
PR_DEV V4 add4(V4 v, V4 u) { return {__fadd_rn(v.x, u.x), __fadd_rn(v.y, u.y), __fadd_rn(v.z, u.z), __fadd_rn(v.w, u.w)}; }
// Vec4.Dot; the FP64 redo of a chain with an unsettled step is out of line.
static __device__ __noinline__ float dot4_exact(V4 v, V4 u) {
    return fma64f_slow(v.x, u.x, fma64f_slow(v.y, u.y, fma64f_slow(v.z, u.z, __fmul_rn(v.w, u.w))));
}
PR_DEV float dot4(V4 v, V4 u) {
    bool bad = false;
    const float r = fma64f_try(v.x, u.x, fma64f_try(v.y, u.y, fma64f_try(v.z, u.z, __fmul_rn(v.w, u.w), bad), bad), bad);
    return __builtin_expect(bad, 0) ? dot4_exact(v, u) : r;
}
PR_DEV float len4(V4 v) { return __fsqrt_rn(dot4(v, v)); }  // sqrt in f64 then f32 == correctly rounded sqrtf
PR_DEV V4 unit4(V4 v) {
    float n = __fdiv_rn(1.0f, len4(v));
    return {__fmul_rn(v.x, n), __fmul_rn(v.y, n), __fmul_rn(v.z, n), __fmul_rn(v.w, n)};
}
static __device__ __noinline__ V4 cross4_exact(V4 v, V4 u) {
    return {fma64f_slow(v.y, u.z, -__fmul_rn(v.z, u.y)), fma64f_slow(v.z, u.x, -__fmul_rn(v.x, u.z)),
            fma64f_slow(v.x, u.y, -__fmul_rn(v.y, u.x)), 0.0f};
}
PR_DEV V4 cross4(V4 v, V4 u) {
    bool bad = false;
    const V4 r = {fma64f_try(v.y, u.z, -__fmul_rn(v.z, u.y), bad), fma64f_try(v.z, u.x, -__fmul_rn(v.x, u.z), bad),
                  fma64f_try(v.x, u.y, -__fmul_rn(v.y, u.x), bad), 0.0f};
    return __builtin_expect(bad, 0) ? cross4_exact(v, u) : r;
}
PR_DEV V4 pos4(V4 v) {
    if (v.w == 1.0f || v.w == 0.0f) return {v.x, v.y, v.z, 1.0f};
    float iw = __fdiv_rn(1.0f, v.w);
    return {__fmul_rn(v.x, iw), __fmul_rn(v.y, iw), __fmul_rn(v.z, iw), 1.0f};
}
// Vec4.Apply with a row-major matrix m[16]
static __device__ __noinline__ V4 apply4_exact(V4 v, const float* m) {
    return {fma64f_slow(m[0], v.x, fma64f_slow(m[1], v.y, fma64f_slow(m[2], v.z, __fmul_rn(m[3], v.w)))),
            fma64f_slow(m[4], v.x, fma64f_slow(m[5], v.y, fma64f_slow(m[6], v.z, __fmul_rn(m[7], v.w)))),
            fma64f_slow(m[8], v.x, fma64f_slow(m[9], v.y, fma64f_slow(m[10], v.z, __fmul_rn(m[11], v.w)))),
            fma64f_slow(m[12], v.x, fma64f_slow(m[13], v.y, fma64f_slow(m[14], v.z, __fmul_rn(m[15], v.w))))};
}
PR_DEV V4 apply4(V4 v, const float* m) {
    bool bad = false;
    const V4 r = {fma64f_try(m[0], v.x, fma64f_try(m[1], v.y, fma64f_try(m[2], v.z, __fmul_rn(m[3], v.w), bad), bad), bad),
                  fma64f_try(m[4], v.x, fma64f_try(m[5], v.y, fma64f_try(m[6], v.z, __fmul_rn(m[7], v.w), bad), bad), bad),
                  fma64f_try(m[8], v.x, fma64f_try(m[9], v.y, fma64f_try(m[10], v.z, __fmul_rn(m[11], v.w), bad), bad), bad),
                  fma64f_try(m[12], v.x, fma64f_try(m[13], v.y, fma64f_try(m[14], v.z, __fmul_rn(m[15], v.w), bad), bad), bad)};
    return __builtin_expect(bad, 0) ? apply4_exact(v, m) : r;
}
// Mat4.MulV: plain float32 sums left to right
PR_DEV V4 mulv(const float* m, V4 v) {
    return {__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], v.x), __fmul_rn(m[1], v.y)), __fmul_rn(m[2], v.z)), __fmul_rn(m[3], v.w)),
            __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[4], v.x), __fmul_rn(m[5], v.y)), __fmul_rn(m[6], v.z)), __fmul_rn(m[7], v.w)),
            __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[8], v.x), __fmul_rn(m[9], v.y)), __fmul_rn(m[10], v.z)), __fmul_rn(m[11], v.w)),
            __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[12], v.x), __fmul_rn(m[13], v.y)), __fmul_rn(m[14], v.z)), __fmul_rn(m[15], v.w))};
}
// Cross(...).Z of two 2-D vectors (Barycoord, cullBackFace)
PR_DEV float cross_z(float vx, float vy, float ux, float uy) { return fma64f(vx, uy, -__fmul_rn(vy, ux)); }

// math.Barycoord (math/interpolate.go:66-78) given the triangle's Sabc.
PR_DEV void barycoord_s(float px, float py, float x1, float y1, float x2, float y2, float x3, float y3,
                        float sabc, float bc[3]) {
    float apx = __fsub_rn(px, x1), apy = __fsub_rn(py, y1);
    float abx = __fsub_rn(x2, x1), aby = __fsub_rn(y2, y1);
    float acx = __fsub_rn(x3, x1), acy = __fsub_rn(y3, y1);
    float bcx = __fsub_rn(x3, x2), bcy = __fsub_rn(y3, y2);
    float bpx = __fsub_rn(px, x2), bpy = __fsub_rn(py, y2);
    float sabp = cross_z(abx, aby, apx, apy);
    float sapc = cross_z(apx, apy, acx, acy);
    float sbcp = cross_z(bcx, bcy, bpx, bpy);
    bc[0] = __fdiv_rn(sbcp, sabc);
    bc[1] = __fdiv_rn(sapc, sabc);
    bc[2] = __fdiv_rn(sabp, sabc);
}
PR_DEV float sabc_of(float x1, float y1, float x2, float y2, float x3, float y3) {
    return cross_z(__fsub_rn(x2, x1), __fsub_rn(y2, y1), __fsub_rn(x3, x1), __fsub_rn(y3, y1));
}

// Orderable keys: monotone float -> uint32 for non-NaN values, with -0 and +0
// mapped to the same key (the reference's comparisons treat them as equal).
PR_DEV uint32_t fkey(float f) {
    if (f == 0.0f) f = 0.0f;
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
PR_DEV float fkey_decode(uint32_t k) {
    uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(b);
}

// ---- Go math.Pow / math.Atan in float64 (Go 1.26 math/pow.go, atan.go) ----
PR_DEV bool is_odd_int(double x) {
    if (fabs(x) >= 9007199254740992.0) return false;
    double xi;
    double xf = modf(x, &xi);
    if (xf != 0) return false;
    long long i = (long long)xi;
    return (i & 1) == 1;
}
static __device__ __noinline__ double go_pow(double x, double y) {
    if (y == 0 || x == 1) return 1;
    if (y == 1) return x;
    if (isnan(x) || isnan(y)) return __longlong_as_double(0x7ff8000000000000ll);
    if (x == 0) {
        if (y < 0) return (signbit(x) && is_odd_int(y)) ? -__longlong_as_double(0x7ff0000000000000ll)
                                                          : __longlong_as_double(0x7ff0000000000000ll);
        if (y > 0) return (signbit(x) && is_odd_int(y)) ? x : 0.0;
    }
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    if (isinf(y)) {
        if (x == -1) return 1;
        if ((fabs(x) < 1) == (y > 0)) return 0;
        return inf;
    }
    if (isinf(x)) {
        if (x < 0) {
            // Pow(-Inf, y) = Pow(-0, -y)
            double y2 = -y;
            if (y2 < 0) return is_odd_int(y2) ? -inf : inf;
            if (y2 > 0) return is_odd_int(y2) ? -0.0 : 0.0;
            return 1;
        }
        if (y < 0) return 0;
        if (y > 0) return inf;
    }
    if (y == 0.5) return __dsqrt_rn(x);
    if (y == -0.5) return __ddiv_rn(1.0, __dsqrt_rn(x));
    double yi;
    double yf = modf(fabs(y), &yi);
    if (yf != 0 && x < 0) return __longlong_as_double(0x7ff8000000000000ll);
    if (yi >= 9223372036854775808.0) {
        if (x == -1) return 1;
        if ((fabs(x) < 1) == (y > 0)) return 0;
        return inf;
    }
    double a1 = 1.0;
    long long ae = 0;
    if (yf != 0) {
        if (yf > 0.5) {
            yf = __dsub_rn(yf, 1.0);
            yi = __dadd_rn(yi, 1.0);
        }
        a1 = exp(__dmul_rn(yf, log(x)));
    }
    int xe_i;
    double x1 = frexp(x, &xe_i);
    long long xe = xe_i;
    for (long long i = (long long)yi; i != 0; i >>= 1) {
        if (xe < -(1 << 12) || (1 << 12) < xe) {
            ae += xe;
            break;
        }
        if ((i & 1) == 1) {
            a1 = __dmul_rn(a1, x1);
            ae += xe;
        }
        x1 = __dmul_rn(x1, x1);
        xe <<= 1;
        if (x1 < .5) {
            x1 = __dadd_rn(x1, x1);
            xe--;
        }
    }
    if (y < 0) {
        a1 = __ddiv_rn(1.0, a1);
        ae = -ae;
    }
    if (ae > 4096) ae = 4096;
    if (ae < -4096) ae = -4096;
    return ldexp(a1, (int)ae);
}

PR_DEV double go_xatan(double x) {
    const double P0 = -8.750608600031904122785e-01, P1 = -1.615753718733365076637e+01,
                 P2 = -7.500855792314704667340e+01, P3 = -1.228866684490136173410e+02,
                 P4 = -6.485021904942025371773e+01;
    const double Q0 = +2.485846490142306297962e+01, Q1 = +1.650270098316988542046e+02,
                 Q2 = +4.328810604912902668951e+02, Q3 = +4.853903996359136964868e+02,
                 Q4 = +1.945506571482613964425e+02;
    double z = __dmul_rn(x, x);
    double num = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(P0, z), P1), z), P2), z), P3), z), P4);
    double den = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(z, Q0), z), Q1), z), Q2), z), Q3), z), Q4);
    z = __ddiv_rn(__dmul_rn(z, num), den);
    return __dadd_rn(__dmul_rn(x, z), x);
}
PR_DEV double go_satan(double x) {
    const double Morebits = 6.123233995736765886130e-17;
    const double Tan3pio8 = 2.41421356237309504880;
    const double PiOver2 = 1.57079632679489661923132169163975144;
    const double PiOver4 = 0.785398163397448309615660845819875721;
    if (x <= 0.66) return go_xatan(x);
    if (x > Tan3pio8) return __dadd_rn(__dsub_rn(PiOver2, go_xatan(__ddiv_rn(1.0, x))), Morebits);
    return __dadd_rn(__dadd_rn(PiOver4, go_xatan(__ddiv_rn(__dsub_rn(x, 1.0), __dadd_rn(x, 1.0)))), 0.5 * Morebits);
}
static __device__ __noinline__ double go_atan(double x) {
    if (x == 0) return x;
    if (x > 0) return go_satan(x);
    return -go_satan(-x);
}

// float32(Go math.Atan(x)) for a positive normal float32 x.
//  * Small x: Atan(x) = x - x^3/3 + O(x^5) lies below x by less than half the
//    gap to the float32 below x whenever x^3 <= that gap (a 1.5x margin over
//    x^3/3, far above the float64 error of Go's Cephes evaluation), so it
//    rounds back to x.
//  * x <= 1/16: Atan(x) = x - c with c = x^3/3 - x^5/5 + ... + x^11/11
//    (truncation below 3e-16 x). c is evaluated in float32 with relative error
//    below 1e-6; s = RN(x - c) and the exact residual e = (x - c) - s
//    (Fast2Sum) place Atan(x), and Go's float64 value of it (relative error
//    far below 1e-14), within |e| + delta of s, delta = 1e-6 c + 1e-14 x. When
//    that interval lies strictly inside the rounding interval of s, the
//    float32 rounding of Go's result is s.
//  * Otherwise, the float64 algorithm.
PR_DEV float atan_f32(float x) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t e = b >> 23;
    if (e >= 1u && e < 255u) {
        // gap to the next float32 below x: 2^(E-23), or 2^(E-24) at a power of two
        const uint32_t ge = (b & 0x7fffffu) ? e - 23u : e - 24u;
        if ((int)ge >= 1) {
            const float gap = __uint_as_float(ge << 23);
            if (__fmul_rn(__fmul_rn(x, x), x) <= __fmul_rn(gap, 0.999f)) return x;
        }
        if (x <= 0.0625f && e >= 40u) {
            const float x2 = __fmul_rn(x, x);
            float p = __fsub_rn(0.111111111f, __fmul_rn(x2, 0.0909090909f));
            p = __fsub_rn(0.142857143f, __fmul_rn(x2, p));
            p = __fsub_rn(0.2f, __fmul_rn(x2, p));
            p = __fsub_rn(0.333333333f, __fmul_rn(x2, p));
            const float c = __fmul_rn(__fmul_rn(x, x2), p);
            const float s = __fsub_rn(x, c);
            const float z = __fsub_rn(s, x);
            const float err = __fsub_rn(-c, z);  // (x - c) - s exactly (Fast2Sum, |c| < |x|)
            const float delta = __fadd_ru(__fmul_ru(c, 1e-6f), __fmul_ru(x, 1e-14f));
            const uint32_t bs = __float_as_uint(s);
            const uint32_t es = bs >> 23;
            const float hu = __uint_as_float((es - 24u) << 23);                                // half ulp above s
            const float hd = (bs & 0x7fffffu) ? hu : __uint_as_float((es - 25u) << 23);      // half gap below s
            if (__fadd_ru(err, delta) < hu && __fsub_rd(err, delta) > -hd) return s;
        }
    }
    return __double2float_rn(go_atan((double)x));
}

// float32(Go math.Pow(float64(x), float64(y))) (math/pow.go), as the
// specular term of shader/blinn_cpu.go:86 needs it. For 0 < x < 1 and an
// integer 2 <= y <= 4096, Go runs binary exponentiation on the frexp
// mantissa of x; that runs here on float32 pairs (hi + lo, products by
// fmaf, each within 2^-45 relative), with the binary exponent kept apart.
// Squaring doubles a relative error, so X^(2^k) is within (2^k - 1) 2^-45
// and the product within y 2^-45 of x^y; Go's float64 result is within
// y 2^-53 of it. When the interval y 2^-44 around the pair lies strictly
// inside one float32 rounding interval (normal or subnormal), the rounding
// is decided; otherwise, and for other arguments, the float64 algorithm
// runs. Go's early exit for |exponent| > 4096 only occurs for results far
// below the float32 range, which round to 0 here as there.
struct DF { float hi, lo; };
PR_DEV DF df_mul(DF a, DF b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const float h = __fadd_rn(p, e);
    return {h, __fsub_rn(e, __fsub_rn(h, p))};
}
PR_DEV float go_pow_f32(float x, float y) {
    const bool yint = y >= 0.0f && y <= 4096.0f && __fsub_rn(__fadd_rz(y, 8388608.0f), 8388608.0f) == y;
    if (yint && x > 0.0f && x < 1.0f && y >= 2.0f && x >= 0x1p-60f) {
        uint32_t n = __float_as_uint(__fadd_rz(y, 8388608.0f)) - 0x4B000000u;
        const float ny = y;
        // frexp: x = m 2^xe, m in [0.5, 1)
        const uint32_t xb = __float_as_uint(x);
        int xe = (int)(xb >> 23) - 126;
        DF X = {__uint_as_float((xb & 0x807fffffu) | 0x3f000000u), 0.0f};
        DF a = {1.0f, 0.0f};
        int ae = 0;
        for (; n != 0; n >>= 1) {
            if (n & 1u) {
                a = df_mul(a, X);
                ae += xe;
                if (a.hi < 0.5f) {
                    a.hi = __fmul_rn(a.hi, 2.0f);
                    a.lo = __fmul_rn(a.lo, 2.0f);
                    ae--;
                }
            }
            if (n == 1u) break;
            X = df_mul(X, X);
            xe <<= 1;
            if (X.hi < 0.5f) {
                X.hi = __fmul_rn(X.hi, 2.0f);
                X.lo = __fmul_rn(X.lo, 2.0f);
                xe--;
            }
        }
        // value (a.hi + a.lo) 2^ae with a.hi in [0.5, 1], |a.lo| <= ulp(a.hi) / 2
        const float tol = __fmul_ru(__fmul_ru(a.hi, ny), 0x1p-44f);
        if (ae >= -125) {
            // normal: a.hi 2^ae is a float32; it is the rounding if the error interval stays inside
            const uint32_t hb = __float_as_uint(a.hi);
            const float hu = __uint_as_float(((hb >> 23) - 24u) << 23);                             // half ulp above
            const float hd = (hb & 0x7fffffu) ? hu : __uint_as_float(((hb >> 23) - 25u) << 23);     // half gap below
            if (__fadd_ru(a.lo, tol) < hu && __fsub_rd(a.lo, tol) > -hd)
                return __uint_as_float((uint32_t)((int)(hb >> 23) + ae) << 23 | (hb & 0x7fffffu));
        } else if (ae >= -149 - 24) {
            // subnormal or zero: q = value / 2^-149 (< 2^23), rounded to an integer
            const float sc = __uint_as_float((uint32_t)(ae + 149 + 127) << 23);
            const float qh = __fmul_rn(a.hi, sc), ql = __fmul_rn(a.lo, sc), qt = __fmul_ru(tol, sc);
            const float qi = __fsub_rn(__fadd_rn(qh, 8388608.0f), 8388608.0f);  // RN(qh), qh < 2^23
            const float r = __fadd_rn(__fsub_rn(qh, qi), ql);                    // qh - qi exact
            if (__fadd_ru(fabsf(r), qt) < 0.5f) return __uint_as_float(__float_as_uint(__fadd_rn(qi, 8388608.0f)) - 0x4B000000u);
        } else {
            if (ae < -149 - 26) return 0.0f;  // below 2^-151 (a.hi <= 1): rounds to +0
        }
    }
    if (y == 0.0f || x == 1.0f) return 1.0f;
    if (y == 1.0f) return x;
    if (x == 0.0f && y > 0.0f && y < 8388608.0f) {
        // Pow(+-0, y) = +-0 for an odd integer y > 0, else +0
        const float t = __fadd_rz(y, 8388608.0f);
        const bool odd = __fsub_rn(t, 8388608.0f) == y && (__float_as_uint(t) & 1u) != 0u;
        return (odd && signbit(x)) ? x : 0.0f;
    }
    return __double2float_rn(go_pow((double)x, (double)y));
}

// The three colour channels of material/ao.go:34-37 after
// total = math.Pow(T, 10000): uint8(float32(Pow(T, 10000)) * float32(ch)).
// Pow runs in float32 with a certified error bound, and its float64 form only
// when that bound leaves a channel undecided:
//  * T NaN: Pow is NaN and so is every product; Go's uint8 of NaN is 0 (the
//    low byte of the out-of-range int32). T == 1: Pow is exactly 1.
//  * 1 - T >= 6e-4: Pow(T, 10000) <= 0.9994^10000 < 0.00248, so every
//    product is below 255 * 0.00248 < 1 and truncates to 0.
//  * otherwise, with d = 1 - T exact: ln T = -(d + d u), u = d/2 + d^2/3 +
//    d^3/4 (truncation below 2e-17 after the factor 10000), 10000 ln T as an
//    unevaluated float pair, p = exp(hi) (1 + lo) with expf (2 ulp). |p/P - 1|
//    stays below 4e-7 (P Go's float64 result, itself within 1e-11 of the exact
//    power after its 27 roundings); float32(P) lies in
//    [RD(p(1 - 1e-6)), RU(p(1 + 1e-6))], the
//    product is monotone in it, and where both ends truncate alike the channel
//    is decided.
PR_DEV uint3 ao_scale(float T, uint32_t c0, uint32_t c1, uint32_t c2) {
    if (isnan(T)) return make_uint3(0u, 0u, 0u);
    if (T == 1.0f) return make_uint3(c0, c1, c2);
    const float d = __fsub_rn(1.0f, T);
    if (d >= 6e-4f) return make_uint3(0u, 0u, 0u);
    if (d > -1e-4f) {
        const float u = __fmul_rn(d, __fadd_rn(0.5f, __fmul_rn(d, __fadd_rn(0.333333333f, __fmul_rn(d, 0.25f)))));
        const float h1 = __fmul_rn(10000.0f, d);
        const float l1 = __fmaf_rn(10000.0f, d, -h1);  // 10000 d = h1 + l1 exactly
        const float w = __fmul_rn(h1, u);
        const float sh = __fadd_rn(h1, w);             // Fast2Sum: |w| < |h1|
        const float e2 = __fsub_rn(w, __fsub_rn(sh, h1));
        const float lo = -__fadd_rn(e2, l1);
        const float E = expf(-sh);
        const float p = __fmaf_rn(E, lo, E);
        const float plo = __fmul_rd(p, 0.999999f), phi = __fmul_ru(p, 1.000001f);
        const uint32_t a0 = go_f2u8(__fmul_rn(plo, small_u2f(c0))), b0 = go_f2u8(__fmul_rn(phi, small_u2f(c0)));
        const uint32_t a1 = go_f2u8(__fmul_rn(plo, small_u2f(c1))), b1 = go_f2u8(__fmul_rn(phi, small_u2f(c1)));
        const uint32_t a2 = go_f2u8(__fmul_rn(plo, small_u2f(c2))), b2 = go_f2u8(__fmul_rn(phi, small_u2f(c2)));
        if (__builtin_expect(a0 == b0 && a1 == b1 && a2 == b2, 1)) return make_uint3(a0, a1, a2);
    }
    const float P = __double2float_rn(go_pow((double)T, 10000.0));
    return make_uint3(go_f2u8(__fmul_rn(P, small_u2f(c0))), go_f2u8(__fmul_rn(P, small_u2f(c1))),
                      go_f2u8(__fmul_rn(P, small_u2f(c2))));
}

}  // namespace prd
