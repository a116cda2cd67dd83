// gomath.h — CPU restatement of the float semantics polyred's Go code relies on.
//
// TEST INFRASTRUCTURE: this file belongs to the oracle. Only tests, the smoke
// check and bench.py's CPU-baseline leg use it; the product never links it.
//
// Compile with -ffp-contract=off -fno-fast-math: every float32 a*b+c below is
// two IEEE roundings, as Go's amd64 back end (GOAMD64=v1) evaluates it.
//
// Go standard library functions the reference calls (Go 1.26, go.mod:3) are
// restated from their published algorithms where the last bit matters:
//   math.Max/Min special cases, math.Pow (integer-exponent repeated squaring),
//   math.Atan (Cephes atan reduction), float->int conversions of amd64.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace gomath {

// math.FMA[float32] — math/math.go:265-267: FMA in float64, rounded to float32.
inline float fma32(float x, float y, float z) {
    return (float)std::fma((double)x, (double)y, (double)z);
}

// Go's math.Max / math.Min special cases (Go math/dim.go):
// Max(x, +Inf) = +Inf, Max(x, NaN) = NaN, Max(+0, -0) = +0.
inline double go_max(double x, double y) {
    if (std::isinf(x) && x > 0) return x;
    if (std::isinf(y) && y > 0) return y;
    if (std::isnan(x) || std::isnan(y)) return NAN;
    if (x == 0 && x == y) return std::signbit(x) ? y : x;
    return x > y ? x : y;
}
inline double go_min(double x, double y) {
    if (std::isinf(x) && x < 0) return x;
    if (std::isinf(y) && y < 0) return y;
    if (std::isnan(x) || std::isnan(y)) return NAN;
    if (x == 0 && x == y) return std::signbit(x) ? x : y;
    return x < y ? x : y;
}

// polyred math.Max/Min with two float32 arguments (math/math.go:245-261):
// fold from -MaxFloat64/+MaxFloat64 in float64, convert to float32.
inline float pmax(float a, float b) { return (float)go_max(go_max(-DBL_MAX, a), b); }
inline float pmin(float a, float b) { return (float)go_min(go_min(DBL_MAX, a), b); }
inline float pmax3(float a, float b, float c) {
    return (float)go_max(go_max(go_max(-DBL_MAX, a), b), c);
}
inline float pmin3(float a, float b, float c) {
    return (float)go_min(go_min(go_min(DBL_MAX, a), b), c);
}

// polyred math.Round (math/math.go:58-60): half away from zero.
inline float pround(float x) { return (float)std::round((double)x); }

// math.Clamp (math/clamp.go:8-16).
inline float pclamp(float n, float lo, float hi) {
    if (n < lo) return lo;
    if (n > hi) return hi;
    return n;
}

// Go int(float32) on amd64: CVTTSS2SQ truncates; NaN and out-of-range give
// the "integer indefinite" 0x8000000000000000.
inline int64_t go_f2i(float x) {
    if (std::isnan(x) || x >= 9.2233720368547758e18f || x < -9.2233720368547758e18f)
        return INT64_MIN;
    return (int64_t)x;
}

// Go uint8(float32) on amd64: float32 -> int32 (CVTTSS2SL), then the low byte.
inline uint8_t go_f2u8(float x) {
    if (std::isnan(x) || x >= 2147483648.0f || x < -2147483648.0f) return 0;  // 0x80000000
    return (uint8_t)((uint32_t)(int32_t)x & 0xffu);
}

// Go math.Log (math/log.go): the fdlibm e_log.c reduction x = 2^k (1 + f),
// s = f / (2 + f), R(s) polynomial, log = k ln2_hi - ((hfsq - (s (hfsq + R)
// + k ln2_lo)) - f).
inline double go_log(double x) {
    static const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    static const double lg[7] = {6.666666666666735130e-01, 3.999999999940941908e-01, 2.857142874366239149e-01,
                                 2.222219843214978396e-01, 1.818357216161805012e-01, 1.531383769920937332e-01,
                                 1.479819860511658591e-01};
    if (std::isnan(x) || (std::isinf(x) && x > 0)) return x;
    if (x < 0) return NAN;
    if (x == 0) return -INFINITY;
    int k;
    double f1 = std::frexp(x, &k);
    if (f1 < 0.70710678118654752440) {
        f1 = f1 * 2;
        k = k - 1;
    }
    double f = f1 - 1;
    double s = f / (2 + f);
    double z = s * s;
    double w = z * z;
    double odd = z * (lg[0] + w * (lg[2] + w * (lg[4] + w * lg[6])));
    double even = w * (lg[1] + w * (lg[3] + w * lg[5]));
    double r = odd + even;
    double hfsq = 0.5 * f * f;
    double dk = (double)k;
    return dk * ln2_hi - ((hfsq - (s * (hfsq + r) + dk * ln2_lo)) - f);
}

// Go math.Log2 (math/log10.go): powers of two exactly, else Log(frac)/Ln2 + exp.
inline double go_log2(double x) {
    int e;
    double frac = std::frexp(x, &e);
    if (std::isfinite(x) && x > 0 && frac == 0.5) return (double)(e - 1);
    if (!std::isfinite(x) || x <= 0) return go_log(x);
    return go_log(frac) * 1.44269504088896340736 + (double)e;  // 1/Ln2 folded exactly, then rounded
}

// Go math.Frexp: frac in [0.5, 1), x = frac * 2^exp (Go math/frexp.go).
inline double go_frexp(double x, int* e) {
    *e = 0;
    if (x == 0 || std::isinf(x) || std::isnan(x)) return x;
    return std::frexp(x, e);
}

inline bool is_odd_int(double x) {
    if (std::fabs(x) >= 9007199254740992.0) return false;  // 2^53: all even
    double xi;
    double xf = std::modf(x, &xi);
    if (xf != 0) return false;
    int64_t i = (int64_t)xi;
    return (i & 1) == 1;
}

// Go math.Pow (Go math/pow.go). The integer part of the exponent is applied by
// repeated squaring of the frexp mantissa; the fractional part (non-integer
// exponents only) by Exp(yf*Log(x)), restated here with libm exp/log.
inline double go_pow(double x, double y) {
    if (y == 0 || x == 1) return 1;
    if (y == 1) return x;
    if (std::isnan(x) || std::isnan(y)) return NAN;
    if (x == 0) {
        if (y < 0) {
            if (std::signbit(x) && is_odd_int(y)) return -INFINITY;
            return INFINITY;
        }
        if (y > 0) {
            if (std::signbit(x) && is_odd_int(y)) return x;
            return 0;
        }
    }
    if (std::isinf(y)) {
        if (x == -1) return 1;
        if ((std::fabs(x) < 1) == (y > 0)) return 0;
        return INFINITY;
    }
    if (std::isinf(x)) {
        if (x < 0) return go_pow(1 / x, -y);
        if (y < 0) return 0;
        if (y > 0) return INFINITY;
    }
    if (y == 0.5) return std::sqrt(x);
    if (y == -0.5) return 1 / std::sqrt(x);

    double yi;
    double yf = std::modf(std::fabs(y), &yi);
    if (yf != 0 && x < 0) return NAN;
    if (yi >= 9223372036854775808.0) {
        if (x == -1) return 1;
        if ((std::fabs(x) < 1) == (y > 0)) return 0;
        return INFINITY;
    }
    double a1 = 1.0;
    int64_t ae = 0;
    if (yf != 0) {
        if (yf > 0.5) {
            yf -= 1;
            yi += 1;
        }
        a1 = std::exp(yf * std::log(x));
    }
    int xe_i;
    double x1 = go_frexp(x, &xe_i);
    int64_t xe = xe_i;
    for (int64_t i = (int64_t)yi; i != 0; i >>= 1) {
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
    if (y < 0) {
        a1 = 1 / a1;
        ae = -ae;
    }
    if (ae > 4096) ae = 4096;
    if (ae < -4096) ae = -4096;
    return std::ldexp(a1, (int)ae);
}

// Go math.Atan (Go math/atan.go): Cephes reduction to [0, 0.66].
inline double go_xatan(double x) {
    const double P0 = -8.750608600031904122785e-01;
    const double P1 = -1.615753718733365076637e+01;
    const double P2 = -7.500855792314704667340e+01;
    const double P3 = -1.228866684490136173410e+02;
    const double P4 = -6.485021904942025371773e+01;
    const double Q0 = +2.485846490142306297962e+01;
    const double Q1 = +1.650270098316988542046e+02;
    const double Q2 = +4.328810604912902668951e+02;
    const double Q3 = +4.853903996359136964868e+02;
    const double Q4 = +1.945506571482613964425e+02;
    double z = x * x;
    z = z * ((((P0 * z + P1) * z + P2) * z + P3) * z + P4) /
        (((((z + Q0) * z + Q1) * z + Q2) * z + Q3) * z + Q4);
    z = x * z + x;
    return z;
}
inline double go_satan(double x) {
    const double Morebits = 6.123233995736765886130e-17;
    const double Tan3pio8 = 2.41421356237309504880;
    const double PiOver2 = 1.57079632679489661923132169163975144;
    const double PiOver4 = 0.785398163397448309615660845819875721;
    if (x <= 0.66) return go_xatan(x);
    if (x > Tan3pio8) return PiOver2 - go_xatan(1 / x) + Morebits;
    return PiOver4 + go_xatan((x - 1) / (x + 1)) + 0.5 * Morebits;
}
inline double go_atan(double x) {
    if (x == 0) return x;
    if (x > 0) return go_satan(x);
    return -go_satan(-x);
}

}  // namespace gomath
