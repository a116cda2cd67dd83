// Material textures: buffer.Texture.Query (buffer/texture.go:83-187) and the
// FragmentShader's level of detail (shader/blinn_cpu.go:28-35), in the
// reference's float32 / float64 order.
//
// One source for both sides: the shade kernel includes it (nvcc with
// -fmad=false) and the host library includes it (g++ -ffp-contract=off) for
// pr_debug_texture_query, so the arithmetic is plain IEEE operators with no
// contraction on either. Texels are packed RGBA8 (R in the low byte), rows
// top-down as image.RGBA stores them; a texture's mipmap levels follow each
// other in one texel buffer.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PR_HD __host__ __device__ __forceinline__
#else
#define PR_HD inline
#endif

namespace prt {

constexpr int kMaxTexLevels = 16;  // int(Log2(16384)) + 1 = 15 levels at most

struct TexDesc {
    int32_t n_levels;    // levels stored: the whole mipmap, or level 0 alone without mipmaps
    int32_t use_mipmap;  // Texture.UseMipmap()
    int32_t size;        // Texture.Size(): the width of level 0
    int32_t reserved;
    int32_t w[kMaxTexLevels], h[kMaxTexLevels];
    uint32_t off[kMaxTexLevels];  // first texel of each level
};

PR_HD uint64_t dbits(double x) {
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
}
PR_HD double dfrom(uint64_t u) {
    double x;
    memcpy(&x, &u, 8);
    return x;
}

// Go's float-to-integer conversion on amd64 (CVTTSS2SQ): truncation, and
// 0x8000000000000000 for NaN and out-of-range values.
PR_HD int64_t f2i64(float x) {
    if (!(x > -9223372036854775808.0f && x < 9223372036854775808.0f)) return INT64_MIN;
    return (int64_t)x;
}
// uint8(f) on amd64: float32 -> int32 (CVTTSS2SL, 0x80000000 for NaN and
// out of range), then the low byte.
PR_HD uint32_t f2u8(float x) {
    if (!(x > -2147483648.0f && x < 2147483648.0f)) return 0u;
    return (uint32_t)(int32_t)x & 0xffu;
}

// math.Max (Go math/dim.go): +Inf wins, then NaN, and +0 > -0.
PR_HD double go_max(double x, double y) {
    if (x == INFINITY || y == INFINITY) return INFINITY;
    if (x != x || y != y) return NAN;
    if (x == 0 && x == y) return (dbits(x) >> 63) ? y : x;
    return x > y ? x : y;
}

// math.Modf (Go math/modf.go): integer and fractional parts with f's sign;
// Modf(+-Inf) = +-Inf, NaN.
PR_HD double go_modf(double f, double* ip) {
    double sgn = 1.0;
    if (f < 1) {
        if (f == 0) {
            *ip = f;
            return f;
        }
        if (f >= 0) {
            *ip = 0;
            return f;
        }
        sgn = -1.0;
        f = -f;
        if (f < 1) {
            *ip = -0.0;
            return -f;
        }
    }
    uint64_t x = dbits(f);
    const uint64_t e = ((x >> 52) & 0x7ff) - 1023;
    if (e < 52) x &= ~((1ull << (52 - e)) - 1);
    const double i = dfrom(x);
    *ip = sgn * i;
    return sgn * (f - i);
}

// math.Log (Go math/log.go, the FreeBSD / fdlibm e_log.c method: argument
// reduction by frexp and a degree-14 odd polynomial in s = f / (2 + f)).
PR_HD double go_log(double x) {
    const double Ln2Hi = 6.93147180369123816490e-01, Ln2Lo = 1.90821492927058770002e-10;
    const double L1 = 6.666666666666735130e-01, L2 = 3.999999999940941908e-01, L3 = 2.857142874366239149e-01,
                 L4 = 2.222219843214978396e-01, L5 = 1.818357216161805012e-01, L6 = 1.531383769920937332e-01,
                 L7 = 1.479819860511658591e-01;
    if (x != x || x == INFINITY) return x;
    if (x < 0) return NAN;
    if (x == 0) return -INFINITY;
    int ki;
    double f1 = frexp(x, &ki);
    if (f1 < 0.70710678118654752440) {  // Sqrt2 / 2
        f1 *= 2;
        ki--;
    }
    const double f = f1 - 1;
    const double k = (double)ki;
    const double s = f / (2 + f);
    const double s2 = s * s;
    const double s4 = s2 * s2;
    const double t1 = s2 * (L1 + s4 * (L3 + s4 * (L5 + s4 * L7)));
    const double t2 = s4 * (L2 + s4 * (L4 + s4 * L6));
    const double R = t1 + t2;
    const double hfsq = 0.5 * f * f;
    return k * Ln2Hi - ((hfsq - (s * (hfsq + R) + k * Ln2Lo)) - f);
}

// math.Log2 (Go math/log10.go): exact for powers of two.
PR_HD double go_log2(double x) {
    if (x != x || x == INFINITY || x <= 0) return go_log(x);
    int e;
    const double frac = frexp(x, &e);
    if (frac == 0.5) return (double)(e - 1);
    return go_log(frac) * 1.44269504088896340736 + (double)e;  // 1 / Ln2
}

// FragmentShader's lod (shader/blinn_cpu.go:28-35): Log2 of the texture
// size times Sqrt(Max(Du, Dv)), at least Log2(1).
PR_HD float tex_lod(const TexDesc& t, float du, float dv) {
    if (!t.use_mipmap) return 0.0f;
    const float m = (float)go_max(go_max(-DBL_MAX, (double)du), (double)dv);
    const float sq = (float)sqrt((double)m);
    float siz = (float)t.size * sq;
    if (siz < 1) siz = 1;
    return (float)go_log2((double)siz);
}

// image.RGBA.RGBAAt: transparent black outside the image.
PR_HD uint32_t tex_at(const TexDesc& t, const uint32_t* tx, int lvl, int64_t x, int64_t y) {
    if (x < 0 || y < 0 || x >= t.w[lvl] || y >= t.h[lvl]) return 0u;
    return tx[t.off[lvl] + (uint32_t)y * (uint32_t)t.w[lvl] + (uint32_t)x];
}

// math.LerpC (math/interpolate.go:55-62): per channel uint8(from + t*(to - from)).
PR_HD uint32_t lerpc(uint32_t a, uint32_t b, float t) {
    uint32_t r = 0;
    for (int k = 0; k < 4; k++) {
        const float fa = (float)((a >> (8 * k)) & 0xffu), fb = (float)((b >> (8 * k)) & 0xffu);
        r |= f2u8(fa + t * (fb - fa)) << (8 * k);
    }
    return r;
}

// queryBilinear (buffer/texture.go:150-186)
PR_HD uint32_t tex_bilinear(const TexDesc& t, const uint32_t* tx, int lvl, float u, float v) {
    const int dx = t.w[lvl], dy = t.h[lvl];
    if (dx == 1 && dy == 1) return tx[t.off[lvl]];
    const float x = u * ((float)dx - 1.0f);
    const float y = v * ((float)dy - 1.0f);
    const float x0 = floorf(x), y0 = floorf(y);
    const int64_t i = f2i64(x0), j = f2i64(y0);
    const uint32_t p1 = tex_at(t, tx, lvl, i, j);
    const uint32_t p2 = i < dx - 1 ? tex_at(t, tx, lvl, i + 1, j) : p1;
    const uint32_t i1 = lerpc(p1, p2, x - x0);
    const uint32_t p3 = j < dy - 1 ? tex_at(t, tx, lvl, i, j + 1) : p1;
    const uint32_t p4 = (i < dx - 1 && j < dy - 1) ? tex_at(t, tx, lvl, i + 1, j + 1) : p1;
    const uint32_t i2 = lerpc(p3, p4, x - x0);
    return lerpc(i1, i2, y - y0);
}

// queryL0 (buffer/texture.go:131-142)
PR_HD uint32_t tex_l0(const TexDesc& t, const uint32_t* tx, float u, float v) {
    const int dx = t.w[0], dy = t.h[0];
    if (dx == 1 && dy == 1) return tx[t.off[0]];
    const int64_t x = f2i64(floorf(u * ((float)dx - 1.0f)));
    const int64_t y = f2i64(floorf(v * ((float)dy - 1.0f)));
    return tex_at(t, tx, 0, x, y);
}

// Texture.Query (buffer/texture.go:83-129). A NaN lod makes the reference
// index its mipmap slice out of range (a panic); here it gives transparent
// black.
PR_HD uint32_t tex_query(const TexDesc& t, const uint32_t* tx, float lod, float u, float v) {
    double ip;
    u = (float)go_modf((double)u, &ip);
    if ((float)ip != 0 && u == 0) u = 1;
    if (u < 0) u = 1 - u;
    v = (float)go_modf((double)v, &ip);
    if ((float)ip != 0 && v == 0) v = 1;
    if (v < 0) v = 1 - v;
    if (!t.use_mipmap) return tex_l0(t, tx, u, v);
    const int L = t.n_levels;
    if (lod < 0)
        lod = 0;
    else if (lod >= (float)L)
        lod = (float)(L - 1);
    if (lod <= 1) return tex_bilinear(t, tx, 0, u, v);
    lod -= 1;
    const int64_t h = f2i64(floorf(lod));
    if (h < 0 || h >= L) return 0u;
    const int64_t l = h + 1;
    if (l >= L) return tex_bilinear(t, tx, (int)h, u, v);
    const float p = lod - (float)h;
    if (fabsf(p - 0.0f) <= 1e-7f) return tex_bilinear(t, tx, (int)h, u, v);  // ApproxEq(p, 0, Epsilon)
    return lerpc(tex_bilinear(t, tx, (int)h, u, v), tex_bilinear(t, tx, (int)l, u, v), p);
}

}  // namespace prt
