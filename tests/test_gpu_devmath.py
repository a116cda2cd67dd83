"""The device's float32 emulation of float32(fma(f64, f64, f64)) (Go's
math.FMA[float32]) against the direct FP64 expression, including inputs
built to hit double-rounding hazards."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _constructed(n, seed):
    """c has an odd mantissa; a*b = half an ulp of c minus/plus a tiny
    amount, so the float64 sum rounds onto the float32 midpoint."""
    g = np.random.default_rng(seed)
    e = g.integers(-30, 30, n)
    mant = (g.integers(0, 1 << 23, n) | 1).astype(np.float64)
    c = np.ldexp(1.0 + mant * 2.0 ** -23, e) * np.where(g.integers(0, 2, n) == 1, 1, -1)
    k = g.integers(1, 100, n).astype(np.float64)
    j = g.integers(-1, 2, n).astype(np.float64)
    a = 1.0 + k * 2.0 ** -23
    b = np.ldexp(1.0 - (k + j) * 2.0 ** -23, e - 24)
    s = np.where(g.integers(0, 2, n) == 1, 1.0, -1.0)
    return (a * s).astype(np.float32), (b * s).astype(np.float32), c.astype(np.float32)


def _below_pow2(n, seed):
    """c = the float just below 2^E (odd significand), a*b = 2^(E-25)
    (1 - k^2 2^-46) +- one ulp of b: s sits next to the midpoint below 2^E."""
    g = np.random.default_rng(seed)
    E = g.integers(-40, 40, n)
    k = g.integers(1, 300, n).astype(np.float64)
    c = np.ldexp(1.0 - 2.0 ** -24, E).astype(np.float32)
    a = (1.0 + k * 2.0 ** -23).astype(np.float32)
    b = np.ldexp(1.0 - k * 2.0 ** -23, E - 25).astype(np.float32)
    b = (b.view(np.int32) + g.integers(-1, 2, n).astype(np.int32)).view(np.float32)
    s = np.where(g.integers(0, 2, n) == 1, 1.0, -1.0).astype(np.float32)
    return a * s, b * s, c * s


def _bits(n, seed, lo, hi):
    """Random significands and signs with biased exponents in [lo, hi)."""
    g = np.random.default_rng(seed)
    m = g.integers(0, 1 << 32, (3, n), dtype=np.uint64).astype(np.uint32) & np.uint32(0x807FFFFF)
    e = g.integers(lo, hi, (3, n)).astype(np.uint32) << np.uint32(23)
    return tuple((m | e).view(np.float32))


def test_fma64f_matches_fp64(native_lib):
    import torch
    g = np.random.default_rng(0)
    n = 1 << 20
    ua, ub = g.uniform(-2000, 2000, (2, n)).astype(np.float32)
    # near-cancellation: c = -RN(ab) moved by up to 4 ulps
    cc = (-(ua * ub)).view(np.int32) + g.integers(-4, 5, n).astype(np.int32)
    sm = (g.integers(-4, 5, (3, n)) * np.where(g.integers(0, 2, (3, n)) == 1, 1.0, 0.5)).astype(np.float32)
    sets = [
        tuple(g.uniform(-2000, 2000, (3, n)).astype(np.float32)),
        _constructed(n, 1),
        (np.floor(g.uniform(0, 4096, n)).astype(np.float32) + 0.5, (g.integers(0, 2000, n) * 0.25 - 250).astype(np.float32),
         (-g.integers(0, 100000, n) * 0.001953125).astype(np.float32)),
        _below_pow2(n, 2),
        (ua, ub, cc.view(np.float32)),
        tuple(sm),
        _bits(n, 3, 0, 256),    # every exponent: subnormals, zeros, infinities, NaNs
        _bits(n, 4, 90, 170),
        # zero addends of either sign (the shortcut for c = +-0): every exponent of a and b
        _bits(n, 5, 0, 256)[:2] + (np.where(g.integers(0, 2, n) == 1, np.float32(0.0), np.float32(-0.0)),),
    ]
    for a, b, c in sets:
        ta, tb, tc = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (a, b, c))
        out = torch.empty_like(ta)
        ref = torch.empty_like(ta)
        rc = native_lib.pr_debug_fma_probe(ta.data_ptr(), tb.data_ptr(), tc.data_ptr(), out.data_ptr(), ref.data_ptr(), n)
        assert rc == 0
        o, r = out.cpu().numpy(), ref.cpu().numpy()
        same = (o.view(np.uint32) == r.view(np.uint32)) | (np.isnan(o) & np.isnan(r))
        assert same.all(), int((~same).sum())


def _ao_probe(native_lib, x, T, col):
    import torch
    n = len(x)
    tx = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    tT = torch.from_numpy(np.ascontiguousarray(T, np.float32)).cuda()
    tc = torch.from_numpy(np.ascontiguousarray(col, np.uint8)).cuda()
    af, ar = torch.empty_like(tx), torch.empty_like(tx)
    of, orf = torch.empty_like(tc), torch.empty_like(tc)
    rc = native_lib.pr_debug_ao_probe(tx.data_ptr(), af.data_ptr(), ar.data_ptr(), tT.data_ptr(), tc.data_ptr(),
                                      of.data_ptr(), orf.data_ptr(), n)
    assert rc == 0
    return af.cpu().numpy(), ar.cpu().numpy(), of.cpu().numpy(), orf.cpu().numpy()


def test_ao_atan_and_pow_shortcuts(native_lib):
    """The AO kernel's float32 Atan (series with a certified rounding check)
    and its float32 Pow(T, 10000) colour scaling give the float64
    algorithm's bits on every input, including Pow values constructed to put
    a channel's product on an integer."""
    g = np.random.default_rng(11)
    n = 1 << 20
    x = np.concatenate([
        np.exp(g.uniform(np.log(1e-6), np.log(1.5), n // 2)),
        g.uniform(2e-4, 0.07, n // 2),
    ]).astype(np.float32)
    # T near 1 over the whole certified range, and T with Pow(T, 10000) * c
    # within a few ulps of an integer m
    d = np.concatenate([g.uniform(-1e-4, 7e-4, n // 2), np.exp(g.uniform(np.log(1e-9), np.log(7e-4), n // 4))])
    c = g.integers(1, 256, n // 4)
    m = np.minimum(g.integers(1, 256, n // 4), c)
    Tm = np.power(m / c, 1e-4)
    Tm = (Tm.astype(np.float32).view(np.int32) + g.integers(-3, 4, n // 4).astype(np.int32)).view(np.float32)
    special = np.float32([1.0, np.nan, 0.0, 0.5, 0.9994, 1.00011])
    T = np.concatenate([special, (1.0 - d[:n // 2 + n // 4 - len(special)]).astype(np.float32), Tm])
    assert len(T) == n
    col = g.integers(0, 256, (n, 4)).astype(np.uint8)
    col[n // 2 + n // 4:, 0] = c
    af, ar, of, orf = _ao_probe(native_lib, x, T, col)
    assert np.array_equal(af.view(np.uint32), ar.view(np.uint32)), int((af != ar).sum())
    bad = np.flatnonzero((of != orf).any(1))
    assert len(bad) == 0, (len(bad), T[bad[:4]], col[bad[:4]], of[bad[:4]], orf[bad[:4]])


def test_pow_float32_matches_float64(native_lib):
    """The shade kernel's Pow (float32 pairs with a certified rounding)
    against the float64 algorithm: shininess exponents, arguments across
    (0, 1] including tiny ones (subnormal and zero results), zeros, ones,
    and non-integer exponents (float64 path)."""
    import torch
    g = np.random.default_rng(13)
    n = 1 << 20
    x = np.concatenate([
        g.uniform(0, 1, n // 4),
        1 - np.exp(g.uniform(np.log(1e-8), np.log(0.5), n // 4)),
        np.exp(g.uniform(np.log(1e-30), 0, n // 4)),
        np.float32([0.0, -0.0, 1.0, 0.5, 0.25, 2.0 ** -60, 2.0 ** -59, 0.9999999]),
    ]).astype(np.float32)
    x = np.concatenate([x, g.uniform(0, 1, n - len(x))]).astype(np.float32)
    ys = np.float32([1, 2, 3, 4, 5, 7, 8, 12, 16, 31, 32, 33, 50, 64, 100, 128, 255, 1000, 4096, 0, 12.5, 4097])
    y = ys[g.integers(0, len(ys), n)].astype(np.float32)
    tx, ty = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    f, r = torch.empty_like(tx), torch.empty_like(tx)
    assert native_lib.pr_debug_pow_probe(tx.data_ptr(), ty.data_ptr(), f.data_ptr(), r.data_ptr(), n) == 0
    f, r = f.cpu().numpy(), r.cpu().numpy()
    bad = np.flatnonzero(f.view(np.uint32) != r.view(np.uint32))
    assert len(bad) == 0, (len(bad), x[bad[:4]], y[bad[:4]], f[bad[:4]], r[bad[:4]])
