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


def test_fma64f_matches_fp64(native_lib):
    import torch
    g = np.random.default_rng(0)
    n = 1 << 20
    sets = [
        tuple(g.uniform(-2000, 2000, (3, n)).astype(np.float32)),
        _constructed(n, 1),
        (np.floor(g.uniform(0, 4096, n)).astype(np.float32) + 0.5, (g.integers(0, 2000, n) * 0.25 - 250).astype(np.float32),
         (-g.integers(0, 100000, n) * 0.001953125).astype(np.float32)),
    ]
    for a, b, c in sets:
        ta, tb, tc = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (a, b, c))
        out = torch.empty_like(ta)
        ref = torch.empty_like(ta)
        rc = native_lib.pr_debug_fma_probe(ta.data_ptr(), tb.data_ptr(), tc.data_ptr(), out.data_ptr(), ref.data_ptr(), n)
        assert rc == 0
        o, r = out.cpu().numpy(), ref.cpu().numpy()
        assert np.array_equal(o.view(np.uint32), r.view(np.uint32))
