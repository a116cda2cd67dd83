"""CPU checks of the exactness arguments behind the AO kernel's shortcuts
(the kernel's own results are compared with the oracle in the GPU tests).

1. float32(Go Atan(x)) == x for positive float32 x with x^3 <= 0.999 * gap,
   gap = distance to the float32 below x.
2. The march distance of material/ao.go:52 satisfies |dist - t| <= 0.002 for
   every direction and tap t >= 1 at pixel coordinates below 16384, which is
   what lets the kernel bound elev/dist from both sides without computing it.
"""
import ctypes as C

import numpy as np

F = np.float32


def test_atan_small_argument_shortcut(oracle_lib):
    rng = np.random.default_rng(5)
    xs = np.concatenate([
        np.exp(rng.uniform(np.log(1e-30), np.log(5e-4), 200_000)),
        np.linspace(2.0e-4, 4.0e-4, 50_000),
    ]).astype(F)
    checked = 0
    for x in xs:
        b = int(x.view(np.uint32))
        e = b >> 23
        ge = e - 23 if (b & 0x7FFFFF) else e - 24
        if ge < 1:
            continue
        gap = np.uint32(ge << 23).view(F)
        if F(F(x * x) * x) <= F(gap * F(0.999)):
            got = F(oracle_lib.orc_go_atan(float(x)))
            assert got == x, (x, got)
            checked += 1
    assert checked > 100_000


def test_ao_distance_lower_bound(oracle_lib):
    cosv, sinv, n = (C.c_float * 8)(), (C.c_float * 8)(), C.c_int()
    oracle_lib.orc_ao_directions(cosv, sinv, C.byref(n))
    assert n.value == 8
    rng = np.random.default_rng(9)
    P = np.concatenate([rng.integers(0, 16384, 4000), np.arange(0, 200)]).astype(F)
    t = np.arange(1, 100, dtype=F)
    worst = np.inf
    worst_hi = -np.inf
    for k in range(8):
        qx = (F(cosv[k]) * t).astype(F)
        qy = (F(sinv[k]) * t).astype(F)
        for px, py in zip(P, P[::-1]):
            cx = (px + qx).astype(F)
            cy = (py + qy).astype(F)
            dx = (px - cx).astype(F)
            dy = (py - cy).astype(F)
            # Len of (dx, dy, 0, 0): sqrt(fma(dx, dx, dy*dy)) with float64 fma then float32
            d2 = (dx.astype(np.float64) * dx + (dy * dy).astype(F).astype(np.float64)).astype(F)
            dist = np.sqrt(d2.astype(np.float64)).astype(F)
            worst = min(worst, float(np.min(dist - t)))
            worst_hi = max(worst_hi, float(np.max(dist - t)))
    assert worst >= -0.002, worst
    assert worst_hi <= 0.002, worst_hi


def _half_gap_below(x):
    """Half the gap from integer x >= 1 to the float32 below it."""
    e = np.floor(np.log2(x)).astype(np.int64)
    pow2 = (x == np.exp2(e))
    return np.where(pow2, np.exp2(e - 25.0), np.exp2(e - 24.0))


def test_ao_tap_offsets(oracle_lib):
    """The AO kernel's table of tap offsets: for each direction component
    c and tap t <= 99, with a = float32(c t) and every pixel coordinate x up to
    16483 whose tap stays at RN(x + a) >= 0, int(RN(x + a)) equals
    x + floor(a), plus one while |a| <= half the gap below x when c is tiny
    and negative. It also checks the classification the host makes (every
    component regular or tiny-negative, so all 8 directions use the table)."""
    cosv, sinv, n = (C.c_float * 8)(), (C.c_float * 8)(), C.c_int()
    oracle_lib.orc_ao_directions(cosv, sinv, C.byref(n))
    x = np.arange(0, 16484, dtype=F)
    h_mx = 2.0 ** (13 - 24)  # half an ulp below 2^14 > 16483 + 100
    n_tiny = 0
    for k in range(n.value):
        for c in (F(cosv[k]), F(sinv[k])):
            tiny = c < 0 and F(-c * F(99)) < 1
            n_tiny += tiny
            for t in range(1, 100):
                a = F(c * F(t))
                if not tiny and a != np.floor(a):
                    assert np.ceil(a) - a > h_mx, (k, t, a)
                cx = (x + a).astype(F)
                m = cx >= 0
                ref = np.floor(cx[m]).astype(np.int64)
                pred = x[m].astype(np.int64) + int(np.floor(a))
                if tiny:
                    xs = x[m].astype(np.float64)
                    pred = pred + ((xs >= 1) & (abs(float(a)) <= _half_gap_below(np.maximum(xs, 1)))).astype(np.int64)
                assert np.array_equal(ref, pred), (k, t, float(a), np.flatnonzero(ref != pred)[:5])
    assert n_tiny == 2
