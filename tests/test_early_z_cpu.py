"""CPU check of the raster's early depth test (early_z_key in
pr_kernels.cu): for every triangle the kernel treats as well-conditioned,
every pixel the reference rasterises (inside test bc >= -Epsilon of the
oracle's Barycoord, render/raster.go:491) gets a depth, interpolated as the
raster does (render/raster.go:494-496), no larger than the bound
max Zi + (eta + 1.5e-6) max |Zi|, eta = (dA + 3 dS) / |Sabc| <= 0.05. A
fragment the early test skips therefore never raises a depth key.

The condition and the bound are computed here in float64 without the
kernel's outward rounding: the kernel's condition is the stricter and its
bound the larger, so every triangle and pixel it skips is covered here."""
import ctypes as C
import math

import numpy as np

from test_tight_box_cpu import EPS, F, U, reference_box, sabc_of, triangles


def eta_of(tri, sabc):
    """(dA + 3 dS) / |Sabc|, or None when the kernel makes no bound."""
    xs, ys = [float(v[0]) for v in tri], [float(v[1]) for v in tri]
    E = (max(xs) - min(xs)) + (max(ys) - min(ys))
    dS, dA = 6 * U * E * (E + 4.0), 6 * U * E * E
    a = abs(float(sabc))
    if not (math.isfinite(a) and a > 0):
        return None
    eta = (dA + 3 * dS) / a
    return eta if eta <= 0.05 else None


def test_depth_bound_holds_for_covered_pixels(oracle_lib):
    rng = np.random.default_rng(0xE2B0)
    checked = conditioned = 0
    worst = 0.0
    for n, (tri, W, H) in enumerate(triangles(rng, 2_500)):
        sabc = sabc_of(tri)
        eta = eta_of(tri, sabc)
        if eta is None:
            continue
        conditioned += 1
        # depths: NDC-like values near -1, shadow-map-like values in [0, 1], wide ranges, mixed signs
        kind = n % 4
        if kind == 0:
            Z = F(-1.0) + rng.uniform(0, 0.02, 3).astype(F)
        elif kind == 1:
            Z = rng.uniform(0, 1, 3).astype(F)
        elif kind == 2:
            Z = (rng.normal(0, 1, 3) * 10.0 ** rng.uniform(-3, 3)).astype(F)
        else:
            Z = np.array([F(-0.5), F(0.5), F(rng.uniform(-1, 1))], F)
        M = max(abs(float(z)) for z in Z)
        zb = max(float(z) for z in Z) + (eta + 1.5e-6) * M
        x0, x1, y0, y1 = reference_box(tri, W, H)
        t = [(C.c_float * 2)(float(v[0]), float(v[1])) for v in tri]
        out = (C.c_float * 3)()
        for py in range(y0, y1 + 1):
            for px in range(x0, x1 + 1):
                if (x1 - x0 + 1) * (y1 - y0 + 1) > 600 and (px + py) % 13:
                    continue  # large boxes: a sample of their pixels
                p = (C.c_float * 2)(px + 0.5, py + 0.5)
                oracle_lib.orc_barycoord(p, t[0], t[1], t[2], out)
                b = [F(out[k]) for k in range(3)]
                if any(v < -EPS for v in b):
                    continue
                z = F(F(F(b[0] * Z[0]) + F(b[1] * Z[1])) + F(b[2] * Z[2]))
                assert float(z) <= zb, (tri.tolist(), Z.tolist(), px, py, b, float(z), zb)
                if M:
                    worst = max(worst, (float(z) - max(float(v) for v in Z)) / M - eta)
                checked += 1
    assert conditioned > 1_600 and checked > 30_000, (conditioned, checked)
    # beyond eta, the arithmetic reaches a small part of the 1.5e-6 allowed
    assert worst < 1.5e-6, worst
