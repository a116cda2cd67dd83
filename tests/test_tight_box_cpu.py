"""CPU check of the raster's narrowed pixel boxes (tighten_box in
pr_kernels.cu): every pixel of the reference's box (rounded bounding box
padded by one, render/raster.go:473-477) that the narrowing leaves out fails
the inside test bc >= -Epsilon (render/raster.go:491) of the oracle's
Barycoord, on random tiny, sliver, large, near-degenerate and grid-aligned
triangles.

The margin here is computed in float64 from the same formula without the
kernel's upward rounding, so it is at most the kernel's: the pixels it
leaves out include every pixel the kernel leaves out."""
import ctypes as C
import math

import numpy as np

F = np.float32
EPS = F(1e-7)
U = 2.0 ** -24


def pround(x):
    return math.floor(x + 0.5) if x >= 0 else math.ceil(x - 0.5)


def reference_box(tri, W, H):
    xs, ys = [float(v[0]) for v in tri], [float(v[1]) for v in tri]
    x0 = max(0, int(F(pround(min(xs)) - 1.0)))
    x1 = min(W - 1, int(F(pround(max(xs)) + 1.0)))
    y0 = max(0, int(F(pround(min(ys)) - 1.0)))
    y1 = min(H - 1, int(F(pround(max(ys)) + 1.0)))
    return x0, x1, y0, y1


def sabc_of(tri):
    """Sabc as the kernel's record holds it: the cross product of the rounded
    edge differences, its second term rounded to float32, the rest through
    float64 and then to float32 (Go's math.FMA[float32])."""
    (ax, ay), (bx, by), (cx, cy) = [(F(v[0]), F(v[1])) for v in tri]
    ex, ey, fx, fy = F(bx - ax), F(by - ay), F(cx - ax), F(cy - ay)
    return F(float(ex) * float(fy) - float(F(ey * fx)))


def tight_box(tri, sabc, box):
    x0, x1, y0, y1 = box
    xs, ys = [float(v[0]) for v in tri], [float(v[1]) for v in tri]
    mnx, mxx, mny, mxy = min(xs), max(xs), min(ys), max(ys)
    if not all(math.isfinite(v) for v in (mnx, mxx, mny, mxy, float(sabc))):
        return box
    wx, wy = mxx - mnx, mxy - mny
    E = wx + wy
    Uu = E + 4.0
    dS, dA = 6 * U * E * Uu, 6 * U * E * E
    a = abs(float(sabc))
    L = a - dA
    if not (L > 2 * dA and L > 0):
        return box
    q = (dS + 2.0e-7 * (a + 2 * dA)) / L
    mx, my = 2 * wx * q * (1 - 1e-9), 2 * wy * q * (1 - 1e-9)
    lx, hx = math.ceil(mnx - mx - 0.5), math.floor(mxx + mx - 0.5)
    ly, hy = math.ceil(mny - my - 0.5), math.floor(mxy + my - 0.5)
    if lx > hx or ly > hy:
        return (1, 0, 1, 0)
    return max(x0, lx), min(x1, hx), max(y0, ly), min(y1, hy)


def rejected(oracle_lib, tri, px, py):
    p = (C.c_float * 2)(px + 0.5, py + 0.5)
    t = [(C.c_float * 2)(float(v[0]), float(v[1])) for v in tri]
    out = (C.c_float * 3)()
    oracle_lib.orc_barycoord(p, t[0], t[1], t[2], out)
    return any(F(out[k]) < -EPS for k in range(3))


def triangles(rng, n):
    W = H = 4096
    for k in range(n):
        kind = k % 6
        c = rng.uniform(2, W - 2, 2)
        if kind == 0:  # tiny, log-uniform size
            s = math.exp(rng.uniform(math.log(1e-3), math.log(4.0)))
            tri = c + rng.normal(0, s, (3, 2))
        elif kind == 1:  # slivers
            d = rng.normal(0, 1, 2)
            d /= np.linalg.norm(d)
            L = math.exp(rng.uniform(0, math.log(300)))
            w = math.exp(rng.uniform(math.log(1e-4), math.log(2.0)))
            tri = np.array([c, c + L * d, c + 0.5 * L * d + w * np.array([-d[1], d[0]])])
        elif kind == 2:  # large
            tri = c + rng.normal(0, rng.uniform(20, 400), (3, 2))
        elif kind == 3:  # nearly collinear
            d = rng.normal(0, 1, 2)
            L = rng.uniform(0.5, 50)
            tri = np.array([c, c + L * d, c + rng.uniform(0.1, 0.9) * L * d + rng.normal(0, 1e-5, 2)])
        elif kind == 4:  # vertices on pixel centres and integers
            base = np.floor(c)
            tri = base + rng.integers(-3, 4, (3, 2)) + rng.choice([0.0, 0.5], (3, 2))
        else:  # near the origin and the far edge (clamped boxes)
            c = rng.choice([rng.uniform(-3, 3, 2), rng.uniform(W - 3, W + 3, 2)])
            tri = c + rng.normal(0, math.exp(rng.uniform(math.log(0.01), math.log(20))), (3, 2))
        yield np.asarray(tri, F), W, H


def test_narrowed_boxes_leave_out_only_rejected_pixels(oracle_lib):
    rng = np.random.default_rng(0x7B0C)
    left_out = narrowed = 0
    for tri, W, H in triangles(rng, 8_000):
        box = reference_box(tri, W, H)
        x0, x1, y0, y1 = box
        if x0 > x1 or y0 > y1:
            continue
        t = tight_box(tri, sabc_of(tri), box)
        if t != box:
            narrowed += 1
        for py in range(y0, y1 + 1):
            inside_y = t[2] <= py <= t[3]
            for px in range(x0, x1 + 1):
                if inside_y and t[0] <= px <= t[1]:
                    continue
                # large boxes: the pixels next to the narrowed box, where a miss would be
                if (x1 - x0 + 1) * (y1 - y0 + 1) > 400 and min(abs(px - t[0]), abs(px - t[1]), abs(py - t[2]),
                                                                abs(py - t[3])) > 2:
                    continue
                assert rejected(oracle_lib, tri, px, py), (tri.tolist(), px, py, box, t)
                left_out += 1
    assert narrowed > 5_000 and left_out > 30_000, (narrowed, left_out)
