"""Screen-space clipping (render/clipping.go:31-157) of triangles whose
clipped polygons have every vertex count from 3 to 9, the largest crossing
all six planes (the four viewport sides, near and far): the clip kernel's
lane group re-interpolates polygon vertex 8 on its first lane and writes all
seven sub-triangles of a 9-vertex fan. The triangles are large and overlap
in random order, so the sub-triangles also compete for pixels. Bit-exact with
the oracle, single view and MSAA 2."""
import numpy as np
import pytest

from helpers import Pair, assert_bitexact, options
from polyred_gb300 import scene as sc

pytestmark = pytest.mark.gpu

W, H = 200, 150


def _cam():
    return sc.Perspective(position=(0, 0, 0), target=(0, 0, -1), up=(0, 1, 0), fov=60, aspect=W / H, near=0.5,
                          far=6.0)


def _polygon_sizes(tris, cam, w, h):
    """The clipped polygon's vertex count of each triangle, in float64 (only
    to pick the triangles: the renderers' float32 counts may differ at the
    margins), 0 for culled or unclipped triangles."""
    pv = (np.asarray(cam.proj_matrix(), np.float64).reshape(4, 4) @
          np.asarray(cam.view_matrix(), np.float64).reshape(4, 4))
    n = tris.shape[0]
    hom = np.concatenate([tris, np.ones((n, 3, 1))], axis=2) @ pv.T
    wv = hom[..., 3:4]
    scr = np.where((wv == 1.0) | (wv == 0.0), hom[..., :3], hom[..., :3] / np.where(wv == 0.0, 1.0, wv))
    scr = scr * [w / 2, h / 2, 1.0] + [w / 2, h / 2, 0.0]
    lo, hi = np.array([0.0, 0.0, -1.0]), np.array([w, h, 1.0])
    out = np.zeros(n, np.int64)
    for i in range(n):
        a, b, c = scr[i]
        if (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]) < 0:
            continue  # back face
        mn, mx = scr[i].min(0), scr[i].max(0)
        if (mn > hi).any() or (mx < lo).any():
            continue  # outside the viewport box
        if ((scr[i] >= lo) & (scr[i] <= hi)).all():
            continue  # contained: not clipped
        poly = [p for p in scr[i]]
        for axis, bound, keep_below in ((0, w, True), (0, 0.0, False), (1, h, True), (1, 0.0, False),
                                        (2, 1.0, True), (2, -1.0, False)):
            if not poly:
                break
            res = []
            s = poly[-1]
            for e in poly:
                fe = e[axis] < bound if keep_below else e[axis] > bound
                fs = s[axis] < bound if keep_below else s[axis] > bound
                if fe != fs:
                    t = (bound - s[axis]) / (e[axis] - s[axis])
                    res.append(s + (e - s) * t)
                if fe:
                    res.append(e)
                s = e
            poly = res
        out[i] = len(poly)
    return out


def _candidates(rng, n=3000):
    """Random triangles around and behind the camera, and triangles whose
    projections enclose most of the view (corners at 120 degrees around its
    centre, 1.2 to 2.2 NDC units out) with one vertex nearer than the near
    plane, one between the planes and one beyond the far plane: these clip to
    6 to 9 vertices."""
    loose = np.stack([rng.uniform(-9, 9, (n, 3)), rng.uniform(-7, 7, (n, 3)), rng.uniform(-9, 0.8, (n, 3))], axis=-1)
    th = rng.uniform(0, 2 * np.pi, n)[:, None] + np.arange(3) * (2 * np.pi / 3)
    r = rng.uniform(1.2, 2.2, (n, 3))
    d = np.stack([rng.uniform(0.25, 0.45, n), rng.uniform(1, 5, n), rng.uniform(8, 20, n)], axis=-1)
    d = np.take_along_axis(d, np.argsort(rng.uniform(size=(n, 3)), axis=1), axis=1)
    tf = np.tan(np.radians(30.0))
    wide = np.stack([r * np.cos(th) * d * tf * (W / H), r * np.sin(th) * d * tf, -d], axis=-1)
    return np.concatenate([loose, wide])


def _scene(seed):
    """Clipped triangles of each polygon size from 3 to 9, in random draw
    order, most of them overlapping."""
    rng = np.random.default_rng(seed)
    cand = _candidates(rng)
    sizes = _polygon_sizes(cand, _cam(), W, H)
    pick = []
    for k in range(3, 10):
        idx = np.flatnonzero(sizes == k)
        pick += list(idx[:12])
    pick = np.asarray(pick)
    counts = {k: int((sizes[pick] == k).sum()) for k in range(3, 10)}
    rng.shuffle(pick)
    tris = cand[pick].astype(np.float32)
    n = tris.shape[0]
    pos = np.ones((n, 3, 4), np.float32)
    pos[..., :3] = tris
    nrm = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=-1, keepdims=True), 1e-30)
    nor = np.zeros((n, 3, 4), np.float32)
    nor[..., :3] = nrm[:, None]
    uv = rng.uniform(0, 1, (n, 3, 2)).astype(np.float32)
    col = rng.integers(0, 256, (n, 3, 4)).astype(np.uint8)
    col[..., 3] = 255
    mesh = sc.Mesh(pos, nor, uv, col, rng.integers(-1, 2, n).astype(np.int32))
    mats = [sc.BlinnPhong(diffuse=sc.color_from_value(0.7, 0.4, 0.2, 1.0),
                          specular=sc.color_from_value(0.5, 0.5, 0.5, 1.0), shininess=24),
            sc.BlinnPhong(diffuse=sc.color_from_value(0.2, 0.6, 0.7, 1.0),
                          specular=sc.color_from_value(0.3, 0.3, 0.3, 1.0), shininess=8, flat_shading=True)]
    s = sc.Scene(sc.Geometry(mesh, *mats), sc.Point(position=(0.5, 1.0, -1.0), intensity=1.0), sc.Ambient(0.2))
    return s, counts


@pytest.mark.parametrize("seed", [0xC11A, 0xC11B])
@pytest.mark.parametrize("msaa", [1, 2])
def test_clipped_polygons_of_every_size(device, seed, msaa):
    s, counts = _scene(seed)
    assert all(v > 0 for v in counts.values()), counts  # 3 ... 9 vertices, 9 included
    p = Pair(device, options(s, _cam(), W, H, msaa=msaa))
    gpu, cpu = p.frame()
    assert_bitexact(gpu, cpu)
    assert p.stats["n_clipped_tris"] >= sum(counts[k] for k in range(4, 10)) // 2, (p.stats, counts)
    assert (gpu["tri_id"] != 0xFFFFFFFF).mean() > 0.5
