"""The raster's early depth test where it decides most: many stacked layers
drawn in random order (most fragments lose to a layer already stored),
coplanar duplicates (equal depths, where the first drawn must keep the
pixel: buffer/buffer.go:230), and a point light's shadow map over the same
stack. The frame is large enough for the single-view raster to use the test
(at least 32 tasks per warp), and the batch uses it on every pass; both are
bit-exact with the oracle and with each other."""
import ctypes as C

import numpy as np
import pytest

from helpers import Pair, assert_bitexact, options, same_bits
from polyred_gb300 import batch as pb, native, render, scene as sc

pytestmark = pytest.mark.gpu

W, H = 640, 480


def _mesh(tris, mats, cols):
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    n = tris.shape[0]
    pos = np.ones((n, 3, 4), np.float32)
    pos[..., :3] = tris
    nrm = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=-1, keepdims=True), 1e-30)
    nor = np.zeros((n, 3, 4), np.float32)
    nor[..., :3] = nrm[:, None]
    uv = np.zeros((n, 3, 2), np.float32)
    col = np.repeat(np.asarray(cols, np.uint8)[:, None], 3, axis=1)
    return sc.Mesh(pos, nor, uv, col, np.asarray(mats, np.int32))


def _stack_scene(seed, n_layers=48, n_dups=12):
    """Quads at random depths, drawn in random order, each duplicated now and
    then (same plane, later in the draw order, another colour), facing +z."""
    rng = np.random.default_rng(seed)
    tris, mats, cols = [], [], []
    layers = []
    for _ in range(n_layers):
        z = float(rng.uniform(-3.0, 1.0))
        cx, cy = rng.uniform(-0.6, 0.6, 2)
        hw, hh = rng.uniform(2.5, 5.0, 2)
        layers.append((z, cx, cy, hw, hh))
    dups = [layers[int(k)] for k in rng.integers(0, n_layers, n_dups)]
    order = list(range(n_layers + n_dups))
    rng.shuffle(order)
    allq = layers + dups
    for k in order:
        z, cx, cy, hw, hh = allq[k]
        a, b, c, d = ([cx - hw, cy - hh, z], [cx + hw, cy - hh, z], [cx + hw, cy + hh, z], [cx - hw, cy + hh, z])
        tris += [[a, b, c], [a, c, d]]
        m = int(k % 2)
        mats += [m, m]
        col = rng.integers(0, 256, 4)
        col[3] = 255
        cols += [col, col]
    mat_ao = sc.BlinnPhong(diffuse=sc.color_from_value(0.8, 0.3, 0.2, 1.0),
                           specular=sc.color_from_value(0.5, 0.5, 0.5, 1.0), shininess=32, ambient_occlusion=True,
                           receive_shadow=True)
    mat_plain = sc.BlinnPhong(diffuse=sc.color_from_value(0.2, 0.5, 0.8, 1.0),
                              specular=sc.color_from_value(0.5, 0.5, 0.5, 1.0), shininess=16, receive_shadow=True)
    g = sc.Geometry(_mesh(tris, mats, cols), mat_ao, mat_plain)
    light = sc.Point(position=(0.5, 0.8, 4.0), intensity=1.0, cast_shadow=True)
    return sc.Scene(g, light, sc.Ambient(intensity=0.15))


def _cam():
    return sc.Perspective(position=(0, 0, 5), target=(0, 0, 0), up=(0, 1, 0), fov=60, aspect=W / H, near=0.1,
                          far=50)


@pytest.mark.parametrize("seed", [0xD0, 0xD1])
def test_stacked_layers_single_view(device, seed):
    s = _stack_scene(seed)
    p = Pair(device, options(s, _cam(), W, H, shadow_map=True, shadow_size=(1024, 1024)))
    gpu, cpu = p.frame(with_shadow_maps=True)
    assert_bitexact(gpu, cpu)
    # enough raster tasks for the single-view raster to take the early test
    assert p.stats["n_raster_tasks"] > 400_000, p.stats["n_raster_tasks"]
    # the duplicates' ties went to the first drawn, as the oracle says; and
    # most pixels see the front layers only
    assert (gpu["tri_id"] != 0xFFFFFFFF).mean() > 0.5


def test_stacked_layers_batch_matches_plain(device):
    scene = _stack_scene(0xD2)
    opts = options(scene, _cam(), W, H, shadow_map=True, shadow_size=(1024, 1024))
    specs = [(0, opts, pb.shadow_cams(opts))]
    outs_names = ("rgba", "tri_id", "depth")
    b = pb.Batch(0)
    try:
        b.add_scene(scene)
        arr, outs, keep = b.views(specs, outs_names)
        b.render(arr)
        got = {k: v.cpu().numpy() for k, v in outs[0].items()}
    finally:
        b.close()
    lib = native.load()
    flat = render.FlatScene(scene)
    d = flat.desc()
    native.check(lib.pr_scene_upload(device.handle, C.byref(d)))
    native.check(lib.pr_shadow_reset(device.handle))
    fd = render.FrameDesc(opts, specs[0][2])
    want = render.Outputs(W, H, outs_names)
    native.check(lib.pr_render(device.handle, C.byref(fd.desc), C.byref(want.desc)))
    for k in outs_names:
        g = got[k].view(np.uint32) if k == "tri_id" else got[k]
        eq = same_bits(g, want.arrays[k])
        assert eq.all(), (k, int((~eq).sum()))
