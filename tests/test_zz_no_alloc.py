"""pr_depth_map_noalloc: the allocation-free depth-map raster.

Some callers cannot allocate device memory — their device memory belongs to
another allocator, or their frame loop cannot pay for cudaMalloc/cudaFree.
For them the library offers this one entry point, which keeps all its scratch
in a fixed static device array. This test calls it through the C ABI and
compares its depth map with the shadow map pr_render computes for the same
light camera, on two calls in a row (the map persists between calls, as the
reference's shadow maps do). It runs last so that a failure here leaves the
rest of the suite already run, and it passes alone or after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import same_bits
from polyred_gb300 import _abi, native, procedural, render, scene as sc

pytestmark = pytest.mark.gpu

SW = SH = 512


def _scene():
    s, cam = procedural.sphere_field(n_spheres=12, lon=24, lat=12, width=320, height=180, ao=False,
                                     directional_shadow=False)
    return s, cam


def _light_camera(scene, light_pos):
    """An orthographic light camera framing the spheres, with its depth range
    chosen so their depths are positive (the maps start at 0 and keep only
    greater depths)."""
    from polyred_gb300 import pmath
    view = pmath.view_matrix(np.asarray(light_pos, np.float32), scene.center(), np.array([0, 1, 0], np.float32))
    proj = pmath.orthographic_matrix(-14, 14, -14, 14, 10, -200)
    return view, proj


def test_depth_map_noalloc_matches_render(device):
    import torch

    lib = native.load()
    s, cam = _scene()
    flat = render.FlatScene(s)
    assert flat.n_tris <= _abi.PR_NOALLOC_MAX_TRIS
    d = flat.desc()
    native.check(lib.pr_scene_upload(device.handle, C.byref(d)))
    native.check(lib.pr_shadow_reset(device.handle))
    opts = dict(width=320, height=180, camera=cam, scene=s, perspective=True, shadow_map=True, gamma=True,
                background=(0, 0, 0, 0), shadow_size=(SW, SH), directional_shadows=False)
    src, _ = s.lights()
    assert isinstance(src[0], sc.Point) and src[0].cast_shadow

    pos = torch.from_numpy(np.ascontiguousarray(flat.pos)).cuda()
    depth = torch.zeros((SH, SW), dtype=torch.float32, device="cuda")

    for light_pos in ([14, 18, 12], [-9, 15, 6]):  # the second call moves the light
        view, proj = _light_camera(s, light_pos)
        # existing entry point: pr_render's shadow map of light 0
        fd = render.FrameDesc(opts, {0: (view, proj)})
        out = render.Outputs(320, 180, ("rgba", "shadow_maps"), n_shadow=len(src), shadow_size=(SW, SH))
        native.check(lib.pr_render(device.handle, C.byref(fd.desc), C.byref(out.desc)))
        want = out.arrays["shadow_maps"][0]

        # the allocation-free entry point on caller-owned device buffers
        nd = _abi.pr_depth_map_desc()
        nd.size = C.sizeof(_abi.pr_depth_map_desc)
        nd.n_tris = flat.n_tris
        nd.n_objects = flat.n_objects
        nd.width, nd.height = SW, SH
        nd.pos = pos.data_ptr()
        nd.objects = flat.objects
        for k in range(16):
            nd.view[k] = float(view[k])
            nd.proj[k] = float(proj[k])
        nd.depth = depth.data_ptr()
        nd.stream = None
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        native.check(lib.pr_depth_map_noalloc(C.byref(nd)))
        free1 = torch.cuda.mem_get_info()[0]
        got = depth.cpu().numpy()
        assert (want != 0).sum() > 5000
        assert same_bits(got, want).all(), int((~same_bits(got, want)).sum())
        if light_pos[0] < 0:  # the second call: nothing on the device was allocated for it
            assert free1 == free0, (free0, free1)


def test_depth_map_noalloc_rejects_oversized_input(native_lib):
    nd = _abi.pr_depth_map_desc()
    nd.size = C.sizeof(_abi.pr_depth_map_desc)
    nd.n_tris = _abi.PR_NOALLOC_MAX_TRIS + 1
    nd.n_objects = 1
    nd.width = nd.height = 16
    assert native_lib.pr_depth_map_noalloc(C.byref(nd)) == _abi.PR_ERR_INVALID_ARG
    assert b"PR_NOALLOC_MAX_TRIS" in native_lib.pr_last_error()
    nd.n_tris = 0
    nd.width, nd.height = 2048, 1024  # 2M texels > PR_NOALLOC_MAX_TEXELS
    assert native_lib.pr_depth_map_noalloc(C.byref(nd)) == _abi.PR_ERR_INVALID_ARG
    assert b"PR_NOALLOC_MAX_TEXELS" in native_lib.pr_last_error()


def _desc(n_tris, objects, width, height, view, proj, pos_ptr, depth_ptr):
    nd = _abi.pr_depth_map_desc()
    nd.size = C.sizeof(_abi.pr_depth_map_desc)
    nd.n_tris = n_tris
    nd.n_objects = len(objects)
    nd.width, nd.height = width, height
    nd.pos = pos_ptr
    nd.objects = objects
    for k in range(16):
        nd.view[k] = float(view[k])
        nd.proj[k] = float(proj[k])
    nd.depth = depth_ptr
    nd.stream = None
    return nd


def _objects(n_tris):
    objs = (_abi.pr_object * 1)()
    objs[0].first_tri, objs[0].n_tris, objs[0].mat_base = 0, n_tris, 0
    for k in range(16):
        objs[0].model[k] = 1.0 if k % 5 == 0 else 0.0
    return objs


def _soup(tris):
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    pos = np.ones((t.shape[0], 3, 4), np.float32)
    pos[..., :3] = t
    return pos


def _ortho():
    from polyred_gb300 import pmath
    view = pmath.view_matrix(np.array([0, 0, 5], np.float32), np.zeros(3, np.float32), np.array([0, 1, 0], np.float32))
    proj = pmath.orthographic_matrix(-2, 2, -2, 2, 1, -20)
    return view, proj


def test_depth_map_noalloc_overflow_leaves_the_map_unchanged(native_lib):
    """More raster tasks than PR_NOALLOC_MAX_TASKS: 260 triangles that each
    cover the whole 1024 x 1024 map need 1024 tasks apiece (each is given in
    both windings, one of which the back-face cull drops). The call reports
    PR_ERR_OVERFLOW and the map keeps every bit (NaN payloads and -0
    included)."""
    import torch
    lib = native_lib
    pairs = 260
    big = []
    for k in range(pairs):
        a, b, c = [-3, -3, -1 + k / pairs], [3, -3, -1 + k / pairs], [0, 4, -1 + k / pairs]
        big += [[a, b, c], [a, c, b]]
    n = len(big)
    pos = torch.from_numpy(_soup(big)).cuda()
    g = np.random.default_rng(7)
    init = g.uniform(-1, 1, (1024, 1024)).astype(np.float32)
    init[::7, ::5] = -0.0
    init.view(np.uint32)[3::11, 2::13] = 0x7FA00001
    depth = torch.from_numpy(init.copy()).cuda()
    view, proj = _ortho()
    objs = _objects(n)
    nd = _desc(n, objs, 1024, 1024, view, proj, pos.data_ptr(), depth.data_ptr())
    assert lib.pr_depth_map_noalloc(C.byref(nd)) == _abi.PR_ERR_OVERFLOW
    assert b"PR_NOALLOC_MAX_TASKS" in lib.pr_last_error()
    assert np.array_equal(depth.cpu().numpy().view(np.uint32), init.view(np.uint32))
    # within the limit (200 covering triangles) the same kind of call succeeds
    nd.n_tris = 400
    objs[0].n_tris = 400
    native.check(lib.pr_depth_map_noalloc(C.byref(nd)))
    got = depth.cpu().numpy()
    assert (got.view(np.uint32) != init.view(np.uint32)).sum() > 100_000


def test_depth_map_noalloc_keeps_untouched_texels(native_lib):
    """Texels no fragment reaches keep their bits, -0 and NaN payloads
    included, as the reference's map does (only a store changes a texel)."""
    import torch
    lib = native_lib
    g = np.random.default_rng(3)
    tris = []
    for _ in range(400):  # all in x < -0.1: the left part of the map
        c = np.array([g.uniform(-1.8, -0.4), g.uniform(-1.7, 1.7), g.uniform(-1, 1)])
        tris.append([c, c + g.normal(0, 0.1, 3), c + g.normal(0, 0.1, 3)])
    tris = np.clip(np.array(tris), [-1.95, -1.95, -1.5], [-0.15, 1.95, 1.5])
    pos = torch.from_numpy(_soup(tris)).cuda()
    W, H = 256, 256
    init = np.zeros((H, W), np.float32)
    right = np.s_[:, W // 2:]
    init[right] = -0.0
    init.view(np.uint32)[:, W // 2::3] = 0x7FA00001 + np.arange(H, dtype=np.uint32)[:, None]
    depth = torch.from_numpy(init.copy()).cuda()
    view, proj = _ortho()
    nd = _desc(len(tris), _objects(len(tris)), W, H, view, proj, pos.data_ptr(), depth.data_ptr())
    native.check(lib.pr_depth_map_noalloc(C.byref(nd)))
    got = depth.cpu().numpy()
    assert (got[:, : W // 2] != 0).sum() > 1000
    assert np.array_equal(got[right].view(np.uint32), init[right].view(np.uint32))


def test_depth_map_noalloc_with_nan_texels_matches_render(device, native_lib):
    """A map already holding NaN texels (left by NaN-depth fragments of
    collapsed triangles in an earlier pass): the call continues it as
    pr_render's persistent map continues into the next frame."""
    import torch
    from test_gpu_parity import _basic_material, _degenerate_scene, _mesh, _ortho_cam
    lib = native_lib
    m = _basic_material(receive_shadow=True)
    geo = sc.Geometry(_mesh(_degenerate_scene(9)), m)
    s = sc.Scene(geo, sc.Point(position=(0, 0, 5), cast_shadow=True), sc.Ambient(0.1))
    cam = _ortho_cam()
    W, H = 160, 128
    flat = render.FlatScene(s)
    d = flat.desc()
    native.check(lib.pr_scene_upload(device.handle, C.byref(d)))
    native.check(lib.pr_shadow_reset(device.handle))
    opts = dict(width=W, height=H, camera=cam, scene=s, perspective=False, shadow_map=True, gamma=True,
                background=(0, 0, 0, 0), shadow_size=None)
    view, proj = cam.view_matrix(), cam.proj_matrix()
    fd = render.FrameDesc(opts, {0: (view, proj)})
    maps = []
    for _ in range(2):
        out = render.Outputs(W, H, ("rgba", "shadow_maps"), n_shadow=1, shadow_size=(W, H))
        native.check(lib.pr_render(device.handle, C.byref(fd.desc), C.byref(out.desc)))
        maps.append(out.arrays["shadow_maps"][0].copy())
    assert np.isnan(maps[0]).any()
    pos = torch.from_numpy(np.ascontiguousarray(flat.pos)).cuda()
    depth = torch.from_numpy(maps[0].copy()).cuda()
    nd = _desc(flat.n_tris, flat.objects, W, H, view, proj, pos.data_ptr(), depth.data_ptr())
    nd.n_objects = flat.n_objects
    native.check(lib.pr_depth_map_noalloc(C.byref(nd)))
    got = depth.cpu().numpy()
    want = maps[1]
    a = np.where(got == 0, np.float32(0), got)
    b = np.where(want == 0, np.float32(0), want)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    assert np.array_equal(np.nan_to_num(a, nan=-7.0).view(np.uint32), np.nan_to_num(b, nan=-7.0).view(np.uint32))
