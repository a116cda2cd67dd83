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
        native.check(lib.pr_depth_map_noalloc(C.byref(nd)))
        got = depth.cpu().numpy()
        assert (want != 0).sum() > 5000
        assert same_bits(got, want).all(), int((~same_bits(got, want)).sum())


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
