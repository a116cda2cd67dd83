"""pr_frame_submit: scene upload and frame in one call that does not wait.
Frames of alternating scenes submitted back to back (each upload overlapping
the previous frame) equal pr_scene_upload + pr_render of the same scene, bit
for bit, into page-locked host outputs, pageable host outputs and device
outputs."""
import ctypes as C

import numpy as np
import pytest

from helpers import options, shadow_cams
from polyred_gb300 import _abi, native, procedural, render

pytestmark = pytest.mark.gpu

W, H = 320, 200
NAMES = ("rgba", "tri_id", "depth", "world_pos")


def _scenes():
    a, cam_a = procedural.small_scene(W, H)
    b, cam_b = procedural.sphere_field(n_spheres=24, lon=20, lat=10, width=W, height=H)
    out = []
    for s, cam, kw in ((a, cam_a, {}), (b, cam_b, dict(shadow_map=True, directional_shadows=True, shadow_size=(256, 256)))):
        o = options(s, cam, W, H, **kw)
        flat = render.FlatScene(s)
        out.append((flat, flat.desc(), render.FrameDesc(o, shadow_cams(o))))
    return out


def test_frame_submit_matches_upload_and_render(device):
    lib = native.load()
    sc = _scenes()
    ref = []
    for flat, d, fd in sc:  # also sizes the capacities for both scenes
        native.check(lib.pr_scene_upload(device.handle, C.byref(d)))
        o = render.Outputs(W, H, NAMES)
        native.check(lib.pr_render(device.handle, C.byref(fd.desc), C.byref(o.desc)))
        ref.append(o.arrays)
    order = [0, 1, 0, 1, 1, 0]
    outs = [render.Outputs(W, H, NAMES, pinned=(k % 2 == 0)) for k in range(len(order))]
    for k, i in enumerate(order):
        _, d, fd = sc[i]
        native.check(lib.pr_frame_submit(device.handle, C.byref(d), C.byref(fd.desc), C.byref(outs[k].desc)))
    native.check(lib.pr_sync(device.handle))
    for k, i in enumerate(order):
        for n in NAMES:
            assert np.array_equal(outs[k].arrays[n].view(np.uint8), ref[i][n].view(np.uint8)), (k, n)
    assert (outs[1].arrays["tri_id"] != 0xFFFFFFFF).sum() > 1000


def test_frame_submit_device_outputs_then_sync_render(device):
    import torch
    lib = native.load()
    sc = _scenes()
    ref = []
    for flat, d, fd in sc:
        native.check(lib.pr_scene_upload(device.handle, C.byref(d)))
        o = render.Outputs(W, H, ("rgba",))
        native.check(lib.pr_render(device.handle, C.byref(fd.desc), C.byref(o.desc)))
        ref.append(o.arrays["rgba"])
    bufs = []
    for i in (1, 0, 1):
        _, d, fd = sc[i]
        t = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
        od = _abi.pr_outputs()
        od.size = C.sizeof(_abi.pr_outputs)
        od.flags = _abi.PR_OUT_DEVICE_PTRS
        od.rgba = t.data_ptr()
        native.check(lib.pr_frame_submit(device.handle, C.byref(d), C.byref(fd.desc), C.byref(od)))
        bufs.append((i, t, od))
    # a synchronous frame after submitted ones renders the last submitted scene
    o = render.Outputs(W, H, ("rgba",))
    native.check(lib.pr_render(device.handle, C.byref(sc[1][2].desc), C.byref(o.desc)))
    native.check(lib.pr_sync(device.handle))
    for i, t, _ in bufs:
        assert np.array_equal(t.cpu().numpy(), ref[i])
    # the last submit reset the shadow maps; the synchronous frame then shadows with fresh maps
    assert np.array_equal(o.arrays["rgba"], ref[1])
