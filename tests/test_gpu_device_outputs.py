"""Device-resident outputs through the C ABI alone (pr_device_alloc /
pr_device_read / pr_device_free): a frame rendered into library-allocated
device memory and read back field by field equals the same frame rendered
into host memory."""
import ctypes as C

import numpy as np
import pytest

from helpers import options
from polyred_gb300 import _abi, native, procedural, render

pytestmark = pytest.mark.gpu

FIELDS = [("rgba", 4, np.uint8, 4), ("tri_id", 4, np.uint32, 1), ("depth", 4, np.float32, 1),
          ("nor", 16, np.float32, 4), ("uvd", 16, np.float32, 4), ("mat_id", 4, np.int32, 1)]


def test_device_outputs_read_back(device):
    lib = native.load()
    W, H = 160, 100
    s, cam = procedural.small_scene(W, H)
    flat = render.FlatScene(s)
    d = flat.desc()
    native.check(lib.pr_scene_upload(device.handle, C.byref(d)))
    fd = render.FrameDesc(options(s, cam, W, H), {})
    host = render.Outputs(W, H, tuple(f[0] for f in FIELDS))
    native.check(lib.pr_render(device.handle, C.byref(fd.desc), C.byref(host.desc)))

    ptrs = {}
    try:
        od = _abi.pr_outputs()
        od.size = C.sizeof(_abi.pr_outputs)
        od.flags = _abi.PR_OUT_DEVICE_PTRS
        for name, size, _, _ in FIELDS:
            p = C.c_void_p()
            native.check(lib.pr_device_alloc(device.handle, W * H * size, C.byref(p)))
            ptrs[name] = p
            setattr(od, name, p.value)
        native.check(lib.pr_render(device.handle, C.byref(fd.desc), C.byref(od)))
        for name, size, dt, k in FIELDS:
            got = np.zeros((H, W, k) if k > 1 else (H, W), dt)
            native.check(lib.pr_device_read(device.handle, ptrs[name], W * H * size, got.ctypes.data))
            assert np.array_equal(got.view(np.uint8), host.arrays[name].view(np.uint8)), name
        # one fragment's depth at an offset, as a FragmentBuffer view reads it
        i = int(np.argmax(host.arrays["tri_id"] != _abi.PR_TRI_NONE))
        one = np.zeros(1, np.float32)
        native.check(lib.pr_device_read(device.handle, ptrs["depth"].value + 4 * i, 4, one.ctypes.data))
        assert one.view(np.uint32)[0] == host.arrays["depth"].reshape(-1)[i:i + 1].view(np.uint32)[0]
    finally:
        for p in ptrs.values():
            native.check(lib.pr_device_free(device.handle, p))
