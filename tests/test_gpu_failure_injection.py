"""Host-side failure injection: every device or page-locked allocation that
pr_create, pr_scene_upload, pr_render, pr_frame_submit and pr_batch_render
make is failed in turn (pr_testing_fail_alloc). The call that made it must
return PR_ERR_OOM with a detail string naming the allocation, and the same
context (or batch) must then render the frame bit for bit as an undisturbed
one does. Only host allocation results are faked: no kernel faults and no
device wait is cut short."""
import ctypes as C

import numpy as np
import pytest

from helpers import options, shadow_cams
from polyred_gb300 import _abi, batch as pb, native, procedural, render, scene as sc

pytestmark = pytest.mark.gpu

W, H = 160, 100
OUTS = ("rgba", "tri_id", "depth", "nor", "mat_id")


def _scene():
    s, cam = procedural.small_scene(W, H)
    for o, _ in s.iter_objects():
        if isinstance(o, sc.Point):
            o.cast_shadow = True
        if isinstance(o, sc.Geometry):
            for m in o.materials:
                m.receive_shadow = True
                m.ambient_occlusion = True
    opts = options(s, cam, W, H, shadow_map=True, shadow_size=(256, 256))
    return s, opts


def _oom(lib, rc):
    assert rc == _abi.PR_ERR_OOM, (rc, lib.pr_last_error())
    msg = lib.pr_last_error().decode()
    assert "cudaMalloc" in msg or "cudaHostAlloc" in msg or "pinned" in msg, msg
    assert "out of memory" in msg or "failed" in msg, msg


@pytest.fixture(autouse=True)
def _injection_off(native_lib):
    yield
    native_lib.pr_testing_fail_alloc(0)


def _frame(lib, h, flat, opts):
    fd = render.FrameDesc(opts, shadow_cams(opts))
    out = render.Outputs(W, H, OUTS)
    native.check(lib.pr_shadow_reset(h))
    rc = lib.pr_render(h, C.byref(fd.desc), C.byref(out.desc))
    return rc, out.arrays


def _same(a, b):
    for k in OUTS:
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k


def test_every_allocation_of_a_frame_can_fail_and_recover(native_lib):
    lib = native_lib
    s, opts = _scene()
    flat = render.FlatScene(s)
    desc = flat.desc()
    # an undisturbed context: the reference frame and the allocation count
    n0 = lib.pr_testing_alloc_count()
    h = C.c_void_p()
    native.check(lib.pr_create(0, C.byref(h)))
    native.check(lib.pr_scene_upload(h, C.byref(desc)))
    rc, want = _frame(lib, h, flat, opts)
    native.check(rc)
    native.check(lib.pr_destroy(h))
    n_alloc = lib.pr_testing_alloc_count() - n0
    assert n_alloc >= 20
    assert (want["tri_id"] != 0xFFFFFFFF).sum() > 1000
    failed = {"create": 0, "upload": 0, "render": 0}
    for k in range(1, n_alloc + 1):
        native.check(lib.pr_testing_fail_alloc(k))
        h = C.c_void_p()
        rc = lib.pr_create(0, C.byref(h))
        if rc != _abi.PR_OK:
            _oom(lib, rc)
            assert not h.value
            failed["create"] += 1
            continue
        try:
            rc = lib.pr_scene_upload(h, C.byref(desc))
            if rc != _abi.PR_OK:
                _oom(lib, rc)
                failed["upload"] += 1
                # no scene is left behind: a frame now reports it
                lib.pr_testing_fail_alloc(0)
                rc2, _ = _frame(lib, h, flat, opts)
                assert rc2 == _abi.PR_ERR_NO_SCENE, rc2
                native.check(lib.pr_scene_upload(h, C.byref(desc)))
            rc, got = _frame(lib, h, flat, opts)
            if rc != _abi.PR_OK:
                _oom(lib, rc)
                failed["render"] += 1
                lib.pr_testing_fail_alloc(0)
                rc, got = _frame(lib, h, flat, opts)
                native.check(rc)
            _same(got, want)
            # and the next frame of the same context as well
            lib.pr_testing_fail_alloc(0)
            rc, got = _frame(lib, h, flat, opts)
            native.check(rc)
            _same(got, want)
        finally:
            lib.pr_testing_fail_alloc(0)
            native.check(lib.pr_destroy(h))
    assert failed["create"] >= 2 and failed["upload"] >= 5 and failed["render"] >= 10, failed


def test_a_grown_frame_recovers_after_failures(native_lib):
    """Failures while a context grows from a small frame to a larger one
    (buffers reallocated, shadow maps re-laid out) leave it able to render
    both sizes."""
    lib = native_lib
    s, opts = _scene()
    flat = render.FlatScene(s)
    desc = flat.desc()
    big = dict(opts, width=2 * W, height=2 * H, shadow_size=(512, 512))

    def frame(h, o):
        fd = render.FrameDesc(o, shadow_cams(o))
        out = render.Outputs(o["width"], o["height"], OUTS)
        native.check(lib.pr_shadow_reset(h))
        return lib.pr_render(h, C.byref(fd.desc), C.byref(out.desc)), out.arrays

    d = render.Device(0)
    try:
        native.check(lib.pr_scene_upload(d.handle, C.byref(desc)))
        rc, small = frame(d.handle, opts)
        native.check(rc)
        n0 = lib.pr_testing_alloc_count()
        rc, want_big = frame(d.handle, big)
        native.check(rc)
        n_grow = lib.pr_testing_alloc_count() - n0
    finally:
        d.close()
    assert n_grow >= 5
    for k in range(1, n_grow + 1):
        d = render.Device(0)
        try:
            native.check(lib.pr_scene_upload(d.handle, C.byref(desc)))
            rc, got = frame(d.handle, opts)
            native.check(rc)
            native.check(lib.pr_testing_fail_alloc(k))
            rc, got = frame(d.handle, big)
            lib.pr_testing_fail_alloc(0)
            if rc != _abi.PR_OK:
                _oom(lib, rc)
            for o, want in ((opts, small), (big, want_big), (opts, small)):
                rc, got = frame(d.handle, o)
                native.check(rc)
                _same(got, want)
        finally:
            lib.pr_testing_fail_alloc(0)
            d.close()


def test_frame_submit_allocation_failures(native_lib):
    lib = native_lib
    s, opts = _scene()
    flat = render.FlatScene(s)
    desc = flat.desc()
    fd = render.FrameDesc(opts, shadow_cams(opts))
    ref = render.Device(0)
    try:
        native.check(lib.pr_scene_upload(ref.handle, C.byref(desc)))
        want = render.Outputs(W, H, OUTS)
        native.check(lib.pr_render(ref.handle, C.byref(fd.desc), C.byref(want.desc)))
    finally:
        ref.close()
    d = render.Device(0)
    try:
        out = render.Outputs(W, H, OUTS, pinned=True)
        n0 = lib.pr_testing_alloc_count()
        native.check(lib.pr_shadow_reset(d.handle))
        native.check(lib.pr_frame_submit(d.handle, C.byref(desc), C.byref(fd.desc), C.byref(out.desc)))
        native.check(lib.pr_sync(d.handle))
        n_sub = lib.pr_testing_alloc_count() - n0
        assert n_sub >= 5
    finally:
        d.close()
    for k in range(1, n_sub + 1):
        d = render.Device(0)
        try:
            out = render.Outputs(W, H, OUTS, pinned=True)
            native.check(lib.pr_testing_fail_alloc(k))
            native.check(lib.pr_shadow_reset(d.handle))
            rc = lib.pr_frame_submit(d.handle, C.byref(desc), C.byref(fd.desc), C.byref(out.desc))
            lib.pr_testing_fail_alloc(0)
            native.check(lib.pr_sync(d.handle))
            if rc != _abi.PR_OK:
                _oom(lib, rc)
                native.check(lib.pr_shadow_reset(d.handle))
                native.check(lib.pr_frame_submit(d.handle, C.byref(desc), C.byref(fd.desc), C.byref(out.desc)))
                native.check(lib.pr_sync(d.handle))
            _same(out.arrays, want.arrays)
        finally:
            lib.pr_testing_fail_alloc(0)
            d.close()


def test_batch_allocation_failures(native_lib):
    lib = native_lib
    scenes, specs = [], []
    for si, n in enumerate((2_000, 6_000)):
        s = pb.sphere_scene(n, 0x5EED0004 + si, n_lights=3)
        scenes.append(s)
        for cam in pb.ring_cameras(2, W, H, radius=12.0):
            o = pb.view_opts(s, cam, W, H, 256)
            specs.append((si, o, pb.shadow_cams(o)))
    b = pb.Batch(0)
    for s in scenes:
        b.add_scene(s)
    arr, outs, keep = b.views(specs, OUTS)
    b.render(arr)
    want = [{k: v.cpu().numpy() for k, v in o.items()} for o in outs]
    b.close()

    n_render = None
    k = 0
    while n_render is None or k < n_render:
        b = pb.Batch(0)
        try:
            for s in scenes:
                b.add_scene(s)
            arr, outs, keep = b.views(specs, OUTS)
            if n_render is None:  # the allocations of the batch's first render
                n0 = lib.pr_testing_alloc_count()
                b.render(arr)
                n_render = lib.pr_testing_alloc_count() - n0
                assert n_render >= 10
                continue
            k += 1
            native.check(lib.pr_testing_fail_alloc(k))
            rc = lib.pr_batch_render(b.handle, len(arr), arr)
            lib.pr_testing_fail_alloc(0)
            if rc != _abi.PR_OK:
                _oom(lib, rc)
                b.render(arr)
            for o, w in zip(outs, want):
                _same({n: v.cpu().numpy() for n, v in o.items()}, w)
        finally:
            lib.pr_testing_fail_alloc(0)
            b.close()
