"""Batched rendering (pr_batch_*): every view's outputs equal pr_render's for
that view on a fresh context (first-frame shadow maps), bit for bit; the
captured graph is relaunched for an unchanged batch; capacities grow when a
pass overflows; the autotuner keeps results unchanged."""
import ctypes as C

import numpy as np
import pytest

from helpers import same_bits
from polyred_gb300 import batch as pb, native, procedural, render, scene as sc

pytestmark = pytest.mark.gpu

OUTS = ("rgba", "tri_id", "depth", "nor", "world_pos", "mat_id")


def _plain(device, scene, specs):
    """pr_render of each view on one fresh context per scene."""
    lib = native.load()
    flat = render.FlatScene(scene)
    d = flat.desc()
    native.check(lib.pr_scene_upload(device.handle, C.byref(d)))
    res = []
    for _, opts, cams in specs:
        fd = render.FrameDesc(opts, cams)
        out = render.Outputs(opts["width"], opts["height"], OUTS)
        native.check(lib.pr_shadow_reset(device.handle))
        native.check(lib.pr_render(device.handle, C.byref(fd.desc), C.byref(out.desc)))
        res.append(out.arrays)
    return res


def _small_batch(W=320, H=180, shadow=256, n_lights=4, counts=(2_000, 9_000, 30_000), views=2, ground=False):
    scenes, specs = [], []
    for si, n in enumerate(counts):
        s = pb.sphere_scene(n, 0x5EED0004 + si, n_lights=n_lights)
        if ground:
            s.add(sc.Geometry(procedural.ground_plane(20.0, -3.0)))
        scenes.append(s)
        for cam in pb.ring_cameras(views, W, H, radius=12.0):
            o = pb.view_opts(s, cam, W, H, shadow)
            specs.append((si, o, pb.shadow_cams(o)))
    return scenes, specs


def _check(device, b, scenes, specs, outs):
    for si, s in enumerate(scenes):
        mine = [k for k, sp in enumerate(specs) if sp[0] == si]
        want = _plain(device, s, [specs[k] for k in mine])
        for k, w in zip(mine, want):
            for name in OUTS:
                got = outs[k][name].cpu().numpy()
                if name == "tri_id":
                    got = got.view(np.uint32)
                eq = same_bits(got, w[name])
                assert eq.all(), (k, name, int((~eq).sum()))


def test_batch_matches_plain(device):
    scenes, specs = _small_batch()
    b = pb.Batch(0)
    for s in scenes:
        b.add_scene(s)
    arr, outs, keep = b.views(specs, OUTS)
    b.render(arr)
    st = b.stats()
    assert st["n_views"] == 6 and st["n_passes"] == 6 + 6 * 4
    assert st["n_fallback_views"] == 0
    _check(device, b, scenes, specs, outs)
    # the same batch again: the captured graph is relaunched, results unchanged
    first = [{k: v.clone() for k, v in o.items()} for o in outs]
    b.render(arr)
    assert b.stats()["graph_reused"] == 1
    for a, o in zip(first, outs):
        for k in OUTS:
            assert same_bits(a[k].cpu().numpy(), o[k].cpu().numpy()).all(), k
    b.close()


def test_batch_capacity_growth(device):
    """Capacities the tuner sized on 320x180 views are far too small for the
    same views at 3840x2160, where a ground plane needs thousands of raster
    tasks: the batch grows them and runs again."""
    small_scenes, small = _small_batch(W=320, H=180, counts=(1_000, 4_000), views=2, ground=True)
    scenes, big = _small_batch(W=3840, H=2160, counts=(1_000, 4_000), views=2, ground=True)
    b = pb.Batch(0)
    for s in scenes:
        b.add_scene(s)
    arr_s, _, keep_s = b.views(small, ("rgba",))
    b.tune(arr_s)
    arr, outs, keep = b.views(big, OUTS)
    b.render(arr)
    assert b.stats()["n_retries"] >= 1
    _check(device, b, scenes, big, outs)
    b.close()


def test_batch_tune_keeps_results(device):
    scenes, specs = _small_batch(counts=(3_000, 12_000), views=2)
    b = pb.Batch(0)
    for s in scenes:
        b.add_scene(s)
    arr, outs, keep = b.views(specs, OUTS)
    rep = b.tune(arr)
    assert len(rep["candidates"]) == 15
    assert rep["task_px"] in (32, 64, 256, 1024, 4096)
    b.render(arr)
    assert b.stats()["task_px"] == rep["task_px"]
    _check(device, b, scenes, specs, outs)
    b.close()
