"""The batched workload at its stated size: 32 sphere scenes of 1k-500k
triangles, 8 ring views each (256 views of 1280x720), 16 casting point
lights per scene with 1024^2 shadow maps, AO, in one pr_batch_render. A
deterministic sample of views from every scene-size bucket is compared bit
for bit with pr_render of the same view on a fresh context, and two views
with the oracle."""
import ctypes as C

import numpy as np
import pytest

from helpers import THREADS, assert_bitexact, same_bits
from polyred_gb300 import batch as pb, native, render

pytestmark = pytest.mark.gpu

OUTS = ("rgba", "tri_id", "depth", "nor", "mat_id")


def _bucket(n):
    return 0 if n < 10_000 else (1 if n < 100_000 else 2)


@pytest.fixture(scope="module")
def full_batch(device):
    scenes, specs = pb.config4()
    b = pb.Batch(0)
    for s in scenes:
        b.add_scene(s)
    arr, outs, keep = b.views(specs, OUTS)
    b.render(arr)
    st = b.stats()
    sizes = [render.FlatScene(s).n_tris for s in scenes]
    keepers = set(_sample(specs, sizes)) | set(_oracle_views(specs, sizes))
    res = {k: {n: v.cpu().numpy() for n, v in outs[k].items()} for k in keepers}
    b.close()
    del outs, keep, arr
    return scenes, specs, res, st, sizes


def _sample(specs, sizes):
    """Two views of every other scene (views (s mod 8) and (s + 4) mod 8),
    32 views over the 16 scenes, every size bucket included."""
    picks = []
    for si in range(0, len(sizes), 2):
        mine = [k for k, sp in enumerate(specs) if sp[0] == si]
        picks += [mine[si % 8], mine[(si + 4) % 8]]
    assert {_bucket(sizes[specs[k][0]]) for k in picks} == {0, 1, 2}
    return picks


def _oracle_views(specs, sizes):
    """View 3 of the smallest scene and of a median-size one."""
    order = np.argsort(sizes)
    return [[j for j, sp in enumerate(specs) if sp[0] == si][3] for si in (int(order[0]), int(order[len(order) // 2]))]


def test_full_batch_matches_plain_per_view(device, full_batch):
    scenes, specs, res, st, sizes = full_batch
    assert st["n_views"] == 256 and st["n_passes"] == 256 + 256 * 16
    lib = native.load()
    picks = _sample(specs, sizes)
    assert len(picks) >= 16
    by_scene = {}
    for k in picks:
        by_scene.setdefault(specs[k][0], []).append(k)
    for si, ks in by_scene.items():
        d = render.Device(0)  # a fresh context per scene
        try:
            flat = render.FlatScene(scenes[si])
            desc = flat.desc()
            native.check(lib.pr_scene_upload(d.handle, C.byref(desc)))
            for k in ks:
                _, opts, cams = specs[k]
                fd = render.FrameDesc(opts, cams)
                out = render.Outputs(opts["width"], opts["height"], OUTS)
                native.check(lib.pr_shadow_reset(d.handle))
                native.check(lib.pr_render(d.handle, C.byref(fd.desc), C.byref(out.desc)))
                for name in OUTS:
                    got = res[k][name].view(np.uint32) if name == "tri_id" else res[k][name]
                    eq = same_bits(got, out.arrays[name])
                    assert eq.all(), (k, sizes[si], name, int((~eq).sum()))
                assert (out.arrays["tri_id"] != 0xFFFFFFFF).sum() > 1000
        finally:
            d.close()


def test_full_batch_views_match_the_oracle(full_batch):
    import oracle
    scenes, specs, res, st, sizes = full_batch
    for k in _oracle_views(specs, sizes):
        si, opts, cams = specs[k]
        flat = render.FlatScene(scenes[si])
        fd = render.FrameDesc(opts, cams)
        src, _ = opts["scene"].lights()
        sw, sh = opts["shadow_size"]
        state = np.zeros((len(src), sh, sw), np.float32)
        cpu = render.Outputs(opts["width"], opts["height"], OUTS)
        oracle.render(flat.desc(), fd.desc, cpu.desc, shadow_state=state, threads=THREADS)
        got = dict(res[k])
        got["tri_id"] = got["tri_id"].view(np.uint32)
        assert_bitexact(got, cpu.arrays, list(OUTS))
