"""MSAA (render.MSAA(n), render/raster.go:147-151 and 361-378): frames that
render at n times the image size, with the reference's viewport test and
clipping at n times the framebuffer, then imageutil.Resize to the image.
Every output bit-exact against the oracle: the image at width x height, the
G-buffer fields and shadow maps at the framebuffer size."""
import numpy as np
import pytest

from helpers import Pair, assert_bitexact, options
from polyred_gb300 import objload, procedural, render, scene as sc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m", [2, 3])
def test_msaa_small_scene_bitexact(device, m):
    s, cam = procedural.small_scene(width=320, height=200)
    for o, _ in s.iter_objects():
        if isinstance(o, sc.Point):
            o.cast_shadow = True
    p = Pair(device, options(s, cam, 320, 200, msaa=m, shadow_map=True))
    for _ in range(2):  # persistent shadow maps at the framebuffer size
        gpu, cpu = p.frame(with_shadow_maps=True)
        assert gpu["rgba"].shape == (200, 320, 4) and gpu["tri_id"].shape == (200 * m, 320 * m)
        assert_bitexact(gpu, cpu)
    assert p.stats["n_clipped_tris"] > 0  # the ground crosses the extent


def test_msaa_4_obj_tori(device, tmp_path):
    obj, mtl, _ = procedural.obj_tori(6, 24, 12)
    (tmp_path / "tori.obj").write_bytes(obj)
    (tmp_path / "tori.mtl").write_bytes(mtl)
    s, cam = procedural.obj_tori_scene(objload.load(str(tmp_path / "tori.obj")), 320, 180)
    p = Pair(device, options(s, cam, 320, 180, msaa=4, shadow_map=True))
    gpu, cpu = p.frame()
    assert_bitexact(gpu, cpu)


def test_msaa_renderer_api(device):
    """NewRenderer(..., MSAA(2)).Render() returns the width x height image."""
    s, cam = procedural.small_scene(width=200, height=120)
    r = render.NewRenderer(render.Size(200, 120), render.Camera(cam), render.Scene(s), render.MSAA(2),
                           render.GammaCorrection(True), render.CUDA(device))
    img = r.Render()
    assert img.shape == (120, 200, 4)
    assert r.tri_id().shape == (240, 400)
    p = Pair(device, options(s, cam, 200, 120, msaa=2), outputs=("rgba",))
    gpu, cpu = p.frame()
    assert np.array_equal(img, cpu["rgba"])
