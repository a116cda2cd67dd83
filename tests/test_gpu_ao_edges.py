"""AmbientOcclusionShade's march (material/ao.go:41-72) where its device
shortcuts meet their edges, bit-exact with the oracle: a dense triangle soup
(depth jumps at every tap, many candidate taps and settled groups), a ground
with spheres seen at grazing and steep angles (long runs of smoothly rising
depth next to sudden occluders), and frames whose every pixel has x or y
below 256, where the tiny components of cos(Pi/2) and sin(Pi) move the taps
to the adjacent column or row within the 100 taps, at odd sizes (taps that
leave the frame early, binary-searched march ends)."""
import numpy as np
import pytest

from helpers import Pair, assert_bitexact, options
from polyred_gb300 import procedural, scene as sc

pytestmark = pytest.mark.gpu


def _ao_material():
    return sc.BlinnPhong(diffuse=sc.color_from_value(0.8, 0.3, 0.2, 1.0), specular=sc.color_from_value(0.5, 0.5, 0.5, 1.0),
                         shininess=32, ambient_occlusion=True)


def _scene(W, H, eye, seed=0xA0E5, n=40, m=None):
    """A ground plane in front of the camera and spheres of several sizes."""
    m = _ao_material() if m is None else m
    objs = [sc.Geometry(procedural.ground_plane(30.0, -1.0, material_id=0), m).translate(0.0, 0.0, -14.0)]
    rng = np.random.default_rng(seed)
    for _ in range(n):
        r = float(rng.uniform(0.3, 1.5))
        objs.append(sc.Geometry(procedural.uv_sphere(20, 10, r), m).translate(float(rng.uniform(-8, 8)), r - 1.0,
                                                                                float(rng.uniform(-10, 3))))
    s = sc.Scene(*objs, sc.Point(position=(4, 6, 3)), sc.Ambient(intensity=0.2))
    cam = sc.Perspective(position=eye, target=(0, -0.5, -2), up=(0, 1, 0), fov=60, aspect=W / H, near=0.1, far=100)
    return s, cam


def _frame(device, s, cam, W, H, min_cover):
    gpu, cpu = Pair(device, options(s, cam, W, H)).frame()
    assert_bitexact(gpu, cpu)
    assert (gpu["tri_id"] != 0xFFFFFFFF).mean() >= min_cover


def test_dense_soup_with_ao(device):
    W, H = 320, 180
    mesh = procedural.triangle_soup(60_000, W, H, seed=0x5EED0A01)
    s = sc.Scene(sc.Geometry(mesh, _ao_material()), sc.Point(position=(0, 5, 5)), sc.Ambient(intensity=0.1))
    cam = sc.Perspective(position=(0, 0, 0), target=(0, 0, -1), up=(0, 1, 0), fov=60, aspect=W / H, near=0.1,
                         far=120)
    _frame(device, s, cam, W, H, 0.5)


@pytest.mark.parametrize("W,H", [(61, 47), (200, 9), (9, 200), (333, 187)])
def test_edges_and_partial_blocks_with_ao(device, W, H):
    s, cam = _scene(W, H, (5.0, 1.0, 4.0))
    _frame(device, s, cam, W, H, 0.4)


@pytest.mark.parametrize("eye", [(0.0, 0.4, 6.0), (5.0, 1.0, 4.0), (-3.0, 6.0, 6.0)])
def test_grazing_and_steep_views_with_ao(device, eye):
    W, H = 256, 160
    s, cam = _scene(W, H, eye)
    _frame(device, s, cam, W, H, 0.3)


def test_scene_without_ao_material_skips_the_march(device):
    """A scene none of whose materials has AO lists no pixel: the march and
    the colour scaling are left out (two launches fewer) and the frame stays
    bit-exact; uploading an AO scene into the same context brings them back."""
    W, H = 160, 120
    s_ao, cam = _scene(W, H, (5.0, 1.0, 4.0), n=12)
    plain = sc.BlinnPhong(diffuse=sc.color_from_value(0.8, 0.3, 0.2, 1.0),
                          specular=sc.color_from_value(0.5, 0.5, 0.5, 1.0), shininess=32)
    s_plain, _ = _scene(W, H, (5.0, 1.0, 4.0), n=12, m=plain)
    stats = []
    for s in (s_ao, s_plain, s_ao):
        p = Pair(device, options(s, cam, W, H))
        gpu, cpu = p.frame()
        assert_bitexact(gpu, cpu)
        stats.append(p.stats)
    assert stats[0]["n_ao_pixels"] > 0 and stats[0]["ms_ao"] > 0
    assert stats[1]["n_ao_pixels"] == 0 and stats[1]["ms_ao"] == 0
    assert stats[1]["n_kernel_launches"] == stats[0]["n_kernel_launches"] - 2
    assert stats[2]["n_ao_pixels"] == stats[0]["n_ao_pixels"]
    assert stats[2]["n_kernel_launches"] == stats[0]["n_kernel_launches"]
