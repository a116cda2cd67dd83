"""Parity of the CUDA render path with the CPU oracle, through the C ABI.

Contract: triangle-ID, depth and every G-buffer field bit-exact; RGBA8
bit-exact (the ±1 LSB allowance is not needed: transcendental calls follow
Go's float64 algorithms on both sides); shadow maps bit-exact (sign of zero
aside, which the reference's comparisons cannot observe).
"""
import numpy as np
import pytest

from helpers import Pair, assert_bitexact, options
from polyred_gb300 import procedural, scene as sc

pytestmark = pytest.mark.gpu


def assert_same_maps(a, b):
    """Shadow maps: equal values, NaN where NaN; +0 and -0 count as equal."""
    a = np.where(a == 0, np.float32(0), a)
    b = np.where(b == 0, np.float32(0), b)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    assert np.array_equal(np.nan_to_num(a, nan=-7.0).view(np.uint32), np.nan_to_num(b, nan=-7.0).view(np.uint32))


def _pair(device, s, cam, W, H, **kw):
    return Pair(device, options(s, cam, W, H, **kw))


def test_small_scene_bitexact(device):
    s, cam = procedural.small_scene()
    p = _pair(device, s, cam, 800, 500)
    gpu, cpu = p.frame()
    assert (gpu["tri_id"] != 0xFFFFFFFF).sum() > 50000
    assert_bitexact(gpu, cpu)
    assert p.stats["n_clipped_tris"] > 0  # the ground crosses the viewport edges


def test_small_scene_gamma_off_background(device):
    s, cam = procedural.small_scene()
    p = _pair(device, s, cam, 800, 500, gamma=False, background=(10, 20, 30, 255))
    gpu, cpu = p.frame()
    assert_bitexact(gpu, cpu)
    assert (gpu["rgba"][0, 0] == [10, 20, 30, 255]).all()


def test_shadow_maps_persist_across_frames(device):
    """Shadow maps start zeroed and are never cleared by a frame
    (render/shadow.go:87, :221-228): frame 2 rasterises into frame 1's maps."""
    s, cam = procedural.small_scene()
    for o, _ in s.iter_objects():
        if isinstance(o, sc.Point):
            o.cast_shadow = True
        if isinstance(o, sc.Geometry):
            for m in o.materials:
                m.receive_shadow = True
    p = _pair(device, s, cam, 320, 200, shadow_map=True)
    for _ in range(2):
        gpu, cpu = p.frame(with_shadow_maps=True)
        assert_bitexact(gpu, cpu, ["rgba", "tri_id", "depth", "nor", "world_pos", "uvd", "vcol", "mat_id"])
        assert_same_maps(gpu["shadow_maps"], cpu["shadow_maps"])


def test_sphere_field_reduced_bitexact(device):
    """32 spheres, point + directional shadow casters, AO, flat shading."""
    s, cam = procedural.sphere_field(n_spheres=32, lon=24, lat=12, width=480, height=270)
    p = _pair(device, s, cam, 480, 270, shadow_map=True, directional_shadows=True, shadow_size=(512, 512))
    for _ in range(2):
        gpu, cpu = p.frame()
        assert_bitexact(gpu, cpu)


def test_sphere_field_full_size_bitexact(device):
    """The 1M-triangle, 1920x1080 workload, shadows (2048^2) and AO on."""
    s, cam = procedural.sphere_field()
    p = _pair(device, s, cam, 1920, 1080, shadow_map=True, directional_shadows=True, shadow_size=(2048, 2048))
    gpu, cpu = p.frame()
    assert_bitexact(gpu, cpu, ["rgba", "tri_id", "depth"])
    assert p.stats["n_tris_in"] == 999936


def _mesh(tris, mat=0, col=(200, 100, 50, 255)):
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    n = tris.shape[0]
    pos = np.ones((n, 3, 4), np.float32)
    pos[..., :3] = tris
    nrm = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=-1, keepdims=True), 1e-30)
    nor = np.zeros((n, 3, 4), np.float32)
    nor[..., :3] = nrm[:, None]
    colr = np.empty((n, 3, 4), np.uint8)
    colr[:] = col
    return sc.Mesh(pos, nor, None, colr, np.full(n, mat, np.int32))


def _basic_material(**kw):
    return sc.BlinnPhong(diffuse=(200, 120, 80, 255), specular=(128, 128, 128, 255), shininess=16, **kw)


def _cam(W, H, pos=(0, 0, 5)):
    return sc.Perspective(position=pos, target=(0, 0, 0), up=(0, 1, 0), fov=50, aspect=W / H, near=0.1, far=50)


def test_depth_ties_first_drawn_wins(device):
    """Coplanar duplicates: equal depth never replaces (buffer/buffer.go:230),
    so the earlier triangle keeps every shared pixel."""
    t = [[-1, -1, 0], [1, -1, 0], [0, 1, 0]]
    g1 = sc.Geometry(_mesh([t], col=(255, 0, 0, 255), mat=-1))
    g2 = sc.Geometry(_mesh([t, t], col=(0, 255, 0, 255), mat=-1))
    s = sc.Scene(g1, g2, sc.Ambient(0.2))
    gpu, cpu = _pair(device, s, _cam(160, 120), 160, 120).frame()
    assert_bitexact(gpu, cpu)
    ids = gpu["tri_id"][gpu["tri_id"] != 0xFFFFFFFF]
    assert ids.size > 100 and (ids == 0).all()


def _degenerate_scene(seed, rows=128):
    """Regular triangles mixed with collapsed ones. A collapsed triangle has
    two vertices sharing (x, y) and its third on the same row y, which under
    the orthographic camera below maps exactly onto a pixel-centre row: there
    all three Barycoord cross products are 0 and 0/0 gives NaN coordinates,
    which pass the inside test with a NaN depth."""
    rng = np.random.default_rng(seed)
    tris = []
    for i in range(600):
        if i % 2 == 0:
            c = rng.uniform(-2, 2, 3)
            tris.append([c, c + rng.normal(0, 0.3, 3), c + rng.normal(0, 0.3, 3)])
        else:
            k = int(rng.integers(4, rows - 4))
            y = (2 * k - (rows - 1)) / 64.0  # screen y = 32*y + 64 = k + 0.5
            x1, x3 = rng.uniform(-2, 2, 2)
            z1, z2, z3 = rng.uniform(-1, 1, 3)
            tris.append([[x1, y, z1], [x1, y, z2], [x3, y, z3]])
    return np.array(tris)


def _ortho_cam():
    # 2/(top-bottom) = 0.5 and a 128-row viewport: y_screen = 32*y + 64 exactly
    return sc.Orthographic(position=(0, 0, 5), target=(0, 0, 0), up=(0, 1, 0), left=-2.5, right=2.5, bottom=-2,
                           top=2, near=1, far=-20)


def test_degenerate_triangles_nan_depth(device):
    """The reference keeps a NaN-depth fragment when it is the first at its
    pixel (DepthTest passes on !Ok, later `z > NaN` never does), shadow maps
    take NaN and recover on the next finite store, and AO spreads NaN to the
    neighbours that march across such a pixel."""
    m = _basic_material(ambient_occlusion=True, receive_shadow=True)
    g = sc.Geometry(_mesh(_degenerate_scene(7)), m)
    s = sc.Scene(g, sc.Point(position=(3, 4, 5), cast_shadow=True), sc.Ambient(0.1))
    p = _pair(device, s, _ortho_cam(), 160, 128, shadow_map=True)
    nan_frags = 0
    for _ in range(2):
        gpu, cpu = p.frame(with_shadow_maps=True)
        assert_bitexact(gpu, cpu, ["rgba", "tri_id", "depth", "nor", "uvd", "vcol", "mat_id", "world_pos"])
        assert_same_maps(gpu["shadow_maps"], cpu["shadow_maps"])
        nan_frags += p.stats["n_nan_fragments"]
    assert nan_frags > 0
    assert np.isnan(gpu["depth"]).any()


def test_degenerate_triangles_nan_shadow_map(device):
    """NaN depths in the shadow pass: the light camera is given the main
    camera's exact orthographic matrices, so the collapsed triangles land on
    pixel-centre rows of the shadow map too."""
    m = _basic_material(receive_shadow=True)
    g = sc.Geometry(_mesh(_degenerate_scene(9)), m)
    s = sc.Scene(g, sc.Point(position=(0, 0, 5), cast_shadow=True), sc.Ambient(0.1))
    cam = _ortho_cam()
    p = Pair(device, options(s, cam, 160, 128, shadow_map=True), cams={0: (cam.view_matrix(), cam.proj_matrix())})
    for _ in range(3):
        gpu, cpu = p.frame(with_shadow_maps=True)
        assert_bitexact(gpu, cpu, ["rgba", "tri_id", "depth", "nor", "uvd", "vcol", "mat_id", "world_pos"])
        assert_same_maps(gpu["shadow_maps"], cpu["shadow_maps"])
    assert np.isnan(cpu["shadow_maps"]).any()


def test_degenerate_triangles_perspective(device):
    m = _basic_material(ambient_occlusion=True)
    g = sc.Geometry(_mesh(_degenerate_scene(11)), m)
    s = sc.Scene(g, sc.Point(position=(3, 4, 5)), sc.Ambient(0.1))
    gpu, cpu = _pair(device, s, _cam(200, 150), 200, 150).frame()
    assert_bitexact(gpu, cpu)


def test_orthographic_camera(device):
    s, _ = procedural.small_scene()
    cam = sc.Orthographic(position=(0, 1.5, 4), target=(0, 0, 0), up=(0, 1, 0), left=-2, right=2, bottom=-1.25,
                          top=1.25, near=1, far=-10)
    gpu, cpu = _pair(device, s, cam, 320, 200).frame()
    assert_bitexact(gpu, cpu)


def test_camera_inside_geometry_clipping(device):
    """Large triangles around and behind the camera: heavy screen-space
    clipping (render/clipping.go) and full-screen raster tasks."""
    s = sc.Scene(sc.Geometry(procedural.uv_sphere(16, 8, 3.0), _basic_material()), sc.Point(position=(0, 0, 0)),
                 sc.Ambient(0.3))
    cam = sc.Perspective(position=(0.3, 0.2, 0.5), target=(1, 0, -2), up=(0, 1, 0), fov=70, aspect=1.5, near=0.1,
                         far=20)
    p = _pair(device, s, cam, 300, 200)
    gpu, cpu = p.frame()
    assert_bitexact(gpu, cpu)


def test_material_edge_cases(device):
    """Vertex-colour fragments (MaterialID -1), out-of-range material ids,
    flat shading, several ambient lights, a directional light."""
    t = np.array([[[-2, -1, 0], [0, -1, 0], [-1, 1, 0]], [[0, -1, 0], [2, -1, 0], [1, 1, 0]],
                  [[-1, -1.5, -1], [1, -1.5, -1], [0, 0.5, -1]], [[-2, 0, 0.5], [-1, 0, 0.5], [-1.5, 1, 0.5]]])
    mesh = _mesh(t)
    mesh.mat_id[:] = [-1, 0, 1, 7]
    g = sc.Geometry(mesh, _basic_material(), _basic_material(flat_shading=True))
    s = sc.Scene(g, sc.Directional(direction=(0.3, -1, -0.4), intensity=0.8), sc.Ambient(0.1), sc.Ambient(0.05))
    gpu, cpu = _pair(device, s, _cam(160, 100), 160, 100).frame()
    assert_bitexact(gpu, cpu)


def test_no_lights_uses_texture_colour(device):
    s = sc.Scene(sc.Geometry(procedural.uv_sphere(12, 6), _basic_material()))
    gpu, cpu = _pair(device, s, _cam(64, 48), 64, 48).frame()
    assert_bitexact(gpu, cpu)


@pytest.mark.parametrize("W,H", [(1, 1), (37, 23), (2, 200)])
def test_odd_sizes(device, W, H):
    s, _ = procedural.small_scene()
    cam = sc.Perspective(position=(0, 1.5, 4), target=(0, 0, 0), fov=45, aspect=W / H, near=0.1, far=100)
    gpu, cpu = _pair(device, s, cam, W, H).frame()
    assert_bitexact(gpu, cpu)


def test_empty_and_all_culled(device):
    # every triangle faces away or is off screen
    t = np.array([[[-1, -1, 0], [0, 1, 0], [1, -1, 0]], [[50, 50, 0], [51, 50, 0], [50, 51, 0]]])
    s = sc.Scene(sc.Geometry(_mesh(t), _basic_material()), sc.Ambient(0.5))
    gpu, cpu = _pair(device, s, _cam(64, 48), 64, 48, background=(1, 2, 3, 4)).frame()
    assert_bitexact(gpu, cpu)
    assert (gpu["tri_id"] == 0xFFFFFFFF).all()


def test_triangle_soup_small(device):
    """Small-triangle stress at reduced size (log-normal areas, 30% back-facing)."""
    W, H = 640, 360
    mesh = procedural.triangle_soup(200_000, W, H)
    s = sc.Scene(sc.Geometry(mesh, _basic_material()), sc.Point(position=(0, 5, 5)), sc.Ambient(0.1))
    cam = sc.Perspective(position=(0, 0, 0), target=(0, 0, -1), up=(0, 1, 0), fov=60, aspect=W / H, near=0.1,
                         far=120)
    gpu, cpu = _pair(device, s, cam, W, H).frame()
    assert_bitexact(gpu, cpu)


def test_repeated_frames_are_deterministic(device):
    s, cam = procedural.sphere_field(n_spheres=16, lon=16, lat=8, width=256, height=144)
    p = _pair(device, s, cam, 256, 144)
    g1, c1 = p.frame()
    g2, _ = p.frame()
    assert_bitexact(g1, g2)
    assert_bitexact(g1, c1)


def test_triangle_soup_full_size(device):
    """The small-triangle stress workload at full size: 10M soup triangles
    (log-normal areas around 1 px, 30% back-facing) at 3840x2160, bit-exact
    with the oracle (threaded, identical to its single-thread order)."""
    W, H = 3840, 2160
    s, cam = procedural.soup_scene(10_000_000, W, H)
    p = Pair(device, options(s, cam, W, H, gamma=True), outputs=("rgba", "tri_id", "depth", "nor", "mat_id"))
    gpu, cpu = p.frame()
    assert (cpu["tri_id"] != 0xFFFFFFFF).sum() > 0.5 * W * H
    assert p.stats["n_raster_tris"] > 5_000_000
    assert_bitexact(gpu, cpu)


def test_pinned_outputs_match_pageable(device):
    """Outputs in page-locked memory (pr_host_alloc) receive the same frame."""
    import ctypes as C
    from polyred_gb300 import native, render
    lib = native.load()
    s, cam = procedural.small_scene(320, 200)
    o = options(s, cam, 320, 200)
    flat = render.FlatScene(s)
    d = flat.desc()
    native.check(lib.pr_scene_upload(device.handle, C.byref(d)))
    fd = render.FrameDesc(o, {})
    names = ("rgba", "tri_id", "depth", "nor", "world_pos")
    a = render.Outputs(320, 200, names)
    b = render.Outputs(320, 200, names, pinned=True)
    for out in (a, b):
        native.check(lib.pr_render(device.handle, C.byref(fd.desc), C.byref(out.desc)))
    for n in names:
        assert np.array_equal(a.arrays[n].view(np.uint8), b.arrays[n].view(np.uint8)), n
    assert (b.arrays["tri_id"] != 0xFFFFFFFF).sum() > 1000
