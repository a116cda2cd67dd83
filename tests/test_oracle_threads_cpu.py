"""The oracle's row-band threads give the single-worker frame bit for bit.

Every GPU parity test and the CPU baseline run the oracle with several
threads, relying on oracle.cpp's claim that a frame split in row bands keeps
render.Workers(1)'s result (each pixel and shadow texel is owned by one
thread, which walks the triangles in draw order). These tests render the
same frames with 1 and 8 threads and compare every output, shadow maps
included, bit for bit (NaN payloads too)."""
import numpy as np

from helpers import ALL_OUTPUTS, options, shadow_cams
from polyred_gb300 import procedural, render, scene as sc
from test_gpu_parity import _basic_material, _cam, _degenerate_scene, _mesh, _ortho_cam


def _frames(opts, n_frames, cams=None, threads=1):
    import oracle
    flat = render.FlatScene(opts["scene"])
    cams = shadow_cams(opts) if cams is None else cams
    src, _ = opts["scene"].lights()
    W, H = opts["width"], opts["height"]
    sw, sh = opts["shadow_size"] or (W, H)
    state = np.zeros((max(len(src), 1), sh, sw), np.float32)
    want = ALL_OUTPUTS + (("shadow_maps",) if opts["shadow_map"] else ())
    frames = []
    for _ in range(n_frames):
        fd = render.FrameDesc(opts, cams)
        out = render.Outputs(W, H, want, n_shadow=len(src), shadow_size=(sw, sh))
        oracle.render(flat.desc(), fd.desc, out.desc, shadow_state=state, threads=threads)
        frames.append({k: v.copy() for k, v in out.arrays.items()})
    return frames


def _assert_threads_agree(opts, n_frames=1, cams=None):
    one = _frames(opts, n_frames, cams, threads=1)
    many = _frames(opts, n_frames, cams, threads=8)
    for f, (a, b) in enumerate(zip(one, many)):
        for k in a:
            ua, ub = a[k].view(np.uint8), b[k].view(np.uint8)
            assert np.array_equal(ua, ub), f"frame {f}: {k} differs between 1 and 8 threads"
    return one


def test_sphere_field_two_casting_lights_ao(native_lib, oracle_lib):
    """Point and directional casters (maps persist over two frames), AO,
    clipping by the viewport edges."""
    s, cam = procedural.sphere_field(n_spheres=32, lon=24, lat=12, width=480, height=270)
    opts = options(s, cam, 480, 270, shadow_map=True, directional_shadows=True, shadow_size=(512, 512))
    frames = _assert_threads_agree(opts, n_frames=2)
    assert (frames[-1]["tri_id"] != 0xFFFFFFFF).sum() > 1000
    assert (frames[-1]["shadow_maps"] != 0).any()


def test_camera_inside_geometry(native_lib, oracle_lib):
    s = sc.Scene(sc.Geometry(procedural.uv_sphere(16, 8, 3.0), _basic_material(ambient_occlusion=True)),
                 sc.Point(position=(0, 0, 0)), sc.Ambient(0.3))
    cam = sc.Perspective(position=(0.3, 0.2, 0.5), target=(1, 0, -2), up=(0, 1, 0), fov=70, aspect=1.5, near=0.1,
                         far=20)
    _assert_threads_agree(options(s, cam, 300, 200))


def test_nan_depth_fragments_and_shadow_maps(native_lib, oracle_lib):
    """Collapsed triangles give NaN depths in the frame, in the shadow map
    and, through AO, in neighbouring pixels."""
    m = _basic_material(ambient_occlusion=True, receive_shadow=True)
    g = sc.Geometry(_mesh(_degenerate_scene(7)), m)
    s = sc.Scene(g, sc.Point(position=(3, 4, 5), cast_shadow=True), sc.Ambient(0.1))
    frames = _assert_threads_agree(options(s, _ortho_cam(), 160, 128, shadow_map=True), n_frames=2)
    assert np.isnan(frames[-1]["depth"]).any()
    m = _basic_material(receive_shadow=True)
    g = sc.Geometry(_mesh(_degenerate_scene(9)), m)
    s = sc.Scene(g, sc.Point(position=(0, 0, 5), cast_shadow=True), sc.Ambient(0.1))
    cam = _ortho_cam()
    frames = _assert_threads_agree(options(s, cam, 160, 128, shadow_map=True), n_frames=3,
                                   cams={0: (cam.view_matrix(), cam.proj_matrix())})
    assert np.isnan(frames[-1]["shadow_maps"]).any()


def test_perspective_degenerates_and_small_sizes(native_lib, oracle_lib):
    g = sc.Geometry(_mesh(_degenerate_scene(11)), _basic_material(ambient_occlusion=True))
    s = sc.Scene(g, sc.Point(position=(3, 4, 5)), sc.Ambient(0.1))
    _assert_threads_agree(options(s, _cam(200, 150), 200, 150))
    s, _ = procedural.small_scene()
    for W, H in ((1, 1), (37, 23), (2, 200)):
        cam = sc.Perspective(position=(0, 1.5, 4), target=(0, 0, 0), fov=45, aspect=W / H, near=0.1, far=100)
        _assert_threads_agree(options(s, cam, W, H))
