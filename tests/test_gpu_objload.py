"""Scenes loaded from Wavefront OBJ text (polyred_gb300.objload) render
through the CUDA path bit for bit as the oracle renders them: meshes from
the reference's TriangleMesh / QuadMesh / PolygonMesh assembly (quads fanned,
triangle+quad objects with MaterialID -1), .mtl Blinn-Phong materials with
the uniform blue texture, shadow maps kept across frames."""
import pytest

from helpers import Pair, assert_bitexact, options
from polyred_gb300 import objload, procedural

pytestmark = pytest.mark.gpu


def _load(tmp_path, n_tori, nu, nv):
    obj, mtl, n_tris = procedural.obj_tori(n_tori, nu, nv)
    (tmp_path / "tori.obj").write_bytes(obj)
    (tmp_path / "tori.mtl").write_bytes(mtl)
    g = objload.load(str(tmp_path / "tori.obj"))
    assert sum(o.mesh.n_tris for o in g.objects) == n_tris
    return g


def test_obj_tori_bitexact(device, tmp_path):
    g = _load(tmp_path, 8, 24, 12)
    s, cam = procedural.obj_tori_scene(g, 640, 360)
    p = Pair(device, options(s, cam, 640, 360, shadow_map=True))
    for _ in range(2):  # the second frame reads the first frame's shadow maps
        gpu, cpu = p.frame()
        assert (gpu["tri_id"] != 0xFFFFFFFF).sum() > 5000
        assert_bitexact(gpu, cpu)


def test_obj_tori_720p_bitexact(device, tmp_path):
    g = _load(tmp_path, 16, 48, 24)
    s, cam = procedural.obj_tori_scene(g, 1280, 720)
    p = Pair(device, options(s, cam, 1280, 720, shadow_map=True, shadow_size=(1024, 1024)))
    gpu, cpu = p.frame()
    assert_bitexact(gpu, cpu)


def _png_rgb(img):
    """A minimal PNG (colour type 2, filter type 0 on every row)."""
    import struct
    import zlib
    h, w, _ = img.shape
    raw = b"".join(b"\x00" + img[r].astype("uint8").tobytes() for r in range(h))

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


def test_obj_png_texture_bitexact(device, tmp_path):
    """An OBJ whose first material has a PNG map_Kd: decoded and
    gamma-corrected as LoadImage does, mipmapped, sampled in the shade
    kernel; bit-exact against the oracle."""
    import numpy as np
    obj, mtl, _ = procedural.obj_tori(6, 24, 12)
    mtl = mtl.replace(b"newmtl m0\n", b"newmtl m0\nmap_Kd wood.png\n")
    img = procedural.checkerboard_image(128, 64, cells=6, seed=12)[..., :3]
    (tmp_path / "tori.obj").write_bytes(obj)
    (tmp_path / "tori.mtl").write_bytes(mtl)
    (tmp_path / "wood.png").write_bytes(_png_rgb(np.ascontiguousarray(img)))
    g = objload.load(str(tmp_path / "tori.obj"))
    assert g.objects[0].materials[0].texture.rgba.shape == (64, 128, 4)
    s, cam = procedural.obj_tori_scene(g, 320, 180)
    p = Pair(device, options(s, cam, 320, 180, shadow_map=True))
    gpu, cpu = p.frame()
    assert_bitexact(gpu, cpu)
