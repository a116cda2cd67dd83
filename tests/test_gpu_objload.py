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
