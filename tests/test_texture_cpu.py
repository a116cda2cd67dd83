"""Image textures on the host: the library's mipmap levels (NewTexture, each
level imageutil.Resize of the image) and its Texture.Query / level of detail
(the source the shade kernel compiles, built for the host here) against the
oracle's restatement of buffer/texture.go, on seeded images and queries.
No GPU."""
import numpy as np
import pytest

import oracle
from polyred_gb300 import native

F32 = np.float32
SIZES = [(1, 1), (2, 2), (3, 5), (8, 2), (2, 8), (16, 16), (33, 17), (64, 32), (128, 1), (256, 256)]


def _ptr(a):
    return None if a is None else a.ctypes.data


def _build(lib_fn, img, mip):
    h, w = img.shape[:2]
    desc = np.zeros(1 + 3 * 16, np.int32)
    n = lib_fn(w, h, img.ctypes.data, int(mip), None, 0, desc.ctypes.data)
    assert n >= 0
    out = np.zeros((max(n, 1), 4), np.uint8)
    assert lib_fn(w, h, img.ctypes.data, int(mip), out.ctypes.data, n, desc.ctypes.data) == n
    return out[:n], desc


def _query(lib_fn, img, mip, u, v, lod=None, du=None, dv=None):
    h, w = img.shape[:2]
    out = np.zeros((len(u), 4), np.uint8)
    rc = lib_fn(w, h, img.ctypes.data, int(mip), len(u), _ptr(lod), _ptr(du), _ptr(dv), _ptr(u), _ptr(v),
                out.ctypes.data)
    assert rc == 0
    return out


def _image(rng, w, h):
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    if w * h > 4:
        img[: h // 2, : w // 2] = [255, 0, 0, 255]  # flat patches and hard edges
        img[h // 2:, w // 2:, 3] = 0
    return np.ascontiguousarray(img)


@pytest.mark.parametrize("w,h", SIZES)
@pytest.mark.parametrize("mip", [True, False])
def test_mipmap_levels_match_oracle(native_lib, w, h, mip):
    img = _image(np.random.default_rng(w * 1000 + h), w, h)
    got, gd = _build(native_lib.pr_debug_texture_build, img, mip)
    want, wd = _build(oracle.load().orc_texture_build, img, mip)
    n = int(wd[0])
    assert int(gd[0]) == n
    assert np.array_equal(gd[: 1 + 3 * n], wd[: 1 + 3 * n])
    assert np.array_equal(got, want)
    assert np.array_equal(got[: w * h].reshape(h, w, 4), img)  # level 0 is the image


def _uv(rng, n):
    u = rng.uniform(-2.5, 3.5, n).astype(F32)
    special = np.array([0, -0.0, 1, -1, 2, 0.5, -0.5, 1e-8, -1e-8, 0.999999, 1.0000001, 3, -2], F32)
    u[: len(special)] = special
    u[len(special): 2 * len(special)] = np.round(u[len(special): 2 * len(special)])  # integers
    return u


@pytest.mark.parametrize("w,h", SIZES)
@pytest.mark.parametrize("mip", [True, False])
def test_query_matches_oracle(native_lib, w, h, mip):
    rng = np.random.default_rng(7 + w * 31 + h)
    img = _image(rng, w, h)
    n = 4000
    u, v = _uv(rng, n), rng.permutation(_uv(rng, n)).astype(F32)
    lod = rng.uniform(-1.0, 10.0, n).astype(F32)
    lod[:40] = np.arange(-2, 8, 0.25, dtype=F32)[:40]  # level boundaries, ApproxEq(p, 0)
    lod[40:43] = [np.nan, np.inf, -np.inf]
    got = _query(native_lib.pr_debug_texture_query, img, mip, u, v, lod=lod)
    want = _query(oracle.load().orc_texture_query, img, mip, u, v, lod=lod)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("w,h", [(64, 64), (256, 128), (37, 300), (1, 1)])
def test_shader_lod_matches_oracle(native_lib, w, h):
    rng = np.random.default_rng(11 + w + h)
    img = _image(rng, w, h)
    n = 4000
    u, v = _uv(rng, n), _uv(rng, n)
    du = (10.0 ** rng.uniform(-9, 1, n)).astype(F32)
    dv = (10.0 ** rng.uniform(-9, 1, n)).astype(F32)
    du[:6] = [0, -0.0, np.nan, np.inf, 1.0 / (w * w), 4.0 / (w * w)]
    dv[:6] = [0, 0, 0, 0, 1.0 / (w * w), 0]
    got = _query(native_lib.pr_debug_texture_query, img, True, u, v, du=du, dv=dv)
    want = _query(oracle.load().orc_texture_query, img, True, u, v, du=du, dv=dv)
    assert np.array_equal(got, want)


# ---------------------------------------------------------------- reference known answers

def _kats():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "reference_kats.json")) as fh:
        return json.load(fh)["texture_query"]


KATS = _kats()


def _kat_texture(case):
    """The texture of one TestQuery case: NewTexture() (1x1 white, mipmap
    on), the test's 2x2 image, or a reference asset loaded without gamma
    correction (MustLoadImage(path)); None when the asset is absent."""
    import os
    import sys
    t = case["texture"]
    if t.get("default"):
        return np.full((1, 1, 4), 255, np.uint8), True
    if t.get("image") == "data":
        x0, y0, x1, y1 = KATS["data_rect"]
        return np.array(KATS["data_pix"], np.uint8).reshape(y1 - y0, x1 - x0, 4), t["mipmap"]
    if not t["asset"].endswith(".png"):
        pytest.skip(f"{t['asset']}: only PNG images are decoded")
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from helpers import reference_testdata
    path = os.path.join(reference_testdata(), t["asset"])
    if not os.path.exists(path):
        pytest.skip("reference test assets not present")
    from polyred_gb300 import imageload
    return imageload.load_image(path, gamma_correct=t["gamma_correct"]), t["mipmap"]


@pytest.mark.parametrize("k", range(len(KATS["cases"])))
def test_reference_texture_query_kats(native_lib, k):
    """TestQuery's vectors (buffer/texture_test.go): Query(lod, u, v) of the
    library (its mipmap levels and the kernel's query source) and of the
    oracle equal the reference's answers."""
    case = KATS["cases"][k]
    img, mip = _kat_texture(case)
    img = np.ascontiguousarray(img)
    u, v, lod = (np.array([case[x]], F32) for x in ("u", "v", "lod"))
    want = np.array([case["want"]], np.uint8)
    assert np.array_equal(_query(native_lib.pr_debug_texture_query, img, mip, u, v, lod=lod), want)
    assert np.array_equal(_query(oracle.load().orc_texture_query, img, mip, u, v, lod=lod), want)
