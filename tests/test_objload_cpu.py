"""OBJ / MTL loading (polyred_gb300.objload over the native pr_obj_* parser)
against the oracle's restatement of model/obj/obj.go and model/load.go:
seeded random files, the number grammar, float32 rounding at midpoints,
every error and panic path, the .mtl fallback rules, and the reference's own
assets when they are present. No GPU."""
import os
import random
import sys
from fractions import Fraction

import numpy as np
import pytest

from helpers import same_bits
from oracle import objparse as op
from polyred_gb300 import _abi, objload

HERE = os.path.dirname(os.path.abspath(__file__))
F32 = np.float32


@pytest.fixture(autouse=True)
def _lib(native_lib):
    return native_lib


def write(tmp_path, obj, mtl=None, name="m.obj", mtlname="m.mtl"):
    p = tmp_path / name
    p.write_bytes(obj.encode() if isinstance(obj, str) else obj)
    if mtl is not None:
        (tmp_path / mtlname).write_bytes(mtl.encode() if isinstance(mtl, str) else mtl)
    return str(p)


# ---------------------------------------------------------------- comparisons

def _f32(xs, k):
    return np.array(xs, F32).reshape(-1, k)


def compare_file(path):
    """parse_file against oracle load_file: same values, or the same error."""
    try:
        of = op.load_file(path)
    except op.GoError as e:
        with pytest.raises(objload.ObjError) as ei:
            objload.parse_file(path)
        assert str(ei.value) == str(e)
        return None
    except op.GoPanic:
        with pytest.raises(objload.ObjPanic):
            objload.parse_file(path)
        return None
    except OSError:
        with pytest.raises(OSError):
            objload.parse_file(path)
        return None
    pf = objload.parse_file(path)
    assert same_bits(pf.vertices, _f32(of.Vertices, 3)).all()
    assert same_bits(pf.normals, _f32(of.Normals, 3)).all()
    assert same_bits(pf.uvs, _f32(of.Uvs, 2)).all()
    faces = [fc for ob in of.Objs for fc in ob.Faces]
    owner = [k for k, ob in enumerate(of.Objs) for _ in ob.Faces]
    assert pf.n_faces == len(faces)
    assert pf.face_start.tolist() == np.cumsum([0] + [len(fc.Vertices) for fc in faces]).tolist()
    assert pf.corner_v.tolist() == [v for fc in faces for v in fc.Vertices]
    assert pf.corner_vt.tolist() == [v for fc in faces for v in fc.Uvs]
    assert pf.corner_vn.tolist() == [v for fc in faces for v in fc.Normals]
    assert pf.face_object.tolist() == owner
    assert pf.face_smooth.tolist() == [fc.Smooth for fc in faces]
    assert list(pf.face_material_names()) == [fc.Material for fc in faces]
    assert pf.objects == [(ob.Name, ob.Materials) for ob in of.Objs]
    assert set(pf.materials) == set(of.Materials)
    for name, m in of.Materials.items():
        got = pf.materials[name]
        if m is None:
            assert got is None
            continue
        for k in ("Illum", "Ambient", "Diffuse", "Specular", "Emissive", "MapKd"):
            assert got[k] == getattr(m, k), (name, k)
        for k in ("Opacity", "Refraction", "Shininess"):
            assert same_bits(got[k], getattr(m, k)).all(), (name, k)
    assert pf.warnings == of.Warnings
    assert pf.matlib == of.Matlib
    assert pf.mtl_dir == of.MtlDir
    return pf


def compare_model(path):
    """load against oracle load_model: same meshes and materials, or the
    same error."""
    try:
        og = op.load_model(path, image_textures="ignore")
    except op.GoError as e:
        with pytest.raises(objload.ObjError) as ei:
            objload.load(path, image_textures="ignore")
        assert str(ei.value) == str(e)
        return None
    except op.GoPanic:
        with pytest.raises(objload.ObjPanic):
            objload.load(path, image_textures="ignore", skip_faceless=True)
        return None
    except OSError:  # a missing mtllib file: the reference panics
        with pytest.raises(OSError):
            objload.load(path, image_textures="ignore", skip_faceless=True)
        return None
    if any(g is None for g in og):
        with pytest.raises(objload.ObjError, match="no triangle or quad faces"):
            objload.load(path, image_textures="ignore")
    group = objload.load(path, image_textures="ignore", skip_faceless=True)
    want = [g for g in og if g is not None]
    assert len(group.objects) == len(want)
    for geo, w in zip(group.objects, want):
        m = geo.mesh
        tris = w["tris"]
        assert m.n_tris == len(tris)
        pos = np.array([[v["pos"] for v in t[:3]] for t in tris], F32).reshape(-1, 3, 4)
        nor = np.array([[v["nor"] for v in t[:3]] for t in tris], F32).reshape(-1, 3, 4)
        uv = np.array([[v["uv"] for v in t[:3]] for t in tris], F32).reshape(-1, 3, 2)
        assert same_bits(m.pos, pos).all()
        assert same_bits(m.nor, nor).all()
        assert same_bits(m.uv, uv).all()
        assert (m.col == 255).all()
        assert m.mat_id.tolist() == [t[3] for t in tris]
        assert len(geo.materials) == len(w["materials"])
        for a, b in zip(geo.materials, w["materials"]):
            assert a.diffuse == tuple(b["diffuse"]) and a.specular == tuple(b["specular"])
            assert same_bits(a.shininess, b["shininess"]).all()
            assert a.texture == b["texture"]
            assert not (a.flat_shading or a.ambient_occlusion or a.receive_shadow) and a.mipmap
    return group


# ---------------------------------------------------------------- random files

def _num(rng, v):
    k = rng.randrange(11)
    if k == 0:
        return "%d" % int(v)
    if k == 1:
        return "%.6f" % v
    if k == 2:
        return "%e" % v
    if k == 3:
        return repr(float(F32(v)))
    if k == 4:
        return ("+" if v >= 0 else "") + "%.9g" % v
    if k == 5:
        s = "%.4f" % v
        return s.replace("0.", ".", 1) if s.startswith("0.") else s
    if k == 6:
        return "%.25f" % v
    if k == 7:
        return "%.3E" % v
    if k == 8:
        return "%d." % int(v)
    if k == 9:
        return float(F32(v)).hex()
    return "%.7g" % v


def random_obj(rng, consistent=True):
    """A seeded .obj / .mtl pair exercising the grammar the loader reads."""
    lines = []
    nv = nvt = nvn = 0
    use_vt = rng.random() < 0.6
    use_vn = rng.random() < 0.7
    sep = lambda: rng.choice([" ", " ", "  ", "\t", " \t "])

    def num(v):
        return _num(rng, v)

    def add_v():
        nonlocal nv
        xyz = [num(rng.uniform(-2, 2)) for _ in range(3)]
        if rng.random() < 0.15:
            xyz.append(num(rng.uniform(0.5, 2.0)))
        lines.append("v" + sep() + sep().join(xyz))
        nv += 1

    def add_vt():
        nonlocal nvt
        uv = [num(rng.uniform(0, 1)) for _ in range(2 if rng.random() < 0.8 else 3)]
        lines.append("vt " + " ".join(uv))
        nvt += 1

    def add_vn():
        nonlocal nvn
        if rng.random() < 0.12:
            lines.append("vn 0 0 0")
        else:
            lines.append("vn " + " ".join(num(rng.uniform(-1, 1)) for _ in range(3)))
        nvn += 1

    if rng.random() < 0.8:
        lines.append("mtllib m.mtl")
    if rng.random() < 0.3:
        lines.append("# a comment")
    for _ in range(rng.randrange(3, 12)):
        add_v()
    if use_vt:
        for _ in range(rng.randrange(1, 6)):
            add_vt()
    if use_vn:
        for _ in range(rng.randrange(1, 6)):
            add_vn()
    for _ in range(rng.randrange(5, 70)):
        r = rng.random()
        if r < 0.06:
            lines.append(rng.choice(["o", "g"]) + " obj%d" % rng.randrange(5))
        elif r < 0.13:
            lines.append("usemtl m%d" % rng.randrange(5))
        elif r < 0.16:
            lines.append("s " + rng.choice(["0", "1", "off", "on", "2"]))
        elif r < 0.21:
            lines.append(rng.choice(["", "   ", "# comment", "l 1 2", "vp 0.5", "#usemtl x", "cstype bezier"]))
        elif r < 0.33:
            rng.choice([add_v, add_v, add_vt if use_vt else add_v, add_vn if use_vn else add_v])()
        else:
            n = rng.choice([3, 3, 3, 4, 4, 5, 6])
            corners = []
            for _ in range(n):
                vi = rng.randrange(1, nv + 1)
                vs = str(vi) if rng.random() < 0.8 else str(vi - nv - 1)
                ts = ns = None
                if use_vt and (consistent or rng.random() < 0.7):
                    ti = rng.randrange(1, nvt + 1)
                    ts = str(ti) if rng.random() < 0.8 else str(ti - nvt - 1)
                if use_vn and (consistent or rng.random() < 0.7):
                    ni = rng.randrange(1, nvn + 1)
                    ns = str(ni) if rng.random() < 0.8 else str(ni - nvn - 1)
                c = vs
                if ts is not None and ns is not None:
                    c = f"{vs}/{ts}/{ns}"
                elif ts is not None:
                    c = f"{vs}/{ts}"
                elif ns is not None:
                    c = f"{vs}//{ns}"
                corners.append(c)
            lines.append("f" + sep() + sep().join(corners))
    eol = "\r\n" if rng.random() < 0.2 else "\n"
    obj = eol.join(lines) + (eol if rng.random() < 0.7 else "")

    mtl = []
    for k in range(rng.randrange(0, 4)):
        mtl.append("newmtl m%d" % k)
        for key in ("Ka", "Kd", "Ks", "Ke"):
            if rng.random() < 0.8:
                mtl.append(key + " " + " ".join(num(rng.uniform(0, 1)) for _ in range(3)))
        if rng.random() < 0.8:
            mtl.append("Ns " + num(rng.uniform(0, 300)))
        if rng.random() < 0.5:
            mtl.append("d " + num(rng.uniform(0, 1)))
        if rng.random() < 0.5:
            mtl.append("Ni " + num(rng.uniform(1, 2)))
        mtl.append("illum " + rng.choice(["0", "2", "2"]))
        if rng.random() < 0.2:
            mtl.append(rng.choice(["Tr 0.5", "map_Bump x.png", "# note", ""]))
    return obj, "\n".join(mtl) + "\n"


@pytest.mark.parametrize("seed", range(60))
def test_random_files_match_oracle(tmp_path, seed):
    rng = random.Random(0x0B1E0000 + seed)
    obj, mtl = random_obj(rng, consistent=seed % 4 != 3)
    path = write(tmp_path, obj, mtl)
    compare_file(path)
    compare_model(path)


def test_reference_assets_match_fixture():
    """The reference's own test assets, when present: the native parser gives
    the arrays the oracle recorded (tests/golden/obj_assets.json)."""
    import json
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_obj_fixtures as mk
    from helpers import reference_testdata
    d = reference_testdata()
    if not os.path.isdir(d):
        pytest.skip("reference OBJ assets not present")
    with open(os.path.join(HERE, "golden", "obj_assets.json")) as fh:
        fx = json.load(fh)
    for name, rec in fx.items():
        f = objload.parse_file(os.path.join(d, name))
        for key, arr in (("vertices", f.vertices), ("normals", f.normals), ("uvs", f.uvs),
                         ("face_start", f.face_start), ("corner_v", f.corner_v), ("corner_vt", f.corner_vt),
                         ("corner_vn", f.corner_vn)):
            assert mk.digest(arr.reshape(-1)) == rec[key], (name, key)
        assert [o[0] for o in f.objects] == rec["objects"]
        assert f.warnings == rec["warnings"]
        g = objload.load(os.path.join(d, name), image_textures="ignore")
        assert sum(o.mesh.n_tris for o in g.objects) > 0


# ---------------------------------------------------------------- numbers

VALID_NUMBERS = [
    "0", "-0", "+0", "1", "-1", "+1.5", ".5", "5.", "-.25", "1e3", "1E3", "1e+3", "1e-3", "-1.5e-7", "3.4028234e38",
    "3.4028235e38", "3.40282356e38", "1e-45", "1.4e-45", "7e-46", "1e-46", "1e-400", "0e99999", "1e-99999",
    "1.17549435e-38", "1.1754942e-38", "123456789", "16777217", "16777219", "0.1", "0.2", "0.3",
    "0.30000001192092896", "9999999999999999999999999", "1_000", "1_0.5_0e1_0", "0x1p0", "0x1.8p1", "-0x.1p4",
    "0X1P-149", "0x1p-150", "0x1.000001p0", "0x1_0p0", "0x_1p0", "inf", "-inf", "+Inf", "INFINITY", "-Infinity",
    "nan", "NaN", "NAN", "00001.5000", "1e0000000000000000000010",
    # both sides of the exact fast path: <= 8 digits and M <= 2^24, |k| <= 10
    "16777216", "16777216e10", "1677721.6", "16777217e-10", "12345678e-10", "12345678e-11", "1.2345678e10",
    "9.9999999e-11", "0.00000000012345678", "99999999", "1e10", "1e11", "1e-10", "1e-11", "0.0000001e-3",
    "4.2949673e9", "-0.000000", "+00000000000000.00000000001",
]

INVALID_NUMBERS = [
    "", "+", "-", ".", "e5", "1e", "1e+", "1e+-5", "1.2.3", "--1", "+-1", "1_", "_1", "1__0", "1_.5", "1._5",
    "0x", "0x1", "0x1.5", "0xp1", "0x1p", "abc", "1a", "infinit", "infx", "in", "+nan", "-nan", "nan1", "1,5",
    "1e999", "-1e39", "3.40282357e38", "0x1p128", "0x1.ffffffp127", "１", "1\x00",
]


def _single_vertex(tmp_path, s):
    return write(tmp_path, b"v " + s.encode("utf-8") + b" 0 0\n")


def test_number_grammar_valid(tmp_path):
    text = "".join(f"v {s} 0 0\n" for s in VALID_NUMBERS)
    path = write(tmp_path, text)
    f = objload.parse_file(path)
    for s, got in zip(VALID_NUMBERS, f.vertices[:, 0]):
        assert same_bits(got, op.parse_float32(s.encode())).all(), s
    compare_file(path)


@pytest.mark.parametrize("s", INVALID_NUMBERS)
def test_number_grammar_invalid(tmp_path, s):
    with pytest.raises(op.GoError):
        op.parse_float32(s.encode("utf-8"))
    compare_file(_single_vertex(tmp_path, s))


def _exact_decimal(fr):
    """The finite decimal expansion of a dyadic rational."""
    sign = "-" if fr < 0 else ""
    fr = abs(fr)
    k = 0
    while fr.denominator != 1 << k:
        k += 1
    digits = str(fr.numerator * 5 ** k)
    if k == 0:
        return sign + digits
    digits = digits.rjust(k + 1, "0")
    return sign + digits[:-k] + "." + digits[-k:]


def test_float32_rounding_at_midpoints(tmp_path):
    """Decimal strings on and beside the midpoint of two float32 neighbours,
    normal and subnormal: correctly rounded, ties to even."""
    rng = np.random.default_rng(7)
    bits = np.concatenate([rng.integers(0x00000001, 0x00800000, 200), rng.integers(0x00800000, 0x7F7FFFFF, 800)])
    strs = []
    for b in bits.astype(np.uint32):
        x = Fraction(float(b.view(F32)))
        y = Fraction(float((b + np.uint32(1)).view(F32)))
        mid = (x + y) / 2
        s = _exact_decimal(mid)
        strs.append(s)
        if "." in s:
            strs.append(s + "1")                     # just above
            strs.append(s[:-1] + str(int(s[-1]) - 1) if s[-1] != "0" else s)  # just below
        strs.append("%.9e" % float(mid))
    text = "".join(f"v {s} 0 0\n" for s in strs)
    f = objload.parse_file(write(tmp_path, text))
    want = np.array([op.parse_float32(s.encode()) for s in strs], F32)
    assert same_bits(f.vertices[:, 0], want).all()


# ---------------------------------------------------------------- errors

OBJ_ERRORS = [
    "v 1 2\n", "v 1 2 abc\n", "v 1 2 3 x\n", "v 1e39 0 0\n", "vn 1 2\n", "vn 1 2 z\n", "vt 1\n", "vt a b\n",
    "f 1 2\n", "v 0 0 0\nf 0 1 1\n", "v 0 0 0\nvt 0 0\nf 1/0 1/1 1/1\n", "v 0 0 0\nvn 0 0 1\nf 1//0 1//1 1//1\n",
    "v 0 0 0\nf 1// 1// 1//\n", "v 0 0 0\nf /1 1 1\n", "v 0 0 0\nf 1.5 1 1\n", "v 0 0 0\nf 2147483648 1 1\n",
    "v 0 0 0\nf -2147483649 1 1\n", "o\n", "g\n", "usemtl\n", "s\n", "mtllib\n", "# fine\n\nv 1 2 3\nf 1 1\n",
]


@pytest.mark.parametrize("k", range(len(OBJ_ERRORS)))
def test_obj_errors(tmp_path, k):
    path = write(tmp_path, OBJ_ERRORS[k])
    with pytest.raises(op.GoError):
        op.load_file(path)
    compare_file(path)
    compare_model(path)


PANICS = [
    # (obj, mtl): inputs on which the reference panics
    ("mtllib m.mtl\nv 0 0 0\nf 1 1 1\n", "newmtl a\nKd 1.5 0 0\n"),            # color.FromValue out of range
    ("mtllib m.mtl\nv 0 0 0\nf 1 1 1\n", "Kd 0.5 0 0\n"),                      # property before newmtl
    ("mtllib m.mtl\nv 0 0 0\nf 1 1 1\n", "map_Kd x.png\n"),
    ("mtllib m.mtl\nusemtl a\nv 0 0 0\nf 1 1 1\n", "newmtl a\nillum 3\n"),     # unsupported illumination model
    ("v 0 0 0\nv 1 0 0\nf 1 2 3\n", None),                                       # index out of range
    ("v 0 0 0\nv 1 0 0\nv 1 1 0\nf -4 1 2\n", None),                             # relative index before the first
    ("v 0 0 0\nv 1 0 0\nv 1 1 0\nvn 0 0 1\nf 1 2 3\n", None),                    # face without vn, file with normals
    ("v 0 0 0\nv 1 0 0\nv 1 1 0\nvt 0 0\nf 1//1 2//1 3//1 1//1 2//1\n", None),  # polygon without vt
]


@pytest.mark.parametrize("k", range(len(PANICS)))
def test_reference_panics(tmp_path, k):
    obj, mtl = PANICS[k]
    path = write(tmp_path, obj, mtl)
    with pytest.raises(op.GoPanic):
        op.load_model(path, image_textures="ignore")
    compare_model(path)


def test_missing_mtllib_file(tmp_path):
    path = write(tmp_path, "mtllib nowhere.mtl\nv 0 0 0\n")
    with pytest.raises(FileNotFoundError):
        objload.parse_file(path)
    compare_file(path)


MTL_FALLBACK = [
    # a malformed .mtl: every material falls back to material.Default()
    ("mtllib m.mtl\nusemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", "newmtl a\nKd 1 1\n"),
    ("mtllib m.mtl\nusemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", "newmtl a\nNs x\n"),
    ("mtllib m.mtl\nusemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", "newmtl a\nillum -1\n"),
    ("mtllib m.mtl\nusemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", "newmtl\n"),
    # the current material carries over from the .obj into the .mtl
    ("mtllib m.mtl\nusemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", "Kd 0.25 0.5 1\nillum 2\n"),
    # usemtl of a name the .mtl lacks: zero-valued material
    ("mtllib m.mtl\nusemtl zz\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", "newmtl a\nKd 1 0 0\n"),
    # no mtllib: usemtl materials are zero-valued, never nil
    ("usemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", None),
    # faces before any usemtl use the name "polyred_default", which a
    # material may carry
    ("mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\nusemtl polyred_default\nf 3 2 1\n",
     "newmtl polyred_default\nKd 0 1 0\nillum 2\n"),
]


@pytest.mark.parametrize("k", range(len(MTL_FALLBACK)))
def test_mtl_fallback_rules(tmp_path, k):
    obj, mtl = MTL_FALLBACK[k]
    path = write(tmp_path, obj, mtl)
    compare_file(path)
    compare_model(path)


def test_mtl_retry_with_obj_name(tmp_path):
    """A malformed mtllib file: the reference retries <name>.mtl beside the
    .obj (with the state the first parse left) and notes it."""
    obj = "mtllib bad.mtl\nusemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n"
    path = write(tmp_path, obj, "newmtl a\nKd 1 1\n", mtlname="bad.mtl")
    (tmp_path / "m.mtl").write_text("newmtl a\nKd 0 0 1\nillum 2\n")
    f = compare_file(path)
    assert f.warnings[-1].endswith("using material file " + str(tmp_path / "m.mtl"))
    assert f.materials["a"]["Diffuse"] == (0, 0, 255, 255)
    compare_model(path)


# ---------------------------------------------------------------- layout

def test_whitespace_line_ends_and_unicode_spaces(tmp_path):
    nbsp, ideo, nel = " ", "　", "\u0085"
    text = ("v\t0 0 0\r\nv 1" + nbsp + "0" + ideo + "0\r\n\x0bv 0\x0c1 0 \r\n"
            "o café x\nf 1 2 3" + nel + "\né unknown\nv 1 1​0 0\n")
    path = write(tmp_path, text.encode("utf-8"))
    f = compare_file(path)
    assert f is None or f.objects[0][0] == "café"


def test_invalid_utf8_is_not_space(tmp_path):
    path = write(tmp_path, b"v 0 0 0\nv 1 0 0\nv 0 1 0\no a\xe2b\xc2\xa0c\nf 1 2 3\xe2\x80\x80\n")
    f = compare_file(path)
    assert f.objects[0][0] == "a\udce2b"


def test_cr_only_file_is_one_line(tmp_path):
    path = write(tmp_path, "v 0 0 0\rv 1 0 0\rv 0 1 0\rf 1 2 3\r")
    compare_file(path)


def test_vertex_w_divides(tmp_path):
    path = write(tmp_path, "v 1 2 3 2\nv 1 2 3 0\nv 1 2 3 1 7\nv 3 3 3 3\nf 1 2 3\n")
    f = compare_file(path)
    assert f.vertices[0].tolist() == [0.5, 1.0, 1.5]
    assert np.isinf(f.vertices[1]).all()
    assert f.vertices[2].tolist() == [1.0, 2.0, 3.0]  # a fifth field: w ignored
    compare_model(path)


# ---------------------------------------------------------------- model.Load

QUAD_TRI = ("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 2 2 0\nvn 0 0 1\nvn 0 0 0\nvt 0 0\n"
            "usemtl a\nf 1/1/1 2/1/1 3/1/1 4/1/1\nf 1/1/2 2/1/1 3/1/1\nusemtl b\nf 1/1/1 2/1/1 3/1/1 4/1/1 5/1/1\n")


def test_mesh_kinds(tmp_path):
    """TriangleMesh / QuadMesh keep face materials and drop polygons; a
    triangle + quad object becomes a PolygonMesh with MaterialID -1."""
    cases = {
        "tris": "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 2 2 0\nusemtl a\nf 1 2 3\nusemtl b\nf 1 3 4\nf 1 2 3 4 5\n",
        "quads": "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 2 2 0\nusemtl b\nf 1 2 3 4\nusemtl a\nf 4 3 2 1\nf 1 2 3 4 5\n",
        "hybrid": QUAD_TRI,
    }
    for name, obj in cases.items():
        path = write(tmp_path, obj, "newmtl a\nKd 1 0 0\nillum 2\nnewmtl b\nKd 0 1 0\nillum 0\n",
                     name=name + ".obj", mtlname="m.mtl")
        path_obj = write(tmp_path, "mtllib m.mtl\n" + obj, name=name + ".obj")
        g = compare_model(path_obj)
        m = g.objects[0].mesh
        if name == "tris":
            assert m.n_tris == 2 and m.mat_id.tolist() == [0, 1]
        elif name == "quads":
            assert m.n_tris == 4 and m.mat_id.tolist() == [0, 0, 1, 1]
        else:
            assert m.n_tris == 1 + 2 + 3 and (m.mat_id == -1).all()
            assert len(g.objects[0].materials) == 2


def test_zero_normal_fixup(tmp_path):
    """A zero corner normal on a triangle face replaces the FIRST corner's
    normal with the face normal (model/load.go:165-176)."""
    obj = ("v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nvn 0 0 0\nvn 0 1e-8 0\n"
           "f 1//1 2//1 3//2\nf 1//3 2//1 3//1\nf 1//1 2//1 3//1\nf 1//2 2//2 3//2 1//2\n")
    g = compare_model(write(tmp_path, obj))
    nor = g.objects[0].mesh.nor
    assert nor[0, 0].tolist() == [0, 0, 1, 0] and nor[0, 2].tolist() == [0, 0, 0, 0]
    assert nor[1, 0].tolist() == [0, 0, 1, 0]


def test_faceless_objects(tmp_path):
    obj = "o empty\no polys\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 2 2 0\nf 1 2 3 4 5\no tri\nf 1 2 3\n"
    path = write(tmp_path, obj)
    with pytest.raises(objload.ObjError, match="'empty'"):
        objload.load(path)
    g = compare_model(path)
    assert len(g.objects) == 1


def test_image_texture_policy(tmp_path):
    """A missing map_Kd file raises (MustLoadImage panics); a file that is
    not PNG raises NotImplementedError; image_textures='ignore' keeps the
    uniform blue texture."""
    path = write(tmp_path, "mtllib m.mtl\nusemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n",
                 "newmtl a\nKd 1 1 1\nillum 2\nmap_Kd tex.png\n")
    with pytest.raises(FileNotFoundError):
        objload.load(path)
    (tmp_path / "tex.png").write_bytes(b"\xff\xd8\xff\xe0" + bytes(16))  # a JPEG header
    with pytest.raises(NotImplementedError, match="tex.png|PNG"):
        objload.load(path)
    g = objload.load(path, image_textures="ignore")
    assert g.objects[0].materials[0].texture == (0, 0, 255, 255)


def test_unsupported_extension(tmp_path):
    path = write(tmp_path, "v 0 0 0\n", name="m.ply")
    with pytest.raises(objload.ObjError, match="unsupported format .ply"):
        objload.load(path)


def test_loaded_scene_flattens(tmp_path):
    """The loaded group goes through the same FlatScene the render path
    uploads: triangles, object ranges and the material table line up."""
    from polyred_gb300 import render, scene as sc
    path = write(tmp_path, "mtllib m.mtl\n" + QUAD_TRI, "newmtl a\nKd 1 0 0\nillum 2\nnewmtl b\nKd 0 1 0\n")
    g = objload.load(path)
    s = sc.Scene(g, sc.Point(position=(0, 2, 2)))
    flat = render.FlatScene(s)
    assert flat.n_tris == 6 and flat.n_objects == 1 and flat.n_materials == 2
    assert flat.mat_id.tolist() == [-1] * 6


def test_null_arguments(native_lib):
    assert native_lib.pr_obj_create(None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_obj_destroy(None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_obj_parse(None, 0, b"", 0) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_obj_get(None, None) == _abi.PR_ERR_INVALID_ARG
    import ctypes as C
    h = C.c_void_p()
    assert native_lib.pr_obj_create(C.byref(h)) == _abi.PR_OK
    assert native_lib.pr_obj_parse(h, 7, b"", 0) == _abi.PR_ERR_INVALID_ARG
    info = _abi.pr_obj_info()
    assert native_lib.pr_obj_get(h, C.byref(info)) == _abi.PR_ERR_INVALID_ARG  # size unset
    assert native_lib.pr_obj_destroy(h) == _abi.PR_OK


def test_nul_bytes_in_names_and_errors(tmp_path):
    """Go strings hold NUL: names, warnings and error messages keep it."""
    path = write(tmp_path, b"o a\x00b\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\nx\x00y 1\n")
    f = compare_file(path)
    assert f.objects[0][0] == "a\x00b" and "x\x00y" in f.warnings[0]
    path = write(tmp_path, b"v 1\x002 3\n", name="e.obj")
    with pytest.raises(objload.ObjError, match="\x00"):
        objload.parse_file(path)
    compare_file(path)


def _mutate(rng, data):
    toks = [b"v", b"f", b"o", b"/", b"//", b"-", b"e", b".", b"0x", b"_", b"inf", b"\t", b"\r\n", b"\n", b" ",
            b"\xc2\xa0", b"\xff", b"\x00", b"1", b"-1", b"2147483648", b"1e39", b"0", b"usemtl", b"Kd", b"illum"]
    data = bytearray(data)
    for _ in range(rng.randrange(1, 6)):
        k, pos = rng.randrange(4), rng.randrange(len(data) + 1)
        if k == 0 and data:
            del data[pos:pos + rng.randrange(1, 8)]
        elif k == 1:
            data[pos:pos] = rng.choice(toks)
        elif k == 2 and data:
            data[min(pos, len(data) - 1)] = rng.randrange(256)
        else:
            data[pos:pos] = bytes(rng.randrange(256) for _ in range(rng.randrange(1, 5)))
    return bytes(data)


@pytest.mark.parametrize("seed", range(150))
def test_mutated_files_match_oracle(tmp_path, seed):
    """Seeded mutations of valid files and random bytes: the same values or
    the same error as the oracle (a larger run of this generator found the
    NUL-byte cases above)."""
    rng = random.Random(0xF022 + seed)
    obj, mtl = random_obj(random.Random(seed), consistent=True)
    obj_b = bytes(rng.randrange(256) for _ in range(rng.randrange(200))) if seed % 5 == 0 else _mutate(rng, obj.encode())
    mtl_b = _mutate(rng, mtl.encode()) if seed % 3 == 0 else mtl.encode()
    path = write(tmp_path, obj_b, mtl_b)
    compare_file(path)
    compare_model(path)
