"""OBJ / MTL loading oracle (TEST INFRASTRUCTURE).

A pure-Python restatement of the reference's model/obj/obj.go (obj.Load and
its line parsers) and model/load.go (loadObj: materials, primitives, mesh
choice), used only by tests/ to check polyred_gb300.objload and the native
pr_obj_* parser. Small inputs only (plain loops).

Numbers are converted independently of the product: Go's strconv grammar is
matched with regular expressions and the value is rounded to float32 from an
exact rational (round half to even, an error at 2^128 and above).

Parity pins: the reference ships no outputs for its loader; its tests only
load internal/testdata/*.obj without error (model/obj/obj_test.go:14-26,
model/load_test.go:19-31). tests/golden/make_obj_fixtures.py records what
this oracle reads from those assets, checked there against counts and
values taken from the files' text by a separate scan.
"""
import math
import os
import re
from fractions import Fraction

import numpy as np

F32 = np.float32
INV_INDEX = 4294967295  # obj.go:73 invINDEX = math.MaxUint32

# unicode.IsSpace as bytes: ASCII \t \n \v \f \r ' ', then U+0085, U+00A0,
# U+1680, U+2000-U+200A, U+2028, U+2029, U+202F, U+205F, U+3000 in UTF-8.
_SPACE = re.compile(rb"(?:[\t\n\v\f\r ]|\xc2[\x85\xa0]|\xe1\x9a\x80|\xe2\x80[\x80-\x8a\xa8\xa9\xaf]"
                    rb"|\xe2\x81\x9f|\xe3\x80\x80)+")


class GoError(Exception):
    """An error value the reference returns."""


class GoPanic(Exception):
    """A panic in the reference."""


def fields(line):
    """strings.Fields (Go), on bytes."""
    return [f for f in _SPACE.split(line) if f]


# ---------------------------------------------------------------- strconv

def _quote(b):
    out = []
    for c in b:
        ch = chr(c)
        if ch == '"':
            out.append('\\"')
        elif ch == "\\":
            out.append("\\\\")
        elif ch in "\a\b\f\n\r\t\v":
            out.append({"\a": "\\a", "\b": "\\b", "\f": "\\f", "\n": "\\n", "\r": "\\r", "\t": "\\t",
                        "\v": "\\v"}[ch])
        elif c < 0x20 or c >= 0x7F:
            out.append("\\x%02x" % c)
        else:
            out.append(ch)
    return '"' + "".join(out) + '"'


def _numerr(fn, s, rng=False):
    return GoError(f"strconv.{fn}: parsing {_quote(s)}: " + ("value out of range" if rng else "invalid syntax"))


def _underscore_ok(s):
    """strconv.underscoreOK."""
    saw = "^"
    i = 0
    if s[:1] in (b"+", b"-"):
        s = s[1:]
    hexa = False
    if len(s) >= 2 and s[0:1] == b"0" and s[1:2].lower() in (b"b", b"o", b"x"):
        i, saw, hexa = 2, "0", s[1:2].lower() == b"x"
    while i < len(s):
        c = s[i:i + 1]
        if c.isdigit() or (hexa and c.lower() in b"abcdef" and c != b""):
            saw = "0"
        elif c == b"_":
            if saw != "0":
                return False
            saw = "_"
        else:
            if saw == "_":
                return False
            saw = "!"
        i += 1
    return saw != "_"


_DEC = re.compile(rb"(?P<sign>[+-]?)(?P<int>[0-9_]*)(?:\.(?P<frac>[0-9_]*))?(?:[eE](?P<exp>[+-]?[0-9][0-9_]*))?")
_HEX = re.compile(rb"(?P<sign>[+-]?)0[xX](?P<int>[0-9a-fA-F_]*)(?:\.(?P<frac>[0-9a-fA-F_]*))?"
                  rb"[pP](?P<exp>[+-]?[0-9][0-9_]*)")


def _go_exp(e):
    """readFloat's exponent: digits accumulate while the value is < 10000."""
    sign = -1 if e[:1] == b"-" else 1
    v = 0
    for c in e.lstrip(b"+-").replace(b"_", b""):
        if v < 10000:
            v = v * 10 + (c - 48)
    return sign * v


def _to_f32(x):
    """Round a non-negative rational to float32, half to even; None when the
    result is 2^128 or more."""
    if x == 0:
        return 0.0
    e = x.numerator.bit_length() - x.denominator.bit_length()
    if Fraction(2) ** e > x:
        e -= 1
    e = max(e, -126)
    scaled = x / Fraction(2) ** (e - 23)
    m = scaled.numerator // scaled.denominator
    r = scaled - m
    if r > Fraction(1, 2) or (r == Fraction(1, 2) and m % 2 == 1):
        m += 1
    v = Fraction(m) * Fraction(2) ** (e - 23)
    if v >= Fraction(2) ** 128:
        return None
    return float(v)


def parse_float32(s):
    """strconv.ParseFloat(s, 32) as a float32 value."""
    low = s.lower()
    body = low[1:] if low[:1] in (b"+", b"-") else low
    neg = low[:1] == b"-"
    if low[:1] in (b"+", b"-") or low[:1] == b"i":
        if body in (b"inf", b"infinity"):
            return F32(-math.inf if neg else math.inf)
    if low == b"nan":
        return F32(math.nan)
    m = None
    if len(body) > 2 and body[:2] == b"0x":
        m = _HEX.fullmatch(s)
        base = 16
    else:
        m = _DEC.fullmatch(s)
        base = 10
    if m is None:
        raise _numerr("ParseFloat", s)
    ip = m.group("int") or b""
    fp = m.group("frac") or b""
    digits = (ip + fp).replace(b"_", b"")
    if not digits:
        raise _numerr("ParseFloat", s)
    if b"_" in s and not _underscore_ok(s):
        raise _numerr("ParseFloat", s)
    nfrac = len(fp.replace(b"_", b""))
    exp = _go_exp(m.group("exp")) if m.group("exp") else 0
    mant = int(digits, base)
    if base == 10:
        val = Fraction(mant) * Fraction(10) ** (exp - nfrac)
    else:
        val = Fraction(mant) * Fraction(2) ** (exp - 4 * nfrac)
    r = _to_f32(val)
    if r is None:
        raise _numerr("ParseFloat", s, True)
    return F32(-r if neg else r)


def parse_int32(s):
    """strconv.ParseInt(s, 10, 32)."""
    body = s[1:] if s[:1] in (b"+", b"-") else s
    if not body or not all(48 <= c <= 57 for c in body):
        raise _numerr("ParseInt", s)
    v = int(body)
    if s[:1] == b"-":
        v = -v
    if v < -(1 << 31) or v >= (1 << 31):
        raise _numerr("ParseInt", s, True)
    return v


def parse_uint32(s):
    """strconv.ParseUint(s, 10, 32)."""
    if not s or not all(48 <= c <= 57 for c in s):
        raise _numerr("ParseUint", s)
    v = int(s)
    if v >= (1 << 32):
        raise _numerr("ParseUint", s, True)
    return v


def from_value32(r, g, b, a):
    """color.FromValue[float32] (color/color.go:33-44)."""
    vals = [F32(v) for v in (r, g, b, a)]
    for v in vals:
        if v < 0 or v > 1:
            raise GoPanic(f"out of range [0, 1], got {tuple(float(x) for x in vals)}")
    out = []
    for v in vals:
        x = float(F32(v * F32(255)))
        if math.isnan(x):
            out.append(0)
        else:
            out.append(int(math.floor(x + 0.5)) if x >= 0 else int(math.ceil(x - 0.5)))
    return tuple(out)


# ---------------------------------------------------------------- obj.File

class Material:
    """obj.Material (obj.go:57-68)."""

    def __init__(self, name):
        self.Name = name
        self.Illum = 0
        self.Opacity = F32(0)
        self.Refraction = F32(0)
        self.Shininess = F32(0)
        self.Ambient = (0, 0, 0, 0)
        self.Diffuse = (0, 0, 0, 0)
        self.Specular = (0, 0, 0, 0)
        self.Emissive = (0, 0, 0, 0)
        self.MapKd = ""


class Face:
    def __init__(self, n):
        self.Vertices = [0] * n
        self.Uvs = [0] * n
        self.Normals = [0] * n
        self.Material = ""
        self.Smooth = False


class Object:
    def __init__(self, name):
        self.Name = name
        self.Faces = []
        self.Materials = []


def _s(b):
    return b.decode("utf-8", errors="surrogateescape")


class File:
    """obj.File and its parsers (obj.go:26-611)."""

    def __init__(self):
        self.Objs = []
        self.Matlib = ""
        self.Materials = {}
        self.Vertices = []
        self.Normals = []
        self.Uvs = []
        self.Warnings = []
        self.MtlDir = ""
        self.line = 1
        self.objCurrent = None
        self.matCurrent = None
        self.smoothCurrent = False

    def parse(self, data, parse_line):
        """File.parse (obj.go:139-159): returns the error, or None."""
        self.line = 1
        lines = data.split(b"\n")
        for k, line in enumerate(lines):
            try:
                parse_line(line)
            except GoError as e:
                return e
            if k == len(lines) - 1:
                break
            self.line += 1
        return None

    def format_error(self, msg):
        return GoError(f"{msg} in line:{self.line}")

    def warn(self, ftype, msg):
        self.Warnings.append(f"{ftype}({self.line}): {msg}")

    # ---- .obj lines (obj.go:161-395)
    def parse_obj_line(self, line):
        fs = fields(line)
        if not fs or fs[0].startswith(b"#"):
            return
        t, rest = fs[0], fs[1:]
        if t == b"mtllib":
            if len(rest) < 1:
                raise self.format_error("Material library (mtllib) with no fields")
            self.Matlib = _s(rest[0])
        elif t in (b"o", b"g"):
            self.parse_object(rest)
        elif t == b"v":
            if len(rest) < 3:
                raise self.format_error("vertex has less than 3 vertices in 'v' line: [%s]"
                                        % " ".join(_s(x) for x in rest))
            w = F32(1)
            if len(rest) == 4:
                w = F32(1) / parse_float32(rest[3])
            for x in rest[:3]:
                v = parse_float32(x)
                self.Vertices.append(v if w == 1 else F32(v * w))
        elif t == b"vn":
            if len(rest) < 3:
                raise self.format_error("normal has less than 3 vertices in 'vn' line: [%s]"
                                        % " ".join(_s(x) for x in rest))
            for x in rest[:3]:
                self.Normals.append(parse_float32(x))
        elif t == b"vt":
            if len(rest) < 2:
                raise self.format_error("Less than 2 texture coords. in 'vt' line")
            for x in rest[:2]:
                self.Uvs.append(parse_float32(x))
        elif t == b"f":
            self.parse_face(rest)
        elif t == b"usemtl":
            if len(rest) < 1:
                raise self.format_error("Usemtl with no fields")
            if self.objCurrent is None:
                self.parse_object([b"unnamed%d" % self.line])
            name = _s(rest[0])
            mat = self.Materials.get(name)
            if mat is None:
                mat = Material(name)
                self.Materials[name] = mat
            self.objCurrent.Materials.append(name)
            self.matCurrent = mat
        elif t == b"s":
            if len(rest) < 1:
                raise self.format_error("'s' with no fields")
            self.smoothCurrent = not (rest[0] == b"0" or rest[0] == b"off")
        else:
            self.warn("obj", "unsupported field: " + _s(t))

    def parse_object(self, rest):
        if len(rest) < 1:
            raise self.format_error("obj line (o) with no fields")
        self.Objs.append(Object(_s(rest[0])))
        self.objCurrent = self.Objs[-1]

    def _index(self, s, count, zero_msg):
        v = parse_int32(s)
        if v > 0:
            return v - 1
        if v < 0:
            return (count - 1) + v + 1
        raise self.format_error(zero_msg)

    def parse_face(self, rest):
        if self.objCurrent is None:
            self.parse_object([b"unnamed%d" % self.line])
        if not self.objCurrent.Materials and self.matCurrent is not None:
            self.objCurrent.Materials.append(self.matCurrent.Name)
        if len(rest) < 3:
            raise self.format_error("face line with less 3 fields")
        face = Face(len(rest))
        face.Material = self.matCurrent.Name if self.matCurrent is not None else "polyred_default"
        face.Smooth = self.smoothCurrent
        for pos, fi in enumerate(rest):
            vf = fi.split(b"/")
            face.Vertices[pos] = self._index(vf[0], len(self.Vertices) // 3, "face vertex index value equal to 0")
            if len(vf) > 1 and len(vf[1]) > 0:
                face.Uvs[pos] = self._index(vf[1], len(self.Uvs) // 2, "face uv index value equal to 0")
            else:
                face.Uvs[pos] = INV_INDEX
            if len(vf) >= 3:
                face.Normals[pos] = self._index(vf[2], len(self.Normals) // 3, "face normal index value equal to 0")
            else:
                face.Normals[pos] = INV_INDEX
        self.objCurrent.Faces.append(face)

    # ---- .mtl lines (obj.go:397-611)
    def parse_mtl_line(self, line):
        fs = fields(line)
        if not fs or fs[0].startswith(b"#"):
            return
        t, rest = fs[0], fs[1:]
        ts = _s(t)
        if t == b"newmtl":
            if len(rest) < 1:
                raise self.format_error("newmtl with no fields")
            name = _s(rest[0])
            mat = self.Materials.get(name)
            if mat is None:
                mat = Material(name)
                self.Materials[name] = mat
            self.matCurrent = mat
        elif t in (b"Ka", b"Kd", b"Ke", b"Ks"):
            if len(rest) < 3:
                raise self.format_error(f"'{ts}' with less than 3 fields")
            c = [parse_float32(x) for x in rest[:3]]
            col = from_value32(c[0], c[1], c[2], 1)
            m = self._current()
            setattr(m, {"Ka": "Ambient", "Kd": "Diffuse", "Ke": "Emissive", "Ks": "Specular"}[ts], col)
        elif t in (b"d", b"Ni", b"Ns"):
            if len(rest) < 1:
                raise self.format_error(f"'{ts}' with no fields")
            try:
                v = parse_float32(rest[0])
            except GoError:
                raise self.format_error("'d' parse float error")
            setattr(self._current(), {"d": "Opacity", "Ni": "Refraction", "Ns": "Shininess"}[ts], v)
        elif t == b"illum":
            if len(rest) < 1:
                raise self.format_error("'illum' with no fields")
            try:
                v = parse_uint32(rest[0])
            except GoError:
                raise self.format_error("'d' parse int error")
            self._current().Illum = v
        elif t == b"map_Kd":
            if len(rest) < 1:
                raise self.format_error("No fields")
            self._current().MapKd = _s(rest[0])
        else:
            self.warn("mtl", "field not supported: " + ts)

    def _current(self):
        if self.matCurrent is None:
            raise GoPanic("invalid memory address or nil pointer dereference")
        return self.matCurrent


def _go_join(*parts):
    parts = [p for p in parts if p]
    return os.path.normpath("/".join(parts)) if parts else ""


def load_file(objpath):
    """obj.Load (obj.go:78-137). Raises GoError / GoPanic / OSError."""
    with np.errstate(all="ignore"):
        return _load_file(objpath)


def _load_file(objpath):
    with open(objpath, "rb") as fh:
        data = fh.read()
    f = File()
    err = f.parse(data, f.parse_obj_line)
    if err is not None:
        raise err
    if f.Matlib != "":
        objdir = os.path.dirname(objpath) or "."
        objdir = os.path.normpath(objdir)
        f.MtlDir = objdir
        with open(_go_join(objdir, f.Matlib), "rb") as fh:  # panic(errMTL) when missing
            err = f.parse(fh.read(), f.parse_mtl_line)
    if err is not None:
        stem = objpath[:-4] if objpath.endswith(".obj") else objpath
        f.MtlDir = stem
        try:
            fh = open(stem + ".mtl", "rb")
        except OSError:
            fh = None
        if fh is not None:
            with fh:
                err = f.parse(fh.read(), f.parse_mtl_line)
            if err is None:
                f.warn("mtl", f"using material file {stem}.mtl")
    if err is not None:
        for k in f.Materials:
            f.Materials[k] = None
        f.warn("mtl", "unable to parse a material file for obj. using default material instead.")
    return f


# ---------------------------------------------------------------- model.Load

def _fma32(x, y, z):
    """float32(math.FMA(float64(x), float64(y), float64(z)))."""
    xs = (float(x), float(y), float(z))
    if not all(math.isfinite(v) and v != 0 for v in xs):
        # math.FMA's own special case (zero, Inf or NaN operand): x*y + z,
        # which keeps the sign of a zero result
        return F32(xs[0] * xs[1] + xs[2])
    exact = Fraction(xs[0]) * Fraction(xs[1]) + Fraction(xs[2])
    return F32(float(exact))


def _sub(a, b):
    return [F32(a[i] - b[i]) for i in range(4)]


def _is_zero(v):
    eps = F32(1e-7)
    return abs(F32(v[0])) <= eps and abs(F32(v[1])) <= eps and abs(F32(v[2])) <= eps


def _tri_normal(p1, p2, p3):
    """Triangle.Normal (geometry/primitive/triangle.go:130-139)."""
    v2v1 = _sub(p1, p2)
    v2v3 = _sub(p3, p2)
    u, v = v2v3, v2v1
    x = _fma32(u[1], v[2], F32(-(u[2] * v[1])))
    y = _fma32(u[2], v[0], F32(-(u[0] * v[2])))
    z = _fma32(u[0], v[1], F32(-(u[1] * v[0])))
    w = F32(0)
    d = _fma32(x, x, _fma32(y, y, _fma32(z, z, F32(w * w))))
    ln = F32(math.sqrt(float(d)))
    with np.errstate(divide="ignore", invalid="ignore"):
        n = F32(F32(1.0) / ln)
        return [F32(x * n), F32(y * n), F32(z * n), F32(w * n)]


def _vertex(f, face, i, n_verts=None):
    vs = face.Vertices
    k = vs[i]
    if k < 0 or 3 * k + 2 >= len(f.Vertices):
        raise GoPanic("index out of range")
    pos = [f.Vertices[3 * k], f.Vertices[3 * k + 1], f.Vertices[3 * k + 2], F32(1)]
    nor = [F32(0)] * 4
    if len(f.Normals) > 0:
        k = face.Normals[i]
        if k < 0 or 3 * k + 2 >= len(f.Normals):
            raise GoPanic("index out of range")
        nor = [f.Normals[3 * k], f.Normals[3 * k + 1], f.Normals[3 * k + 2], F32(0)]
    uv = [F32(0), F32(0)]
    if len(f.Uvs) > 0:
        k = face.Uvs[i]
        if k < 0 or 2 * k + 1 >= len(f.Uvs):
            raise GoPanic("index out of range")
        uv = [f.Uvs[2 * k], f.Uvs[2 * k + 1]]
    return {"pos": pos, "nor": nor, "uv": uv}


def _from_value64(*vals):
    """color.FromValue[float64] with constant arguments: r*255 in float64,
    rounded half away from zero (0.7*255 is 178.5 in float64)."""
    return tuple(int(math.floor(float(v) * 255.0 + 0.5)) for v in vals)


DEFAULT = {"name": "default", "diffuse": _from_value64(0.7, 0.7, 0.7, 1.0),
           "specular": _from_value64(0.5, 0.5, 0.5, 1.0), "shininess": F32(30),
           "texture": (0, 0, 255, 255)}  # material/pool.go:17-29


def load_model(path, image_textures="error"):
    """model.Load -> list of geometries, each {"tris": [(v1, v2, v3, mat)],
    "materials": [material dicts]}; None for a geometry with a nil mesh."""
    with np.errstate(all="ignore"):
        return _load_model(path, image_textures)


def _load_model(path, image_textures):
    if os.path.splitext(path)[1] != ".obj":
        raise GoError("model: unsupported format " + os.path.splitext(path)[1])
    try:
        fi = load_file(path)
    except GoError as e:
        raise GoError(f"model: cannot load the given file {path}: {e}")
    all_mats = {}
    for name, m in fi.Materials.items():
        if m is None:
            continue
        if m.Illum not in (0, 2):
            raise GoPanic("unsupported illumination model")
        if m.MapKd and image_textures != "ignore":
            raise NotImplementedError("image texture")
        all_mats[name] = {"name": name, "diffuse": m.Diffuse, "specular": m.Specular, "shininess": m.Shininess,
                          "texture": (0, 0, 255, 255)}
    geoms = []
    for ob in fi.Objs:
        tris, quads, polys = [], [], []
        geom_mats, local = [], {}
        for face in ob.Faces:
            mat = all_mats.get(face.Material) or DEFAULT
            if id(mat) not in local:
                local[id(mat)] = len(geom_mats)
                geom_mats.append(mat)
            mid = local[id(mat)]
            n = len(face.Vertices)
            vs = [_vertex(fi, face, i) for i in range(n)]
            if n == 3:
                if len(fi.Normals) > 0:
                    for k in range(3):
                        if _is_zero(vs[k]["nor"]):
                            vs[0]["nor"] = _tri_normal(vs[0]["pos"], vs[1]["pos"], vs[2]["pos"])
                tris.append((vs, mid))
            elif n == 4:
                quads.append((vs, mid))
            else:
                polys.append((vs, mid))
        out = []
        if tris and not quads:
            out = [(v[0], v[1], v[2], mid) for v, mid in tris]
        elif quads and not tris:
            for v, mid in quads:
                out += [(v[0], v[1], v[2], mid), (v[0], v[2], v[3], mid)]
        elif tris and quads:
            for v, _ in tris + quads + polys:
                out += [(v[0], v[i + 1], v[i + 2], -1) for i in range(len(v) - 2)]
        else:
            geoms.append(None)
            continue
        geoms.append({"tris": out, "materials": geom_mats, "name": ob.Name})
    return geoms
