"""Wavefront OBJ / MTL loading: model.Load (model/load.go:23-152) and
obj.Load (model/obj/obj.go:78-137) for the render path's host.

  parse_file(path)  -> ObjFile   obj.Load: the .obj text, then the .mtl its
                                 mtllib names (or <name>.mtl), parsed by the
                                 native pr_obj_* parser into flat arrays
  load(path)        -> Group     model.Load: one Geometry per OBJ object,
                                 meshes assembled with numpy from the flat
                                 arrays, in the reference's triangle order

The parse runs in libpolyred_cuda.so (C++, one pass, no per-line Python);
there is no Python parser to fall back to. Differences from the reference,
each an error where the reference would go on:

  - an object whose faces give no mesh (no faces, or only polygons of five
    or more corners, or triangles with such polygons but no quads) raises
    ValueError here; the reference builds a Geometry with a nil mesh, which
    panics on first use (AABB, Triangles);
  - map_Kd images are decoded by polyred_gb300.imageload, which reads PNG
    only; another format raises NotImplementedError (image_textures="ignore"
    gives such materials the uniform blue texture instead).
"""
import ctypes as C
import os
import struct

import numpy as np

from . import _abi, native
from . import scene as sc

F32 = np.float32

DEFAULT_NAME = "polyred_default"  # obj.go's material name of faces before any usemtl


class ObjError(ValueError):
    """obj.Load / model.Load returned an error for this input."""


class ObjPanic(RuntimeError):
    """The reference panics on this input (e.g. an .mtl colour outside
    [0, 1], an .mtl property before any newmtl, illum other than 0 or 2)."""


def _entry(blob, off):
    """One string of the parser's table: uint32 length, bytes, NUL."""
    n = struct.unpack_from("=I", blob, off)[0]
    return blob[off + 4:off + 4 + n].decode("utf-8", errors="surrogateescape")


def _info(lib, handle):
    info = _abi.pr_obj_info()
    info.size = C.sizeof(_abi.pr_obj_info)
    native.check(lib.pr_obj_get(handle, C.byref(info)))
    return info


def _np(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class ObjFile:
    """obj.File (obj.go:26-41) as flat arrays.

    vertices [n,3] f32, normals [n,3] f32, uvs [n,2] f32;
    face_start [n_faces+1] i64 and corner_v/vt/vn [n_corners] i64 (0-based,
    relative indices resolved, PR_OBJ_NO_INDEX where a corner has no vt/vn);
    face_object, face_material (-1 = "polyred_default") [n_faces] i32;
    face_smooth [n_faces] bool; objects: list of (name, [material names]);
    materials: name -> dict of the obj.Material fields, or None once a failed
    .mtl parse reset them; warnings, matlib, mtl_dir as in the reference.
    """

    def __init__(self, handle, lib):
        info = _abi.pr_obj_info()
        info.size = C.sizeof(_abi.pr_obj_info)
        native.check(lib.pr_obj_get(handle, C.byref(info)))
        blob = C.string_at(info.strings, info.strings_len) if info.strings_len else b""

        def s(off):
            return _entry(blob, off)

        self.vertices = _np(info.vertices, 3 * info.n_vertices, F32).reshape(-1, 3)
        self.normals = _np(info.normals, 3 * info.n_normals, F32).reshape(-1, 3)
        self.uvs = _np(info.uvs, 2 * info.n_uvs, F32).reshape(-1, 2)
        self.face_start = _np(info.face_start, info.n_faces + 1, np.int64)
        self.corner_v = _np(info.corner_v, info.n_corners, np.int64)
        self.corner_vt = _np(info.corner_vt, info.n_corners, np.int64)
        self.corner_vn = _np(info.corner_vn, info.n_corners, np.int64)
        self.face_object = _np(info.face_object, info.n_faces, np.int32)
        self.face_material = _np(info.face_material, info.n_faces, np.int32)
        self.face_smooth = _np(info.face_smooth, info.n_faces, np.uint8).astype(bool)
        mats = [info.materials[i] for i in range(info.n_materials)]
        self.material_names = [s(m.name) for m in mats]
        self.materials = {}
        for name, m in zip(self.material_names, mats):
            self.materials[name] = {
                "Name": name, "Illum": int(m.illum), "Opacity": F32(m.opacity),
                "Refraction": F32(m.refraction), "Shininess": F32(m.shininess),
                "Ambient": tuple(m.ambient), "Diffuse": tuple(m.diffuse),
                "Specular": tuple(m.specular), "Emissive": tuple(m.emissive),
                "MapKd": s(m.map_kd) if m.map_kd >= 0 else "",
            }
        ms = _np(info.object_mat_start, info.n_objects + 1, np.int64)
        om = _np(info.object_mat, int(ms[-1]) if info.n_objects else 0, np.int32)
        self.objects = [(s(info.object_name[i]), [self.material_names[k] for k in om[ms[i]:ms[i + 1]]])
                        for i in range(info.n_objects)]
        self.warnings = [s(info.warnings[i]) for i in range(info.n_warnings)]
        self.matlib = s(info.matlib) if info.matlib >= 0 else ""
        self.line = int(info.line)
        self.mtl_dir = ""

    @property
    def n_faces(self):
        return len(self.face_object)

    def face_material_names(self):
        names = np.array(self.material_names + [DEFAULT_NAME], dtype=object)
        return names[self.face_material]  # -1 picks DEFAULT_NAME


def _go_join(*parts):
    """filepath.Join: join with '/', then Clean (absolute later parts do not
    reset the path, unlike os.path.join)."""
    parts = [p for p in parts if p]
    if not parts:
        return ""
    return os.path.normpath("/".join(parts))


def _go_dir(path):
    """filepath.Dir: everything but the last element, cleaned; "." if none."""
    d = os.path.dirname(path)
    return os.path.normpath(d) if d else "."


def _feed(lib, handle, kind, data):
    st = lib.pr_obj_parse(handle, kind, data, len(data))
    if st == _abi.PR_OK:
        return None
    info = _info(lib, handle)  # the message with every byte (pr_last_error stops at a NUL)
    msg = C.string_at(info.error, info.error_len).decode("utf-8", errors="surrogateescape") if info.error_len \
        else lib.pr_last_error().decode("utf-8", errors="replace")
    if st == _abi.PR_ERR_FATAL:
        raise ObjPanic(msg)
    if st == _abi.PR_ERR_INVALID_ARG:
        return msg
    native.check(st)


def _matlib(lib, handle):
    info = _info(lib, handle)
    if info.matlib < 0:
        return ""
    return _entry(C.string_at(info.strings, info.strings_len), info.matlib)


def parse_file(path):
    """obj.Load (obj.go:78-137). Raises ObjError where it returns an error,
    ObjPanic (or FileNotFoundError for a missing mtllib file) where it
    panics."""
    lib = native.load()
    with open(path, "rb") as fh:
        text = fh.read()
    h = C.c_void_p()
    native.check(lib.pr_obj_create(C.byref(h)))
    try:
        err = _feed(lib, h, _abi.PR_OBJ_TEXT_OBJ, text)
        if err is not None:
            raise ObjError(err)
        matlib = _matlib(lib, h)
        mtl_dir = ""
        note = None
        if matlib:
            mtl_dir = _go_dir(path)
            with open(_go_join(mtl_dir, matlib), "rb") as fh:  # the reference panics when it is missing
                err = _feed(lib, h, _abi.PR_OBJ_TEXT_MTL, fh.read())
        if err is not None:
            # the mtllib file did not parse: try <name>.mtl beside the .obj
            mtl_dir = path[:-4] if path.endswith(".obj") else path
            mtlpath = mtl_dir + ".mtl"
            if os.path.isfile(mtlpath):
                with open(mtlpath, "rb") as fh:
                    err = _feed(lib, h, _abi.PR_OBJ_TEXT_MTL, fh.read())
                if err is None:
                    note = f"using material file {mtlpath}"
        f = ObjFile(h, lib)
        f.mtl_dir = mtl_dir
        if err is not None:
            for k in f.materials:
                f.materials[k] = None
            note = "unable to parse a material file for obj. using default material instead."
        if note is not None:
            f.warnings.append(f"mtl({f.line}): {note}")
        return f
    finally:
        lib.pr_obj_destroy(h)


# ---------------------------------------------------------------- model.Load

def default_material():
    """material.Default() (material/pool.go:15-29): one shared instance."""
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = sc.BlinnPhong(diffuse=sc.color_from_value(0.7, 0.7, 0.7, 1.0),
                                 specular=sc.color_from_value(0.5, 0.5, 0.5, 1.0), shininess=30.0,
                                 texture=BLUE)
    return _DEFAULT


_DEFAULT = None
BLUE = (0, 0, 255, 255)  # color.Blue


def _materials(f, path, image_textures):
    """loadObj's material table (model/load.go:47-84): name -> BlinnPhong for
    every material the .mtl left in place; a map_Kd image is loaded with
    GammaCorrect(true) and sampled with isotropic mipmaps."""
    from . import imageload
    out = {}
    for name, m in f.materials.items():
        if m is None:
            continue
        if m["Illum"] not in (0, 2):
            raise ObjPanic("unsupported illumination model")
        texture = BLUE
        if m["MapKd"] and image_textures != "ignore":
            tex = _go_join(os.path.normpath(f.mtl_dir), os.path.normpath(m["MapKd"]))
            try:
                texture = sc.ImageTexture(imageload.load_image(tex, gamma_correct=True), mipmap=True)
            except NotImplementedError as e:
                raise NotImplementedError(f"material {name!r} of {path}: {e} (pass image_textures='ignore' to "
                                          "render it with the uniform blue texture)") from None
        out[name] = sc.BlinnPhong(diffuse=m["Diffuse"], specular=m["Specular"], shininess=m["Shininess"],
                                  texture=texture, flat_shading=False, ambient_occlusion=False,
                                  receive_shadow=False)
    return out


def _is_zero(n):
    """Vec4.IsZero (math/vec4.go:64-70): |x|, |y|, |z| <= float32(1e-7)."""
    eps = F32(1e-7)
    return (np.abs(n[..., 0]) <= eps) & (np.abs(n[..., 1]) <= eps) & (np.abs(n[..., 2]) <= eps)


def _fma32(x, y, z):
    """math.FMA[float32] (math/math.go:265-267): the float32 product is exact
    in float64, so one float64 add rounds as fma64 does; then to float32."""
    return (x.astype(np.float64) * y.astype(np.float64) + z.astype(np.float64)).astype(F32)


def _face_normal(p1, p2, p3):
    """Triangle.Normal (geometry/primitive/triangle.go:130-139):
    (v3 - v2) x (v1 - v2), normalised, all in float32 with Go's FMA order."""
    with np.errstate(all="ignore"):
        a = p3 - p2  # v2v3
        b = p1 - p2  # v2v1
        x = _fma32(a[:, 1], b[:, 2], -(a[:, 2] * b[:, 1]))
        y = _fma32(a[:, 2], b[:, 0], -(a[:, 0] * b[:, 2]))
        z = _fma32(a[:, 0], b[:, 1], -(a[:, 1] * b[:, 0]))
        w = np.zeros_like(x)
        d = _fma32(x, x, _fma32(y, y, _fma32(z, z, w * w)))
        ln = np.sqrt(d.astype(np.float64)).astype(F32)
        n = F32(1.0) / ln
        return np.stack([x * n, y * n, z * n, w * n], axis=1)


def _check_range(idx, n, what, path):
    if idx.size and (idx.min() < 0 or idx.max() >= n):
        bad = idx[(idx < 0) | (idx >= n)][0]
        raise ObjPanic(f"{path}: {what} index {bad} out of range [0, {n})")


def load(path, image_textures="load", skip_faceless=False):
    """model.Load (model/load.go:23-38, loadObj 40-152): a Group holding one
    Geometry per OBJ object ('o' / 'g'), each with its own materials.

    Per object, faces become triangles as the reference meshes them:
    triangles only (polygons dropped) -> TriangleMesh, face order;
    quads only (polygons dropped) -> QuadMesh, (v0,v1,v2),(v0,v2,v3) per quad;
    triangles and quads -> PolygonMesh: triangles, then quads, then polygons,
    each fanned from its first corner, all with MaterialID -1 (NewPolygon's
    default). Vertices: position (x,y,z,1); normal (x,y,z,0) when the file
    has any normal, else zero, and on triangle faces the first corner takes
    the face normal when any corner's normal is zero (load.go:165-176); UV
    when the file has any, else zero; colour white.
    """
    ext = os.path.splitext(path)[1]
    if ext != ".obj":
        raise ObjError(f"model: unsupported format {ext}")
    try:
        f = parse_file(path)
    except ObjError as e:
        raise ObjError(f"model: cannot load the given file {path}: {e}") from None
    return build_group(f, path, image_textures, skip_faceless)


def build_group(f, path="", image_textures="load", skip_faceless=False):
    """loadObj's second half (model/load.go:47-152) on a parsed ObjFile."""
    mats = _materials(f, path, image_textures)
    default = default_material()
    names = f.material_names

    # The material of every face as a key into `table` (parsed materials by
    # index, then material.Default()); a key stands for one material
    # instance, as loadObj's pointer-keyed localIndex does. Faces without a
    # usemtl look up the name "polyred_default" like any other.
    table = [mats.get(n) for n in names] + [default]
    dflt = len(names)
    keys = [k if m is not None else dflt for k, m in enumerate(table[:-1])]
    keys.append(names.index(DEFAULT_NAME) if DEFAULT_NAME in mats else dflt)
    keys = np.array(keys, np.int64)
    fkey = keys[f.face_material] if f.n_faces else np.zeros(0, np.int64)  # -1 picks the last slot

    counts = np.diff(f.face_start)
    nv = len(f.vertices)
    has_nor = len(f.normals) > 0
    has_uv = len(f.uvs) > 0
    # every face builds its primitive, including those the mesh drops later
    _check_range(f.corner_v, nv, "vertex", path)
    if has_nor:
        _check_range(f.corner_vn, len(f.normals), "normal", path)
    if has_uv:
        _check_range(f.corner_vt, len(f.uvs), "uv", path)

    pos_c = np.concatenate([f.vertices, np.ones((nv, 1), F32)], axis=1)[f.corner_v] if nv else np.zeros((0, 4), F32)
    nor_c = (np.concatenate([f.normals, np.zeros((len(f.normals), 1), F32)], axis=1)[f.corner_vn]
             if has_nor else np.zeros((len(f.corner_v), 4), F32))
    uv_c = f.uvs[f.corner_vt] if has_uv else np.zeros((len(f.corner_v), 2), F32)

    if has_nor:
        # newTrianglePrimitive's fix-up: V1.Nor = t.Normal() when any corner's
        # normal is zero (each of its three checks assigns V1)
        tri_faces = np.nonzero(counts == 3)[0]
        if tri_faces.size:
            c0 = f.face_start[tri_faces]
            zero = _is_zero(nor_c[c0]) | _is_zero(nor_c[c0 + 1]) | _is_zero(nor_c[c0 + 2])
            fix = c0[zero]
            if fix.size:
                nor_c[fix] = _face_normal(pos_c[fix], pos_c[fix + 1], pos_c[fix + 2])

    group = sc.Group()
    order = np.argsort(f.face_object, kind="stable")
    bounds = np.searchsorted(f.face_object[order], np.arange(len(f.objects) + 1))
    for oi, (oname, _) in enumerate(f.objects):
        faces = order[bounds[oi]:bounds[oi + 1]]
        # geometry-local material indices in order of first use
        fk = fkey[faces]
        uniq, first = np.unique(fk, return_index=True)
        used = uniq[np.argsort(first)]
        local = np.empty(len(table), np.int32)
        local[used] = np.arange(len(used), dtype=np.int32)
        geom_mats = [table[k] for k in used]
        fmat = local[fk] if faces.size else np.zeros(0, np.int32)

        nc = counts[faces]
        tris, quads, polys = faces[nc == 3], faces[nc == 4], faces[nc >= 5]
        if tris.size and not quads.size:
            corners, tmat = _fan(f.face_start, tris, 3), fmat[nc == 3]
        elif quads.size and not tris.size:
            corners, tmat = _fan(f.face_start, quads, 4), np.repeat(fmat[nc == 4], 2)
        elif tris.size and quads.size:
            corners = np.concatenate([_fan(f.face_start, tris, 3), _fan(f.face_start, quads, 4),
                                      _fan_polygons(f.face_start, counts, polys)])
            tmat = np.full(len(corners), -1, np.int32)
        else:
            if skip_faceless:
                continue
            raise ObjError(f"model: object {oname!r} of {path} has no triangle or quad faces; the reference "
                           "builds no mesh for it")
        mesh = sc.Mesh(pos_c[corners], nor_c[corners], uv_c[corners], None, tmat)
        group.add(sc.Geometry(mesh, *geom_mats))
    return group


def _fan(face_start, faces, n):
    """Corner indices [k, 3] of faces that all have n corners, fanned from
    the first corner: (0,1,2), (0,2,3), ... per face, faces in order."""
    if not faces.size:
        return np.zeros((0, 3), np.int64)
    base = face_start[faces][:, None, None]
    fan = np.array([[0, j + 1, j + 2] for j in range(n - 2)], np.int64)[None]
    return (base + fan).reshape(-1, 3)


def _fan_polygons(face_start, counts, faces):
    """Polygon.Triangles (geometry/primitive/polygon.go:71-78) of polygons of
    any size, in face order."""
    if not faces.size:
        return np.zeros((0, 3), np.int64)
    ntri = counts[faces] - 2
    owner = np.repeat(np.arange(len(faces)), ntri)
    j = np.arange(int(ntri.sum())) - np.repeat(np.cumsum(ntri) - ntri, ntri)
    base = face_start[faces][owner]
    return np.stack([base, base + j + 1, base + j + 2], axis=1)
