"""CPU oracle for the render path (TEST INFRASTRUCTURE).

A restatement of polyred's Go CPU renderer in C++ (oracle.cpp), loaded with
ctypes. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
use it, always as the reference to compare with; the product never imports it.
"""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "liboracle.so")
_lib = None


def build(force=False):
    srcs = [os.path.join(HERE, f) for f in ("oracle.cpp", "adjoint.cpp", "oracle.h", "gomath.h", "vecmath.h")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in srcs):
        subprocess.run(["sh", os.path.join(HERE, "build.sh")], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        from polyred_gb300 import _abi
        lib = C.CDLL(LIB)
        lib.orc_texture_build.restype = C.c_longlong
        lib.orc_texture_build.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p]
        lib.orc_texture_query.restype = C.c_int
        lib.orc_texture_query.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 6
        lib.orc_resize.restype = C.c_int
        lib.orc_resize.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        lib.orc_render.restype = C.c_int
        lib.orc_render.argtypes = [C.POINTER(_abi.pr_scene_desc), C.POINTER(_abi.pr_frame_desc),
                                   C.c_void_p, C.c_int, C.POINTER(_abi.pr_outputs), C.c_void_p]
        f = C.c_float
        lib.orc_perspective_matrix.argtypes = [f, f, f, f, C.c_void_p]
        lib.orc_ortho_matrix.argtypes = [f] * 6 + [C.c_void_p]
        lib.orc_fma32.restype = f
        lib.orc_fma32.argtypes = [f, f, f]
        lib.orc_go_pow.restype = C.c_double
        lib.orc_go_pow.argtypes = [C.c_double, C.c_double]
        lib.orc_go_atan.restype = C.c_double
        lib.orc_go_atan.argtypes = [C.c_double]
        lib.orc_go_f2i.restype = C.c_int64
        lib.orc_go_f2i.argtypes = [f]
        lib.orc_go_f2u8.restype = C.c_uint8
        lib.orc_go_f2u8.argtypes = [f]
        lib.orc_from_linear_srgb.restype = f
        lib.orc_from_linear_srgb.argtypes = [f]
        lib.orc_mat4_inv.restype = C.c_int
        lib.orc_shadow_camera.restype = C.c_int
        lib.orc_aabb_intersect.restype = C.c_int
        lib.orc_aabb_contains.restype = C.c_int
        lib.orc_tri_is_valid.restype = C.c_int
        _lib = lib
    return _lib


def render(scene_desc, frame_desc, outputs_desc, shadow_state=None, threads=1):
    """One Render() of the reference in single-worker order."""
    lib = load()
    ptr = None
    if shadow_state is not None:
        # the oracle reads and writes n_lights maps of the frame's shadow size
        f = frame_desc
        m = f.msaa if f.msaa > 1 else 1
        sw = f.shadow_width if f.shadow_width > 0 else f.width * m
        sh = f.shadow_height if f.shadow_height > 0 else f.height * m
        need = int(f.n_lights) * sw * sh
        if shadow_state.dtype.itemsize != 4 or not shadow_state.flags.c_contiguous or shadow_state.size < need:
            raise ValueError(f"shadow_state needs {need} contiguous float32 values, has {shadow_state.size}")
        ptr = shadow_state.ctypes.data
    rc = lib.orc_render(C.byref(scene_desc), C.byref(frame_desc), ptr, int(threads), C.byref(outputs_desc), None)
    if rc != 0:
        raise RuntimeError(f"oracle render failed: {rc}")


# ---- FP64 differentiable shading (adjoint.cpp) ----------------------------

class orc_diff_in(C.Structure):
    _fields_ = [
        ("W", C.c_int32), ("H", C.c_int32),
        ("gbuf", C.c_void_p),
        ("n_tris", C.c_uint32), ("n_objects", C.c_uint32),
        ("vcol", C.c_void_p), ("vnor", C.c_void_p),
        ("obj_first", C.c_void_p), ("obj_normal", C.c_void_p),
        ("n_mats", C.c_int32), ("n_lights", C.c_int32),
        ("kd", C.c_void_p), ("ks", C.c_void_p), ("shin", C.c_void_p), ("tex", C.c_void_p),
        ("ltype", C.c_void_p), ("lpos", C.c_void_p), ("ldir", C.c_void_p), ("lint", C.c_void_p),
        ("lcol", C.c_void_p),
        ("n_amb", C.c_int32), ("only_tri", C.c_int32),
        ("amb", C.c_void_p),
        ("cam", C.c_double * 3), ("bg", C.c_double * 4),
        ("only_mat", C.c_int32), ("flags", C.c_int32),
    ]


class orc_diff_out(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("vcol", "vnor", "kd", "ks", "shin", "lpos", "lint", "amb")]


def normal_matrices(flat):
    """Per-object (Model^-1)^T as the reference's Mat4.Inv / T compute them."""
    import numpy as np
    lib = load()
    out = np.zeros((max(flat.n_objects, 1), 16), np.float32)
    for o in range(flat.n_objects):
        m = np.array(flat.objects[o].model[:], np.float32)
        inv = np.zeros(16, np.float32)
        if lib.orc_mat4_inv(m.ctypes.data, inv.ctypes.data) != 0:
            raise ValueError(f"object {o}: singular model matrix")
        out[o] = inv.reshape(4, 4).T.reshape(16)
    return out


class DiffInputs:
    """orc_diff_in over numpy arrays (parameters in float64) it keeps alive."""

    def __init__(self, flat, gbuf, params, frame, normal_mats, only_tri=-1, only_mat=-1):
        import numpy as np
        f = frame
        H, W = int(f.height), int(f.width)
        self.a = {}
        k = self.a
        k["gbuf"] = np.ascontiguousarray(gbuf, np.float32).reshape(H * W, 16)
        for name in ("vertex_color", "vertex_normal", "kd", "ks", "shininess", "light_pos", "light_intensity",
                     "ambient"):
            k[name] = np.ascontiguousarray(params[name], np.float64)
        first = np.array([flat.objects[o].first_tri for o in range(flat.n_objects)], np.uint32)
        k["first"] = first
        k["nmat"] = np.ascontiguousarray(normal_mats, np.float32)
        k["tex"] = np.array([list(flat.materials[m].texture) for m in range(flat.n_materials)] or [[0] * 4], np.uint8)
        nl = int(f.n_lights)
        k["ltype"] = np.array([f.lights[l].type for l in range(nl)] or [0], np.int32)
        k["ldir"] = np.array([list(f.lights[l].dir) for l in range(nl)] or [[0] * 3], np.float32)
        k["lcol"] = np.array([list(f.lights[l].color) for l in range(nl)] or [[0] * 4], np.uint8)
        s = orc_diff_in()
        s.W, s.H = W, H
        s.gbuf = k["gbuf"].ctypes.data
        s.n_tris, s.n_objects = flat.n_tris, flat.n_objects
        s.vcol, s.vnor = k["vertex_color"].ctypes.data, k["vertex_normal"].ctypes.data
        s.obj_first, s.obj_normal = first.ctypes.data, k["nmat"].ctypes.data
        s.n_mats, s.n_lights = flat.n_materials, nl
        s.kd, s.ks, s.shin, s.tex = (k["kd"].ctypes.data, k["ks"].ctypes.data, k["shininess"].ctypes.data,
                                     k["tex"].ctypes.data)
        s.ltype, s.lpos, s.ldir = k["ltype"].ctypes.data, k["light_pos"].ctypes.data, k["ldir"].ctypes.data
        s.lint, s.lcol = k["light_intensity"].ctypes.data, k["lcol"].ctypes.data
        s.n_amb = int(f.n_ambient)
        s.amb = k["ambient"].ctypes.data
        s.cam[:] = [float(c) for c in f.cam_pos]
        s.bg[:] = [float(c) for c in f.background]
        s.only_tri, s.only_mat = only_tri, only_mat
        self.s = s

    def param(self, name):
        """The float64 parameter array (edit in place for finite differences)."""
        return self.a[name]


def diff_forward64(inp, target=None, want_radiance=True):
    """(loss, radiance[H, W, 4]) in float64."""
    import numpy as np
    lib = load()
    lib.orc_diff_forward64.restype = C.c_double
    lib.orc_diff_forward64.argtypes = [C.POINTER(orc_diff_in), C.c_void_p, C.c_void_p]
    rad = np.zeros((inp.s.H, inp.s.W, 4), np.float64) if want_radiance else None
    tgt = None if target is None else np.ascontiguousarray(target, np.float32)
    loss = lib.orc_diff_forward64(C.byref(inp.s), None if rad is None else rad.ctypes.data,
                                  None if tgt is None else tgt.ctypes.data)
    return loss, rad


def diff_backward64(inp, grad, absolute=False):
    """Gradients of sum(grad * radiance) in float64, shaped like the
    parameters; with absolute=True, for each gradient a majorant of its
    terms instead (every factor and sum of every pixel's contribution taken
    in magnitude: the scale of the rounding error of a float32 evaluation)."""
    import numpy as np
    lib = load()
    lib.orc_diff_backward64.restype = None
    lib.orc_diff_backward64.argtypes = [C.POINTER(orc_diff_in), C.c_void_p, C.POINTER(orc_diff_out)]
    g = np.ascontiguousarray(grad, np.float64)
    names = {"vcol": "vertex_color", "vnor": "vertex_normal", "kd": "kd", "ks": "ks", "shin": "shininess",
             "lpos": "light_pos", "lint": "light_intensity", "amb": "ambient"}
    res = {v: np.zeros_like(inp.a[v]) for v in names.values()}
    o = orc_diff_out()
    for k, v in names.items():
        setattr(o, k, res[v].ctypes.data)
    inp.s.flags = 1 if absolute else 0
    try:
        lib.orc_diff_backward64(C.byref(inp.s), g.ctypes.data, C.byref(o))
    finally:
        inp.s.flags = 0
    return res


def resize(img, width, height):
    """imageutil.Resize of an (H, W, 4) uint8 image to (height, width, 4)."""
    import numpy as np
    img = np.ascontiguousarray(img, np.uint8)
    out = np.zeros((height, width, 4), np.uint8)
    rc = load().orc_resize(img.ctypes.data, img.shape[1], img.shape[0], width, height, out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"orc_resize failed: {rc}")
    return out
