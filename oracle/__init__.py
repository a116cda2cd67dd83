"""CPU oracle for the render path (TEST INFRASTRUCTURE).

A restatement of polyred's Go CPU renderer in C++ (oracle.cpp), loaded with
ctypes. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
use it, always as the checker; the product never imports it.
"""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "liboracle.so")
_lib = None


def build(force=False):
    srcs = [os.path.join(HERE, f) for f in ("oracle.cpp", "oracle.h", "gomath.h", "vecmath.h")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in srcs):
        subprocess.run(["sh", os.path.join(HERE, "build.sh")], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        from polyred_gb300 import _abi
        lib = C.CDLL(LIB)
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
    ptr = None if shadow_state is None else shadow_state.ctypes.data
    rc = lib.orc_render(C.byref(scene_desc), C.byref(frame_desc), ptr, int(threads), C.byref(outputs_desc), None)
    if rc != 0:
        raise RuntimeError(f"oracle render failed: {rc}")
