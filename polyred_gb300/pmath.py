"""Host float32 math with the reference's evaluation order.

Matrix products, inverses and camera matrices go through the library's C
helpers (compiled with -ffp-contract=off), so a Python host builds the same
bits the Go renderer does (math/mat4.go, camera/*.go). Vector helpers that
need Go's math.FMA semantics use exact rational arithmetic.
"""
import ctypes as C
from fractions import Fraction

import numpy as np

from . import native

F32 = np.float32

# Another implementation of the six matrix functions below (same names and
# results), or None for the library's C helpers.
_backend = None


def set_backend(backend):
    """Route mat4_mul, mat4_inv, view_matrix, perspective_matrix,
    orthographic_matrix and shadow_camera through `backend` (a module or
    object with functions of those names), or back to the library with
    None. A process that must not load the library uses this to build
    scenes and frames with a CPU implementation of the same arithmetic."""
    global _backend
    _backend = backend


def _fp(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


def identity():
    return np.eye(4, dtype=np.float32).reshape(16)


def mat4_mul(a, b):
    """Mat4.MulM (math/mat4.go:201-220): a * b, row-major 16 floats."""
    if _backend is not None:
        return _backend.mat4_mul(a, b)
    lib = native.load()
    a, pa = _fp(a)
    b, pb = _fp(b)
    out, po = _fp(np.zeros(16, np.float32))
    native.check(lib.pr_mat4_mul(pa, pb, po))
    return out


def mat4_inv(m):
    if _backend is not None:
        return _backend.mat4_inv(m)
    lib = native.load()
    m, pm = _fp(m)
    out, po = _fp(np.zeros(16, np.float32))
    native.check(lib.pr_mat4_inv(pm, po))
    return out


def view_matrix(pos, target, up):
    """camera.ViewMatrix (camera/camera.go:42-53)."""
    if _backend is not None:
        return _backend.view_matrix(pos, target, up)
    lib = native.load()
    a, pa = _fp(pos)
    b, pb = _fp(target)
    c, pc = _fp(up)
    out, po = _fp(np.zeros(16, np.float32))
    native.check(lib.pr_view_matrix(pa, pb, pc, po))
    return out


def perspective_matrix(fov, aspect, near, far):
    if _backend is not None:
        return _backend.perspective_matrix(fov, aspect, near, far)
    lib = native.load()
    out, po = _fp(np.zeros(16, np.float32))
    native.check(lib.pr_perspective_matrix(float(F32(fov)), float(F32(aspect)), float(F32(near)), float(F32(far)), po))
    return out


def orthographic_matrix(left, right, bottom, top, near, far):
    if _backend is not None:
        return _backend.orthographic_matrix(left, right, bottom, top, near, far)
    lib = native.load()
    out, po = _fp(np.zeros(16, np.float32))
    vals = [float(F32(v)) for v in (left, right, bottom, top, near, far)]
    native.check(lib.pr_orthographic_matrix(*vals, po))
    return out


def shadow_camera(light_pos, center, cam_view, cam_proj):
    if _backend is not None:
        return _backend.shadow_camera(light_pos, center, cam_view, cam_proj)
    lib = native.load()
    a, pa = _fp(light_pos)
    b, pb = _fp(center)
    c, pc = _fp(cam_view)
    d, pd = _fp(cam_proj)
    v, pv = _fp(np.zeros(16, np.float32))
    p, pp = _fp(np.zeros(16, np.float32))
    native.check(lib.pr_shadow_camera(pa, pb, pc, pd, pv, pp))
    return v, p


def fma32(x, y, z):
    """float32(fma(float64(x), float64(y), float64(z))) — math/math.go:265-267."""
    exact = Fraction(float(x)) * Fraction(float(y)) + Fraction(float(z))
    return F32(float(exact))  # Fraction -> float64 rounds once, then float32


def vec3_unit(v):
    """Vec3.Unit (math/vec3.go:84-93) in float32 with FMA-through-float64 Dot."""
    x, y, z = (F32(c) for c in v)
    d = fma32(x, x, fma32(y, y, F32(z * z)))
    n = F32(1.0) / F32(np.sqrt(np.float64(d)))
    return np.array([x * n, y * n, z * n], np.float32)


def scale_matrix(sx, sy, sz):
    return np.array([sx, 0, 0, 0, 0, sy, 0, 0, 0, 0, sz, 0, 0, 0, 0, 1], np.float32)


def translate_matrix(tx, ty, tz):
    return np.array([1, 0, 0, tx, 0, 1, 0, ty, 0, 0, 1, tz, 0, 0, 0, 1], np.float32)
