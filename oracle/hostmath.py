"""The oracle's float32 host math behind polyred_gb300.pmath's interface
(TEST INFRASTRUCTURE).

pmath computes camera, model and shadow-camera matrices through the product
library's C helpers. A process that must not map the product library (the
CPU baseline that times the oracle as the reference renderer) routes pmath
through these functions instead, with `pmath.set_backend(oracle.hostmath)`.
Each follows the same reference code as its product twin:

  mat4_mul            Mat4.MulM        math/mat4.go:201-222
  mat4_inv            Mat4.Inv         math/mat4.go:259-283
  view_matrix         ViewMatrix       camera/camera.go:42-53
  perspective_matrix  ProjMatrix       camera/perspective.go:100-111
  orthographic_matrix ProjMatrix       camera/orthographic.go:106-119
  shadow_camera       initShadowMaps   render/shadow.go:41-85

tests/test_abi_cpu.py checks both implementations bit-equal.
"""
import ctypes as C

import numpy as np

from . import load

F32 = np.float32


def _fp(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data


def _singular(what):
    from polyred_gb300 import _abi, native
    return native.RenderError(_abi.PR_ERR_SINGULAR, f"{what}: singular matrix")


def mat4_mul(a, b):
    lib = load()
    a, pa = _fp(a)
    b, pb = _fp(b)
    out = np.zeros(16, np.float32)
    lib.orc_mat4_mul(C.c_void_p(pa), C.c_void_p(pb), C.c_void_p(out.ctypes.data))
    return out


def mat4_inv(m):
    lib = load()
    m, pm = _fp(m)
    out = np.zeros(16, np.float32)
    if lib.orc_mat4_inv(C.c_void_p(pm), C.c_void_p(out.ctypes.data)) != 0:
        raise _singular("mat4_inv")
    return out


def view_matrix(pos, target, up):
    lib = load()
    a, pa = _fp(pos)
    b, pb = _fp(target)
    c, pc = _fp(up)
    out = np.zeros(16, np.float32)
    lib.orc_view_matrix(C.c_void_p(pa), C.c_void_p(pb), C.c_void_p(pc), C.c_void_p(out.ctypes.data))
    return out


def perspective_matrix(fov, aspect, near, far):
    lib = load()
    out = np.zeros(16, np.float32)
    lib.orc_perspective_matrix(float(F32(fov)), float(F32(aspect)), float(F32(near)), float(F32(far)),
                               out.ctypes.data)
    return out


def orthographic_matrix(left, right, bottom, top, near, far):
    lib = load()
    out = np.zeros(16, np.float32)
    vals = [float(F32(v)) for v in (left, right, bottom, top, near, far)]
    lib.orc_ortho_matrix(*vals, out.ctypes.data)
    return out


def shadow_camera(light_pos, center, cam_view, cam_proj):
    lib = load()
    a, pa = _fp(light_pos)
    b, pb = _fp(center)
    c, pc = _fp(cam_view)
    d, pd = _fp(cam_proj)
    v = np.zeros(16, np.float32)
    p = np.zeros(16, np.float32)
    if lib.orc_shadow_camera(*(C.c_void_p(x) for x in (pa, pb, pc, pd, v.ctypes.data, p.ctypes.data))) != 0:
        raise _singular("shadow_camera")
    return v, p
