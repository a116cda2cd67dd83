"""The AO march's per-direction set-up on the host (pr_debug_ao_dirs, no
device): the 8 directions of material/ao.go:28 (float32 angle stepped by
Pi/4, float32 Cos/Sin), which of them may use the device's tap offset table,
and their tiny components."""
import ctypes as C
import math

import numpy as np
import pytest

F = np.float32


def _dirs(lib, W, H):
    cosv, sinv = (C.c_float * 8)(), (C.c_float * 8)()
    fast, tiny = (C.c_int8 * 8)(), (C.c_int8 * 8)()
    n = lib.pr_debug_ao_dirs(W, H, cosv, sinv, fast, tiny)
    return n, np.array(cosv, F), np.array(sinv, F), list(fast), list(tiny)


def test_directions_follow_the_reference_loop(native_lib):
    n, c, s, *_ = _dirs(native_lib, 64, 48)
    assert n == 8
    a = F(0)
    for k in range(8):
        assert c[k] == F(math.cos(float(a))) and s[k] == F(math.sin(float(a))), k
        a = F(a + F(math.pi / 4))
    assert not a < F(2 * math.pi - 1e-4)


@pytest.mark.parametrize("W,H", [(1, 1), (64, 48), (1920, 1080), (3840, 2160), (8000, 3)])
def test_table_directions_and_tiny_components(native_lib, W, H):
    n, c, s, fast, tiny = _dirs(native_lib, W, H)
    # cos(float32(Pi/2)) and sin(float32(Pi)) are tiny negatives; cos(float32(3Pi/2)) is a tiny positive
    assert tiny == [0, 0, 1, 0, 2, 0, 0, 0]
    # the table needs every regular component a = RN(c t), t < 100, to be an
    # integer or more than half an ulp of the largest coordinate below the next one
    E = 0
    while (2 << E) <= max(W, H) + 100:
        E += 1
    h = 2.0 ** (E - 24)
    t = np.arange(1, 100, dtype=F)
    for k in range(8):
        ok = True
        for a, comp in enumerate((c[k], s[k])):
            if tiny[k] == a + 1:
                continue
            at = (comp * t).astype(F).astype(np.float64)
            frac = np.ceil(at) - at
            ok &= bool(np.all((at == np.floor(at)) | (frac > h)))
        assert fast[k] == int(ok), k
    assert fast == [1] * 8


def test_bad_arguments(native_lib):
    from polyred_gb300 import _abi
    z = (C.c_int8 * 8)()
    f = (C.c_float * 8)()
    assert native_lib.pr_debug_ao_dirs(0, 5, f, f, z, z) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_debug_ao_dirs(5, 5, None, f, z, z) == _abi.PR_ERR_INVALID_ARG
