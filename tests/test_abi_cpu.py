"""C ABI checks that need no GPU: the library loads, exports every symbol
include/polyred_cuda.h declares, and its host math equals the oracle's."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from polyred_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "polyred_cuda.h")
TESTING_HEADER = os.path.join(ROOT, "include", "polyred_cuda_testing.h")
F = C.c_float


def declared_symbols(header=HEADER):
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pr_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "pr_render" in names and "pr_create" in names
    assert set(names) == {n for n, _, _ in _abi.ENTRY_POINTS}


def test_library_exports_every_declared_symbol(native_lib):
    for name in declared_symbols():
        assert hasattr(native_lib, name), name


def test_testing_header_declares_the_test_hooks(native_lib):
    names = declared_symbols(TESTING_HEADER)
    assert set(names) == {n for n, _, _ in _abi.TESTING_ENTRY_POINTS}
    assert not set(names) & set(declared_symbols())
    for name in names:
        assert hasattr(native_lib, name), name


def test_injected_allocation_failure_is_reported(native_lib):
    """The injection fails the n-th allocation without calling CUDA, so it
    runs without a GPU: pr_host_alloc reports PR_ERR_OOM with the call named,
    the count advances, and with the injection off the call goes to CUDA."""
    n0 = native_lib.pr_testing_alloc_count()
    assert native_lib.pr_testing_fail_alloc(-1) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_testing_fail_alloc(2) == _abi.PR_OK
    p = C.c_void_p()
    try:
        rc1 = native_lib.pr_host_alloc(64, C.byref(p))
        if rc1 == _abi.PR_OK:  # a CUDA host is present: the first allocation is real
            native_lib.pr_host_free(p)
        rc2 = native_lib.pr_host_alloc(64, C.byref(p))
        assert rc2 == _abi.PR_ERR_OOM
        assert b"cudaHostAlloc" in native_lib.pr_last_error()
        assert not p.value
    finally:
        native_lib.pr_testing_fail_alloc(0)
    assert native_lib.pr_testing_alloc_count() - n0 == 2


def test_abi_version(native_lib):
    assert native_lib.pr_abi_version() == _abi.ABI_VERSION
    assert native_lib.pr_error_string(_abi.PR_ERR_SINGULAR) == b"singular matrix"


def test_struct_layouts_match_the_header(tmp_path):
    """Compile a probe against include/polyred_cuda.h and compare every
    struct's size and field offsets with the ctypes mirror."""
    import subprocess
    structs = [_abi.pr_object, _abi.pr_material, _abi.pr_scene_desc, _abi.pr_light, _abi.pr_frame_desc,
               _abi.pr_outputs, _abi.pr_stats, _abi.pr_depth_map_desc, _abi.pr_diff_params,
               _abi.pr_diff_grads, _abi.pr_batch_view, _abi.pr_batch_stats, _abi.pr_obj_material,
               _abi.pr_obj_info]
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){"]
    for st in structs:
        n = st.__name__
        lines.append(f'printf("{n} %zu\\n", sizeof({n}));')
        for f, _ in st._fields_:
            lines.append(f'printf("{n}.{f} %zu\\n", offsetof({n}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for st in structs:
        n = st.__name__
        assert int(got[n]) == C.sizeof(st), n
        for f, _ in st._fields_:
            assert int(got[f"{n}.{f}"]) == getattr(st, f).offset, f"{n}.{f}"


def test_null_arguments_are_errors(native_lib):
    assert native_lib.pr_render(None, None, None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_destroy(None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_scene_upload(None, None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_view_matrix(None, None, None, None) == _abi.PR_ERR_INVALID_ARG
    assert b"NULL" in native_lib.pr_last_error()
    assert native_lib.pr_host_alloc(16, None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_host_free(None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_frame_submit(None, None, None, None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_sync(None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_device_alloc(None, 16, None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_device_free(None, None) == _abi.PR_ERR_INVALID_ARG
    assert native_lib.pr_device_read(None, None, 4, None) == _abi.PR_ERR_INVALID_ARG


def test_singular_inverse(native_lib):
    z = (F * 16)()
    o = (F * 16)()
    assert native_lib.pr_mat4_inv(z, o) == _abi.PR_ERR_SINGULAR


def _rand_mats(n, seed):
    g = np.random.default_rng(seed)
    return g.uniform(-3, 3, (n, 16)).astype(np.float32)


def test_host_matrix_math_matches_oracle(native_lib, oracle_lib):
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    for a, b in zip(_rand_mats(200, 1), _rand_mats(200, 2)):
        o1, o2 = np.zeros(16, np.float32), np.zeros(16, np.float32)
        native_lib.pr_mat4_mul(P(a), P(b), P(o1))
        oracle_lib.orc_mat4_mul(P(a), P(b), P(o2))
        assert np.array_equal(o1.view(np.uint32), o2.view(np.uint32))
        r1 = native_lib.pr_mat4_inv(P(a), P(o1))
        r2 = oracle_lib.orc_mat4_inv(P(a), P(o2))
        assert r1 == r2
        if r1 == 0:
            assert np.array_equal(o1.view(np.uint32), o2.view(np.uint32))


def test_camera_helpers_match_oracle(native_lib, oracle_lib):
    g = np.random.default_rng(3)
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    for _ in range(200):
        pos, tgt = g.uniform(-100, 100, 3).astype(np.float32), g.uniform(-100, 100, 3).astype(np.float32)
        up = np.array([0, 1, 0], np.float32)
        o1, o2 = np.zeros(16, np.float32), np.zeros(16, np.float32)
        native_lib.pr_view_matrix(P(pos), P(tgt), P(up), P(o1))
        oracle_lib.orc_view_matrix(P(pos), P(tgt), P(up), P(o2))
        assert np.array_equal(o1.view(np.uint32), o2.view(np.uint32))
        fov, asp, n, f = (float(np.float32(v)) for v in (g.uniform(20, 100), g.uniform(0.5, 3), 0.1, 100))
        native_lib.pr_perspective_matrix(fov, asp, n, f, P(o1))
        oracle_lib.orc_perspective_matrix(fov, asp, n, f, P(o2))
        assert np.array_equal(o1.view(np.uint32), o2.view(np.uint32))
        vals = [float(np.float32(v)) for v in g.uniform(-10, 10, 6)]
        native_lib.pr_orthographic_matrix(*vals, P(o1))
        oracle_lib.orc_ortho_matrix(*vals, P(o2))
        assert np.array_equal(o1.view(np.uint32), o2.view(np.uint32))


def test_shadow_camera_matches_oracle(native_lib, oracle_lib):
    from polyred_gb300 import procedural
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    s, cam = procedural.small_scene()
    v, p = cam.view_matrix(), cam.proj_matrix()
    for lp in ([4, 4, 2], [14, 18, 12], [-3, 7, 1]):
        lp = np.array(lp, np.float32)
        c = s.center()
        a1, b1, a2, b2 = (np.zeros(16, np.float32) for _ in range(4))
        assert native_lib.pr_shadow_camera(P(lp), P(c), P(v), P(p), P(a1), P(b1)) == 0
        assert oracle_lib.orc_shadow_camera(P(lp), P(c), P(v), P(p), P(a2), P(b2)) == 0
        assert np.array_equal(a1.view(np.uint32), a2.view(np.uint32))
        assert np.array_equal(b1.view(np.uint32), b2.view(np.uint32))


def test_create_without_gpu_reports_no_device(native_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    rc = native_lib.pr_create(0, C.byref(h))
    assert rc in (_abi.PR_ERR_NO_DEVICE, _abi.PR_ERR_CUDA)
    assert not h.value
