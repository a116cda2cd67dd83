"""The C ABI from a plain C program (tests/c/pr_c_host.c, compiled here with
gcc against include/polyred_cuda.h and libpolyred_cuda.so): its values
equal the Python host's, and with a GPU it renders a frame."""
import os
import subprocess

import numpy as np
import pytest

from polyred_gb300 import _abi, imageload, native, pmath

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def c_host(native_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("c") / "pr_c_host")
    libdir = os.path.dirname(native.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "c", "pr_c_host.c"), "-L", libdir, "-lpolyred_cuda", "-Wl,-rpath," + libdir,
                    "-o", exe], check=True)
    return exe


def _run(exe, *args):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=120)
    lines = dict(l.split(" ", 1) for l in r.stdout.splitlines())
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fail" not in lines, lines.get("fail")
    return lines


def _bits(m):
    return " ".join("%08x" % v for v in np.asarray(m, np.float32).view(np.uint32))


def test_c_host_matches_python_host(c_host):
    out = _run(c_host)
    assert out["abi"] == f"{_abi.ABI_VERSION} {_abi.ABI_VERSION}"
    view = pmath.view_matrix([0, 1.5, 4], [0, 0, 0], [0, 1, 0])
    proj = pmath.perspective_matrix(45.0, 1.6, 0.1, 100.0)
    pv = pmath.mat4_mul(proj, view)
    assert out["view"] == _bits(view) and out["proj"] == _bits(proj) and out["pv"] == _bits(pv)
    assert out["inv"] == _bits(pmath.mat4_inv(pv))
    assert int(out["singular"]) == _abi.PR_ERR_SINGULAR
    # 3 vertices (the third with w = 2), 2 faces, 1 object; no vt on face 2;
    # y of vertex 3 = 1 / 2; the relative index -1 is vertex 2 (0-based)
    assert out["obj"] == f"3 2 1 {_abi.PR_OBJ_NO_INDEX} 3f000000 2"
    assert out["obj_error"] == f"{_abi.PR_ERR_INVALID_ARG} vertex has less than 3 vertices in 'v' line: [1 2] in line:1"
    t = imageload.srgb_decode_table()
    assert out["srgb"] == f"{t[64]} {t[128]} {t[200]}"
    assert out["unfilter"] == "10 20 30 11 21 31 15 25 35 16 26 36"  # Sub then Up, 3 bytes per pixel
    assert int(out["create"]) in (_abi.PR_OK, _abi.PR_ERR_NO_DEVICE)


@pytest.mark.gpu
def test_c_host_renders(c_host):
    """A 64x64 frame of one triangle, as the oracle renders it: 722 pixels
    covered and lit."""
    out = _run(c_host, "--render")
    assert int(out["create"]) == _abi.PR_OK
    assert out["render"] == "covered 722 lit 722"
