"""The reference arm of bench.py (the oracle timed as the reference
renderer) builds its scene and frame without the product library, and the
oracle's host math it uses gives the same bits as the library's."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_maps_only_the_oracle():
    code = ("import bench, oracle; f = bench.oracle_frame(1); oracle.load(); "
            "print(';'.join(bench.mapped_libraries()))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    libs = r.stdout.strip().splitlines()[-1].split(";")
    assert libs == ["oracle/build/liboracle.so"], libs


def _frame_bytes(scene, cam, opts_extra):
    from polyred_gb300 import render
    import bench
    opts = dict(width=640, height=360, camera=cam, scene=scene, perspective=True, shadow_map=True, gamma=True,
                background=(0, 0, 0, 0), shadow_size=(512, 512), directional_shadows=True)
    opts.update(opts_extra)
    flat = render.FlatScene(scene)
    fd = render.FrameDesc(opts, bench.shadow_cams(opts))
    objs = bytes(C.string_at(C.addressof(flat.objects), C.sizeof(flat.objects)))
    lights = bytes(C.string_at(C.addressof(fd.lights), C.sizeof(fd.lights)))
    # the frame descriptor holds pointers, which differ between builds:
    # compare its matrices and camera position
    return objs, lights, bytes(fd.desc.view), bytes(fd.desc.proj), bytes(fd.desc.cam_pos)


def test_hostmath_backends_give_identical_descriptors(native_lib, oracle_lib):
    from oracle import hostmath
    from polyred_gb300 import pmath, procedural
    for make in (procedural.small_scene, lambda: procedural.sphere_field(width=640, height=360)):
        pmath.set_backend(None)
        s1, c1 = make()
        a = _frame_bytes(s1, c1, {})
        pmath.set_backend(hostmath)
        try:
            s2, c2 = make()
            b = _frame_bytes(s2, c2, {})
        finally:
            pmath.set_backend(None)
        assert a == b


def test_hostmath_matches_library_on_random_inputs(native_lib, oracle_lib):
    from oracle import hostmath
    from polyred_gb300 import pmath
    g = np.random.default_rng(11)
    same = lambda x, y: np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))
    for _ in range(100):
        a, b = g.uniform(-4, 4, (2, 16)).astype(np.float32)
        assert same(pmath.mat4_mul(a, b), hostmath.mat4_mul(a, b))
        assert same(pmath.mat4_inv(a), hostmath.mat4_inv(a))
        pos, tgt = g.uniform(-50, 50, (2, 3)).astype(np.float32)
        up = np.array([0, 1, 0], np.float32)
        assert same(pmath.view_matrix(pos, tgt, up), hostmath.view_matrix(pos, tgt, up))
        fov, asp = g.uniform(20, 100), g.uniform(0.5, 3)
        assert same(pmath.perspective_matrix(fov, asp, 0.1, 100), hostmath.perspective_matrix(fov, asp, 0.1, 100))
        lrbtnf = g.uniform(-10, 10, 6)
        assert same(pmath.orthographic_matrix(*lrbtnf), hostmath.orthographic_matrix(*lrbtnf))
        cv = pmath.view_matrix(pos, tgt, up)
        cp = pmath.perspective_matrix(fov, asp, 0.1, 100)
        lp = g.uniform(-20, 20, 3).astype(np.float32)
        v1, p1 = pmath.shadow_camera(lp, tgt, cv, cp)
        v2, p2 = hostmath.shadow_camera(lp, tgt, cv, cp)
        assert same(v1, v2) and same(p1, p2)


def test_bench_reads_the_committed_ao_profile():
    """The bench's roofline line takes the AO kernel's DRAM traffic and
    instruction count from its committed ncu summary: both parse, and the
    summary's issue-rate arithmetic matches its own figures."""
    import re
    import bench
    traffic, inst = bench.ncu_traffic(), bench.ncu_instructions()
    assert traffic is not None and 1e6 < traffic < 1e9, traffic
    assert inst is not None and 1e7 < inst < 1e10, inst
    text = open(os.path.join(ROOT, "profiles", "ao_kernel_sphere_field_1080p.txt")).read()
    dur = float(re.search(r"^duration_us: ([0-9.]+)", text, re.M).group(1))
    stated = float(re.search(r"fraction of its own time: .* = ([0-9.]+)\.", text).group(1))
    assert abs(inst / (152 * 4 * 2.07e9 * dur * 1e-6) - stated) < 0.01, (inst, dur, stated)
