"""The FP64 adjoint of the differentiable shading model (oracle/adjoint.cpp)
against FP64 central finite differences, on a synthetic differentiation
G-buffer: pixels of every kind (smooth and flat material pixels, constant
texture pixels, material-less pixels, background), random parameters and
lights. This pins the reference adjoint the GPU gradients are checked
against; the GPU side is tested in test_gpu_diff.py."""
import numpy as np
import pytest

import oracle
from polyred_gb300 import _abi, procedural, render, scene as sc


def _setup(seed=3, W=24, H=16):
    g = np.random.default_rng(seed)
    s, cam = procedural.small_scene(W, H)
    kd = sc.color_from_value(0.3, 0.6, 0.5, 1.0)
    flat_mat = sc.BlinnPhong(diffuse=kd, specular=kd, shininess=12, flat_shading=True)
    s.add(sc.Geometry(procedural.uv_sphere(8, 6, 0.5), flat_mat).translate(1.5, 0, 0))
    s.add(sc.Directional(direction=(-1, -2, -0.5), intensity=0.7))
    s.add(sc.Ambient(intensity=0.05))
    flat = render.FlatScene(s)
    opts = dict(width=W, height=H, camera=cam, scene=s, perspective=True, shadow_map=False, gamma=False,
                background=(10, 20, 30, 255), shadow_size=None)
    fd = render.FrameDesc(opts, {})
    nt = flat.n_tris
    gb = np.zeros((H * W, 16), np.float32)
    kinds = g.integers(0, 5, H * W)
    first_flat = flat.objects[flat.n_objects - 1].first_tri
    for i, k in enumerate(kinds):
        b = g.dirichlet([1, 1, 1]).astype(np.float32)
        if k == 0:  # background
            gb[i, 0] = np.uint32(0xFFFFFFFF).view(np.float32)
            continue
        if k == 1:  # material-less (ground plane triangles carry MaterialID -1)
            t = int(g.integers(0, 2)) + flat.objects[1].first_tri
            m, fl = -1, _abi.DGB_UNLIT
        elif k == 2:  # smooth material pixel (the big sphere)
            t, m, fl = int(g.integers(0, flat.objects[0].n_tris)), 0, _abi.DGB_LIT
        elif k == 3:  # flat material pixel
            t, m, fl = int(g.integers(first_flat, nt)), flat.n_materials - 1, _abi.DGB_LIT | _abi.DGB_FLAT
        else:  # constant texture pixel
            t, m, fl = int(g.integers(0, flat.objects[0].n_tris)), 0, _abi.DGB_CONST
        gb[i, 0] = np.uint32(t).view(np.float32)
        gb[i, 1] = np.int32(m).view(np.float32)
        gb[i, 2] = np.uint32(fl).view(np.float32)
        gb[i, 3] = g.uniform(0.25, 1.0)
        gb[i, 4:7] = b
        gb[i, 7] = 255
        gb[i, 8:11] = g.uniform(-1, 1, 3)
        gb[i, 11] = 1
        fn = g.normal(size=3)
        gb[i, 12:15] = fn / np.linalg.norm(fn)
    src, env = s.lights()
    params = {
        "vertex_color": g.uniform(0, 1, (nt, 3, 4)),
        "vertex_normal": np.concatenate([g.normal(size=(nt, 3, 3)), np.zeros((nt, 3, 1))], -1),
        "kd": g.uniform(0.2, 0.8, (flat.n_materials, 3)),
        "ks": g.uniform(0.2, 0.8, (flat.n_materials, 3)),
        "shininess": g.uniform(4, 40, flat.n_materials),
        "light_pos": np.array([[float(c) for c in l.position] for l in src]),
        "light_intensity": g.uniform(0.5, 2.0, len(src)),
        "ambient": g.uniform(0.05, 0.2, len(env)),
    }
    inp = oracle.DiffInputs(flat, gb, params, fd.desc, oracle.normal_matrices(flat))
    return inp, g


def test_fp64_adjoint_matches_central_differences():
    inp, g = _setup()
    _, R = oracle.diff_forward64(inp)
    target = (R + g.normal(0, 5, R.shape)).astype(np.float32)
    loss0, R = oracle.diff_forward64(inp, target)
    grad = np.zeros_like(R)
    grad[..., :3] = 2 * (R[..., :3] - target[..., :3])
    adj = oracle.diff_backward64(inp, grad)
    checked = 0
    for name in ("vertex_color", "vertex_normal", "kd", "ks", "shininess", "light_pos", "light_intensity",
                 "ambient"):
        a = inp.param(name).reshape(-1)
        ga = adj[name].reshape(-1)
        idx = np.flatnonzero(np.abs(ga) > 1e-6 * (np.abs(ga).max() + 1e-30))
        if name == "vertex_normal":
            idx = idx[(idx % 4) != 3]
        assert len(idx) > 0, name
        for j in g.choice(idx, min(6, len(idx)), replace=False):
            h = 1e-6 * max(1.0, abs(a[j]))
            a0 = a[j]
            a[j] = a0 + h
            lp, _ = oracle.diff_forward64(inp, target, want_radiance=False)
            a[j] = a0 - h
            lm, _ = oracle.diff_forward64(inp, target, want_radiance=False)
            a[j] = a0
            fd = (lp - lm) / (2 * h)
            assert fd == pytest.approx(ga[j], rel=1e-4, abs=1e-6 * abs(loss0)), (name, j, fd, ga[j])
            checked += 1
    assert checked >= 25
