"""Differentiable shading on the GPU (pr_diff_forward / pr_diff_backward)
against the FP64 reference (oracle/adjoint.cpp) on the G-buffer the GPU
wrote: radiance within 1e-5 relative, gradients against the FP64 adjoint,
and against FP64 central finite differences (h = 1e-4) on 64 random
parameters within 1e-3 relative; the autograd contract; a short
inverse-rendering run."""
import numpy as np
import pytest

import oracle
from polyred_gb300 import diff, procedural, scene as sc

pytestmark = pytest.mark.gpu

W, H = 480, 270


@pytest.fixture(scope="module")
def setup(device):
    import torch
    s, cam = procedural.diff_scene(width=W, height=H, n_spheres=48, lon=32, lat=16, grid=24)
    r = diff.DiffRenderer(s, [diff.View(cam, W, H)], device=device, shadow_size=(512, 512))
    p = r.initial_params()
    g = torch.Generator(device="cpu").manual_seed(5)
    # perturb away from RGBA8-exact values so no parameter sits on a kink
    p["kd"] = (p["kd"] + 0.01 * torch.rand(p["kd"].shape, generator=g)).contiguous()
    p["ks"] = (p["ks"] + 0.01 * torch.rand(p["ks"].shape, generator=g)).contiguous()
    rad, gbuf = r.forward_raw(0, p)
    fd = r.frame(0, p["light_pos"].numpy(), p["light_intensity"].numpy(), p["ambient"].numpy())
    np_params = {k: v.detach().cpu().numpy().astype(np.float64) for k, v in p.items()}
    inp = oracle.DiffInputs(r.flat, gbuf.cpu().numpy(), np_params, fd.desc, oracle.normal_matrices(r.flat))
    return r, p, rad, gbuf, inp


def test_radiance_matches_fp64(setup):
    r, p, rad, gbuf, inp = setup
    got = rad.cpu().numpy().astype(np.float64)
    _, want = oracle.diff_forward64(inp)
    flags = gbuf.cpu().numpy()[..., 2].view(np.uint32)
    assert (flags & 1).sum() > 10000 and (flags & 8).sum() > 1000  # lit and vertex-coloured pixels
    err = np.abs(got[..., :3] - want[..., :3])
    assert (err <= 1e-5 * np.abs(want[..., :3]) + 1e-4).all(), float(err.max())


_TARGET = {}


def _loss_setup(setup):
    """The L2 loss against a target rendered with perturbed parameters: Kd
    + 0.1, light position + (0.5, 0, 0), vertex colours + N(0, 0.05).
    Returns (target, dL/d(radiance)); the upstream gradient is that of the
    FP64 loss the central differences differentiate, 2 (R64 - target) with
    R64 the FP64 radiance: from the GPU's float32 radiance instead, pixels
    whose radiance nearly equals the target would carry the float32
    rounding of R as a relative error of R - target."""
    import torch
    r, p, rad, gbuf, inp = setup
    if id(r) not in _TARGET:
        g = torch.Generator(device="cpu").manual_seed(0x5EED0005)
        q = {k: v.clone() for k, v in p.items()}
        q["kd"] = (q["kd"] + 0.1).contiguous()
        q["light_pos"] = (q["light_pos"] + torch.tensor([0.5, 0.0, 0.0])).contiguous()
        noise = torch.randn(q["vertex_color"].shape, generator=g) * 0.05
        q["vertex_color"] = (q["vertex_color"] + noise.cuda()).contiguous()
        target = r.forward_raw(0, q)[0].cpu().numpy()
        _, R64 = oracle.diff_forward64(inp)
        grad = np.zeros_like(R64)
        grad[..., :3] = 2 * (R64[..., :3] - target[..., :3])
        _TARGET[id(r)] = (target, grad)
    return _TARGET[id(r)]


def _gpu_grads(setup, grad):
    import torch
    r, p, rad, gbuf, inp = setup
    gt = torch.from_numpy(grad.astype(np.float32)).cuda()
    return {k: v.detach().cpu().numpy().astype(np.float64) for k, v in r.backward_raw(0, p, gbuf, gt).items()}


def test_gradients_match_fp64_adjoint(setup):
    r, p, rad, gbuf, inp = setup
    target, grad = _loss_setup(setup)
    gpu = _gpu_grads(setup, grad)
    ref = oracle.diff_backward64(inp, grad)
    for name in diff.PARAM_NAMES:
        a, b = gpu[name].reshape(-1), ref[name].reshape(-1)
        scale = np.abs(b).max()
        assert scale > 0, name
        assert np.allclose(a, b, rtol=1e-3, atol=1e-4 * scale), (name, float(np.abs(a - b).max()), float(scale))


def central_difference_picks(setup, seed=11):
    """64 random parameters: 16 vertex colours of material-less triangles, 16
    vertex normals of lit triangles, 8 kd and 8 ks entries, 10 shininesses,
    the point light's position (3), both light intensities and the ambient
    intensity."""
    r, p, rad, gbuf, inp = setup
    g = np.random.default_rng(seed)
    gb = gbuf.cpu().numpy()
    tri = gb[..., 0].reshape(-1).view(np.uint32)
    fl = gb[..., 2].reshape(-1).view(np.uint32)
    lit_tris = np.unique(tri[((fl & 1) != 0) & ((fl & 2) == 0)])
    unlit_tris = np.unique(tri[(fl & 8) != 0])
    picks = []
    for _ in range(16):
        picks.append(("vertex_color", int(g.choice(unlit_tris)), int(g.integers(0, 3)), int(g.integers(0, 3))))
        picks.append(("vertex_normal", int(g.choice(lit_tris)), int(g.integers(0, 3)), int(g.integers(0, 3))))
    nm = inp.param("kd").shape[0]
    for _ in range(8):
        picks.append(("kd", int(g.integers(0, nm)), int(g.integers(0, 3)), None))
        picks.append(("ks", int(g.integers(0, nm)), int(g.integers(0, 3)), None))
    for m in g.choice(nm, 10, replace=False):
        picks.append(("shininess", int(m), None, None))
    picks += [("light_pos", 0, k, None) for k in range(3)]
    picks += [("light_intensity", 0, None, None), ("light_intensity", 1, None, None), ("ambient", 0, None, None)]
    assert len(picks) == 64
    return picks


def central_differences(setup, picks, h=1e-4):
    """[(name, index, FP64 central difference with step h, GPU gradient,
    FD error estimate, float32 error scale)] for picks. The FD error
    estimate is the spread of the central differences with steps 2h and h/2
    around the one with h, plus their rounding (the loss's float64 ulp over
    the step: a contribution below it leaves the loss unchanged, so the
    difference reads 0); the float32 error scale is 2^-17 times a majorant
    of the gradient's terms (the FP64 adjoint in its absolute mode: every
    factor and sum of every pixel's contribution in magnitude, projections of
    the unit-vector derivatives included), which bounds the rounding of a
    float32 evaluation (about a hundred roundings per term, each within
    2^-24)."""
    r, p, rad, gbuf, inp = setup
    target, grad = _loss_setup(setup)
    gpu = _gpu_grads(setup, grad)
    mag = oracle.diff_backward64(inp, grad, absolute=True)
    res = []
    for name, a0, a1, a2 in picks:
        arr = inp.param(name)
        idx = (a0,) if a1 is None else ((a0, a1) if a2 is None else (a0, a1, a2))
        inp.s.only_tri = a0 if name.startswith("vertex") else -1
        inp.s.only_mat = a0 if name in ("kd", "ks", "shininess") else -1
        v0 = arr[idx]
        fd, lmax = {}, 0.0
        for step in (2 * h, h, h / 2):
            arr[idx] = v0 + step
            lp, _ = oracle.diff_forward64(inp, target, want_radiance=False)
            arr[idx] = v0 - step
            lm, _ = oracle.diff_forward64(inp, target, want_radiance=False)
            arr[idx] = v0
            fd[step] = (lp - lm) / (2 * step)
            lmax = max(lmax, abs(lp), abs(lm))
        e_fd = max(abs(fd[2 * h] - fd[h]), abs(fd[h / 2] - fd[h])) + 2.0 ** -50 * lmax / (h / 2)
        res.append((name, idx, fd[h], float(gpu[name][idx]), e_fd, 2.0 ** -17 * float(mag[name][idx])))
    inp.s.only_tri = inp.s.only_mat = -1
    return res


def test_gradients_match_central_differences(setup):
    """64 random parameters, FP64 central differences with h = 1e-4 of the
    FP64 loss (visibility fixed), against the GPU gradients: within 1e-3
    relative, plus the FD's own error estimate and the float32 error scale
    of the gradient (central_differences). Only gradients at the noise level
    of their own terms need those terms: vertex normals of triangles whose
    pixels already match the target to about 1e-6, whose gradients are
    1e-26 to 1e-15 (below the float64 resolution of a loss near 1e-13 over
    the step, so the central difference reads 0, or a derivative that
    vanishes exactly, the perturbation lying along the unit normal, where
    both adjoints return their rounding); at most a few of the 64 picks are
    such."""
    res = central_differences(setup, central_difference_picks(setup))
    bad = [x for x in res if not abs(x[3] - x[2]) <= 1e-3 * abs(x[2]) + x[4] + x[5]]
    assert not bad, bad[:6]
    floor_only = [x for x in res if not abs(x[3] - x[2]) <= 1e-3 * abs(x[2])]
    assert len(floor_only) <= 6, floor_only
    assert all(x[0] == "vertex_normal" for x in floor_only), floor_only


def test_autograd_contract(setup):
    import torch
    r, p, rad, gbuf, inp = setup
    q = {k: v.clone().requires_grad_(k in ("kd", "light_pos", "vertex_color")) for k, v in p.items()}
    out = diff.shade(q, r, 0)
    assert out.shape == (H, W, 4) and out.dtype == torch.float32
    assert torch.allclose(out, rad)
    loss = (out[..., :3] ** 2).sum()
    loss.backward()
    g4 = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    g4[..., :3] = 2 * out[..., :3].detach()
    ref = r.backward_raw(0, p, gbuf, g4)
    for k in ("kd", "light_pos", "vertex_color"):
        assert q[k].grad is not None
        assert torch.allclose(q[k].grad.cpu(), ref[k].cpu(), rtol=1e-5, atol=1e-6)
    for k in ("ks", "shininess", "vertex_normal"):
        assert q[k].grad is None


def test_inverse_render_reduces_loss(device):
    import torch
    s, cam = procedural.diff_scene(width=160, height=90, n_spheres=12, lon=16, lat=8, grid=8)
    cams = [sc.Perspective(position=(6 * np.cos(a), 2, 6 * np.sin(a)), target=(0, 0, 0), up=(0, 1, 0), fov=60,
                           aspect=160 / 90, near=0.1, far=100) for a in (0.0, 2.0)]
    r = diff.DiffRenderer(s, [diff.View(c, 160, 90) for c in cams], device=device, shadow_size=(256, 256))
    p0 = r.initial_params()
    targets = [r.forward_raw(v, p0)[0] for v in range(2)]
    p = {k: v.clone() for k, v in p0.items()}
    p["kd"] = (p["kd"] + 0.1).clamp(0, 1).contiguous().requires_grad_(True)
    p["light_intensity"] = (p["light_intensity"] * 1.3).contiguous().requires_grad_(True)
    losses = diff.inverse_render(r, targets, p, ("kd", "light_intensity"), steps=12, lr=0.01)
    assert losses[-1] < 0.5 * losses[0], losses
