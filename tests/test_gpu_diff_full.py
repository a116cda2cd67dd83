"""The adjoint at its stated size: the 1M-triangle sphere field over a
vertex-coloured ground grid at 1920x1080 (2048^2 shadow maps). GPU radiance
against the FP64 forward within 1e-5 relative; GPU gradients of the L2 loss
(target rendered with Kd + 0.1, light + (0.5, 0, 0), vertex colours +
N(0, 0.05)) against FP64 central differences (h = 1e-4) on 64 random
parameters within 1e-3 relative, with no absolute term."""
import numpy as np
import pytest

import oracle
from polyred_gb300 import diff, procedural
from test_gpu_diff import central_difference_picks, central_differences

pytestmark = pytest.mark.gpu

W, H = 1920, 1080


@pytest.fixture(scope="module")
def setup(device):
    import torch
    s, cam = procedural.diff_scene(width=W, height=H)
    r = diff.DiffRenderer(s, [diff.View(cam, W, H)], device=device, shadow_size=(2048, 2048))
    p = r.initial_params()
    g = torch.Generator(device="cpu").manual_seed(5)
    p["kd"] = (p["kd"] + 0.01 * torch.rand(p["kd"].shape, generator=g)).contiguous()
    p["ks"] = (p["ks"] + 0.01 * torch.rand(p["ks"].shape, generator=g)).contiguous()
    rad, gbuf = r.forward_raw(0, p)
    fd = r.frame(0, p["light_pos"].numpy(), p["light_intensity"].numpy(), p["ambient"].numpy())
    np_params = {k: v.detach().cpu().numpy().astype(np.float64) for k, v in p.items()}
    inp = oracle.DiffInputs(r.flat, gbuf.cpu().numpy(), np_params, fd.desc, oracle.normal_matrices(r.flat))
    assert r.flat.n_tris > 999_936
    return r, p, rad, gbuf, inp


def test_full_size_radiance_matches_fp64(setup):
    r, p, rad, gbuf, inp = setup
    got = rad.cpu().numpy().astype(np.float64)
    _, want = oracle.diff_forward64(inp)
    flags = gbuf.cpu().numpy()[..., 2].view(np.uint32)
    assert (flags & 1).sum() > 500_000 and (flags & 8).sum() > 10_000
    err = np.abs(got[..., :3] - want[..., :3])
    rel = err / np.maximum(np.abs(want[..., :3]), 1e-300)
    bad = ~(err <= 1e-5 * np.abs(want[..., :3]))
    assert not bad.any(), (int(bad.sum()), float(rel[bad].max()), float(np.abs(want[..., :3])[bad].min()))


def test_full_size_gradients_match_central_differences(setup):
    """Purely relative: |GPU - FD| <= 1e-3 |FD| for every one of the 64."""
    res = central_differences(setup, central_difference_picks(setup, seed=0x5EED0005))
    bad = [x for x in res if not abs(x[3] - x[2]) <= 1e-3 * abs(x[2])]
    worst = max(abs(x[3] - x[2]) / max(abs(x[2]), 1e-300) for x in res)
    assert not bad, (len(bad), worst, bad[:8])
