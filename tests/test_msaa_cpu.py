"""MSAA on the host side: the oracle's imageutil.Resize against a plain
restatement of internal/imageutil/resize.go, the frame descriptor's msaa
field and its limits, and the oracle's MSAA framebuffer sizes. No GPU."""
import ctypes as C

import numpy as np
import pytest

import oracle
from helpers import options, shadow_cams
from polyred_gb300 import _abi, procedural, render

F32 = np.float32


def _weights(dy, scale):
    """createWeights8(dy, 2, scale, linear) in float32 (resize.go:161-181)."""
    scale = F32(scale)
    n = 2 * int(max(np.ceil(scale), F32(1)))
    factor = min(F32(1) / scale, F32(1))
    coeffs, start = [], []
    for y in range(dy):
        interp = F32(scale * F32(F32(y) + F32(0.5))) - F32(0.5)
        s = int(interp) - n // 2 + 1
        interp = F32(interp - F32(s))
        row = []
        for i in range(n):
            x = abs(F32(F32(interp - F32(i)) * factor))
            k = F32(1) - x if x <= 1 else F32(0)
            row.append(int(F32(k * F32(256))))
        coeffs.append(row)
        start.append(s)
    return coeffs, start, n


def _resize_rgba(img, out_dx, out_dy, coeffs, start, n):
    """resizeRGBA: output (out_dy rows, out_dx cols) from input row x."""
    maxx = img.shape[1] - 1
    out = np.zeros((out_dy, out_dx, 4), np.uint8)
    for x in range(out_dx):
        row = img[x]
        for y in range(out_dy):
            acc = [0, 0, 0, 0]
            tot = 0
            for i in range(n):
                c = coeffs[y][i]
                if c == 0:
                    continue
                xi = start[y] + i
                xi = xi if 0 <= xi < maxx else (maxx if xi >= maxx else 0)
                for k in range(4):
                    acc[k] += c * int(row[xi][k])
                tot += c
            out[y, x] = [min(max(a // tot, 0), 255) for a in acc]
    return out


def go_resize(img, w, h):
    dy, dx = img.shape[:2]
    if (dx, dy) == (w, h):
        return img.copy()
    cx, sx, nx = _weights(w, F32(dx) / F32(w))
    temp = _resize_rgba(img, dy, w, cx, sx, nx)          # transposed: (w rows, dy cols)
    cy, sy, ny = _weights(h, F32(dy) / F32(h))
    return _resize_rgba(temp, w, h, cy, sy, ny)


@pytest.mark.parametrize("m,w,h", [(2, 9, 7), (3, 8, 5), (4, 6, 6), (5, 3, 4), (2, 1, 1), (16, 2, 3)])
def test_resize_matches_go_restatement(m, w, h):
    rng = np.random.default_rng(m * 100 + w)
    img = rng.integers(0, 256, (h * m, w * m, 4), dtype=np.uint8)
    img[: h * m // 3] = 255  # flat areas and hard edges
    want = go_resize(img, w, h)
    got = oracle.resize(img, w, h)
    assert np.array_equal(got, want)


def test_resize_identity_at_msaa_1():
    img = np.arange(5 * 7 * 4, dtype=np.uint8).reshape(5, 7, 4)
    assert np.array_equal(oracle.resize(img, 7, 5), img)


def test_frame_desc_layout_and_v1_size():
    assert _abi.pr_frame_desc.msaa.offset == _abi.PR_FRAME_DESC_SIZE_V1
    assert C.sizeof(_abi.pr_frame_desc) == _abi.PR_FRAME_DESC_SIZE_V1 + 8


def test_outputs_sizes():
    o = render.Outputs(8, 5, ("rgba", "tri_id", "nor"), msaa=3)
    assert o.arrays["rgba"].shape == (5, 8, 4)
    assert o.arrays["tri_id"].shape == (15, 24)
    assert o.arrays["nor"].shape == (15, 24, 4)


def test_oracle_msaa_frame():
    """The oracle at MSAA 2: the framebuffer fields are twice the image, the
    image is the resize of a framebuffer rendered at twice the size with the
    extent quirk (so not always the plain 2x render's resize)."""
    s, cam = procedural.small_scene(width=160, height=100)
    opts = options(s, cam, 160, 100, msaa=2)
    fd = render.FrameDesc(opts, shadow_cams(opts))
    out = render.Outputs(160, 100, ("rgba", "tri_id"), msaa=2)
    flat = render.FlatScene(s)  # owns the arrays the descriptor points to
    oracle.render(flat.desc(), fd.desc, out.desc, threads=4)
    assert out.arrays["rgba"].shape == (100, 160, 4) and out.arrays["tri_id"].shape == (200, 320)
    assert (out.arrays["tri_id"].view(np.uint32) != 0xFFFFFFFF).sum() > 1000
    assert out.arrays["rgba"][..., 3].max() > 0


def test_msaa_limits(native_lib):
    s, cam = procedural.small_scene(width=64, height=40)
    opts = options(s, cam, 64, 40, msaa=17)
    fd = render.FrameDesc(opts, {})
    assert native_lib.pr_render(None, C.byref(fd.desc), None) == _abi.PR_ERR_INVALID_ARG
