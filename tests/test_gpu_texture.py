"""Image textures (pr_scene_desc.textures): Texture.Query at the
FragmentShader's level of detail in the shade kernel, with the mipmap the
library builds at upload, bit-exact against the oracle: mipmapped square,
mipmapped non-square non-power-of-two, and queryL0 (no mipmap) textures,
with shadows, across frames, and with MSAA."""
import numpy as np
import pytest

from helpers import Pair, assert_bitexact, options
from polyred_gb300 import _abi, batch as pb, native, procedural

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H", [(320, 200), (800, 500)])
def test_textured_scene_bitexact(device, W, H):
    s, cam = procedural.textured_scene(W, H)
    p = Pair(device, options(s, cam, W, H, shadow_map=True))
    for _ in range(2):
        gpu, cpu = p.frame()
        assert_bitexact(gpu, cpu)
    mats = np.unique(gpu["mat_id"])
    assert {0, 1, 2} <= set(mats.tolist())
    assert len(np.unique(gpu["rgba"].reshape(-1, 4), axis=0)) > 1000  # the images show


def test_textured_scene_msaa_bitexact(device):
    s, cam = procedural.textured_scene(240, 150)
    p = Pair(device, options(s, cam, 240, 150, shadow_map=True, msaa=2))
    gpu, cpu = p.frame()
    assert_bitexact(gpu, cpu)


def test_textures_rejected_in_batches(device):
    s, cam = procedural.textured_scene(64, 40)
    b = pb.Batch(0)
    with pytest.raises(native.RenderError) as ei:
        b.add_scene(s)
    assert ei.value.status == _abi.PR_ERR_UNSUPPORTED
    b.close()
