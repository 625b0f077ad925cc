"""Render parity: the sm_103a frame render against the CPU oracle."""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes
from barney_gb300.device import GpuScene
import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("layout", [N.GBV_LAYOUT_LINEAR, N.GBV_LAYOUT_BRICK_CORNERS])
def test_single_scatter_bit_exact(cuda, layout):
    """Single-scatter frames (the reference's default build) touch no
    transcendental on the device path, so the GPU frame equals the oracle's
    bit for bit, pass after pass."""
    import torch
    s = scenes.small_scene(dims=64, spp=4, width=128, height=96)
    g = GpuScene(s, layout=layout)
    o = oracle.Oracle(s)
    acc_g = g.render(spp=4)
    torch.cuda.synchronize()
    acc_o = o.render(spp=4)
    a = acc_g.cpu().numpy()
    np.testing.assert_array_equal(a.view(np.uint32), acc_o.view(np.uint32))
    # progressive accumulation continues exactly
    g.render(spp=3, accum=acc_g, accum_id_start=4)
    o.render(spp=3, accum=acc_o, accum_id_start=4)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(acc_g.cpu().numpy().view(np.uint32), acc_o.view(np.uint32))
