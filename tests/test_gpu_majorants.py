"""Macrocell ranges and majorants on the GPU against the oracle: bit-exact."""
import numpy as np
import pytest

from barney_gb300 import scenes
from barney_gb300 import _native as N
from barney_gb300.device import GpuScene
import oracle

pytestmark = pytest.mark.gpu


def check(scene):
    import torch
    g = GpuScene(scene, layout=N.GBV_LAYOUT_LINEAR)
    torch.cuda.synchronize()
    o = oracle.Oracle(scene)
    assert g.mc == o.mc_dims()
    r_o = o.mc_ranges()
    r_g = g.ranges.cpu().numpy().reshape(-1, 2)[: r_o.shape[0]]
    np.testing.assert_array_equal(r_g, r_o)
    m_o = o.majorants_of(r_o)
    m_g = g.majorants.cpu().numpy()[: m_o.shape[0]]
    np.testing.assert_array_equal(m_g.view(np.uint32), m_o.view(np.uint32))
    return g, m_o


def test_small_8cubed_macrocells(cuda):
    check(scenes.small_scene(dims=64))


def test_frame_16cubed_macrocells(cuda):
    # the full 512^3 frame volume with 16^3-voxel macrocells (32^3 cells)
    s = scenes.frame_scene(dims=512, width=64, height=64, spp=1, with_env=False)
    g, m = check(s)
    assert g.mc == (32, 32, 32)
    assert (m > 0).mean() > 0.05


@pytest.mark.parametrize("dims,cpm", [((37, 20, 9), 8), ((2, 2, 2), 8), ((17, 33, 65), 16), ((9, 9, 9), 4)])
def test_ragged_grids(cuda, dims, cpm):
    vol = scenes.blob_volume(dims, 4, seed=11)
    s = scenes.Scene(scalars=vol, tf=scenes.tf_two_peaks(64), cells_per_mc=cpm, base_density=3.0)
    check(s)


def test_constant_volume_and_step_tf(cuda):
    # known answers: a constant volume gives one majorant everywhere; a step
    # TF gives baseDensity*max over the step inside each range
    vol = np.full((24, 24, 24), 0.42, np.float32)
    tf = np.zeros((8, 4), np.float32)
    tf[4:, 3] = 1.0
    s = scenes.Scene(scalars=vol, tf=tf, cells_per_mc=8, base_density=5.0)
    g, m = check(s)
    assert np.all(m == m[0])
    vol2 = vol.copy()
    vol2[3, 3, 3] = 0.9  # one hot voxel: only the macrocells whose footprint holds it see the step
    s2 = scenes.Scene(scalars=vol2, tf=tf, cells_per_mc=8, base_density=5.0)
    g2, m2 = check(s2)
    assert (m2 == np.float32(5.0)).sum() == 1


def test_values_outside_domain(cuda):
    vol = scenes.blob_volume((20, 20, 20), 4, seed=3) * 3.0 - 1.0
    s = scenes.Scene(scalars=vol.astype(np.float32), tf=scenes.tf_ramp(16), domain=(0.25, 0.5), cells_per_mc=4)
    check(s)


def test_remap_after_tf_change(cuda):
    import torch
    s = scenes.small_scene(dims=32)
    g = GpuScene(s, layout=N.GBV_LAYOUT_LINEAR)
    s2 = scenes.small_scene(dims=32)
    s2.tf = scenes.tf_two_peaks(256)
    g.s = s2
    g.tf = torch.from_numpy(s2.tf).cuda()
    g.map_majorants()
    torch.cuda.synchronize()
    o = oracle.Oracle(s2)
    m_o = o.majorants_of(o.mc_ranges())
    np.testing.assert_array_equal(g.majorants.cpu().numpy()[: m_o.size].view(np.uint32), m_o.view(np.uint32))
