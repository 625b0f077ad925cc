"""The wavefront render mode (trace kernel over a ray queue, shade kernel
over the active pixels, path state in HBM) against the persistent kernel:
bit-identical accumulation buffers and event counts, every voxel store, single
and multiple scattering, env map, progressive accumulation, ragged frames."""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes
from barney_gb300.device import GpuScene

pytestmark = pytest.mark.gpu

WF = {"mode": N.GBV_RENDER_WAVEFRONT}


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _pair(g, spp, start=0, config=None, w=None, h=None):
    import torch
    c0 = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    c1 = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    a = g.new_accum(w, h)
    b = g.new_accum(w, h)
    if start:
        a.fill_(0.25)
        b.fill_(0.25)
    g.render(spp=spp, accum=a, accum_id_start=start, counters=c0, width=w, height=h)
    g.render(spp=spp, accum=b, accum_id_start=start, counters=c1, width=w, height=h, config=config or WF)
    torch.cuda.synchronize()
    return a.cpu().numpy(), b.cpu().numpy(), c0.cpu().tolist(), c1.cpu().tolist()


@pytest.mark.parametrize("store", [(N.GBV_LAYOUT_BRICK_CORNERS, N.GBV_VOXEL_F32),
                                   (N.GBV_LAYOUT_BRICK_CORNERS, N.GBV_VOXEL_F16),
                                   (N.GBV_LAYOUT_BRICK_CORNERS, N.GBV_VOXEL_U8_SCALED),
                                   (N.GBV_LAYOUT_LINEAR, N.GBV_VOXEL_F32)], ids=["f32", "f16", "u8", "linear"])
def test_single_scatter_frames_identical(cuda, store):
    s = scenes.small_scene(dims=48, spp=6, width=70, height=45)
    g = GpuScene(s, layout=store[0], fmt=store[1])
    a, b, c0, c1 = _pair(g, 6)
    np.testing.assert_array_equal(bits(a), bits(b))
    assert c0[:5] == c1[:5] and c0[0] > 0


@pytest.mark.parametrize("env", [False, True])
def test_multi_scatter_frames_identical(cuda, env):
    s = scenes.frame_scene(dims=40, width=61, height=37, spp=5)
    if env:
        s.env = scenes.env_sky(64, 32)
    else:
        s.env = None
    g = GpuScene(s)
    a, b, c0, c1 = _pair(g, 5)
    np.testing.assert_array_equal(bits(a), bits(b))
    assert c0[:5] == c1[:5]


def test_progressive_accumulation_and_settings(cuda):
    """accum_id_start > 0 (the buffer's sum continues), refill thresholds
    and staging modes: the same frame."""
    s = scenes.frame_scene(dims=40, width=48, height=40, spp=3)
    s.env = scenes.env_sky(64, 32)
    g = GpuScene(s)
    for cfg in (dict(WF), dict(WF, threshold_pct=100), dict(WF, threshold_pct=1, skip_cells=1),
                dict(WF, stage=N.GBV_STAGE_NONE), dict(WF, stage=N.GBV_STAGE_ALL)):
        a, b, c0, c1 = _pair(g, 3, start=7, config=cfg)
        np.testing.assert_array_equal(bits(a), bits(b))
        assert c0[:5] == c1[:5]


def test_bench_frame_one_pass_identical(cuda):
    """The bench's scene (512^3, 1920x1080, multiple scattering, env map),
    two passes: identical accumulation buffers and counts."""
    import torch
    s = scenes.frame_scene(spp=2)
    g = GpuScene(s)
    a, b, c0, c1 = _pair(g, 2)
    np.testing.assert_array_equal(bits(a), bits(b))
    assert c0[:5] == c1[:5]
    del g
    torch.cuda.empty_cache()
