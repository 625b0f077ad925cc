"""Batched rendering: many uneven scenes in one persistent launch equal the
same scenes rendered one by one, bit for bit; a captured CUDA graph replays
the launch."""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes
from barney_gb300.batch import GpuBatch
from barney_gb300.device import GpuScene

pytestmark = pytest.mark.gpu


def small_items(n=6):
    items = scenes.batch_items(n, seed=5, lo=16, hi=48)
    for k, s in enumerate(items):
        s.width, s.height = [(24, 16), (40, 40), (17, 33), (64, 24), (8, 8), (33, 17)][k % 6]
        s.spp = 3
    items[1].multi_scatter, items[1].volume_multi_scatter, items[1].max_volume_bounces = 1, 1, 4
    items[1].env = scenes.env_sky(64, 32)
    return items


def test_batch_equals_separate_renders(cuda):
    import torch
    items = small_items()
    b = GpuBatch(items)
    b.render(spp=3)
    b.render(spp=2, accum_id_start=3)
    torch.cuda.synchronize()
    for s, acc in zip(items, b.accums):
        g = GpuScene(s)
        ref = g.render(spp=3)
        g.render(spp=2, accum=ref, accum_id_start=3)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(acc.cpu().numpy().view(np.uint32), ref.cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("shape", [(4, 30, 4), (5, 5, 8), (6, 90, 16)])
def test_launch_shapes_do_not_change_results(cuda, shape):
    import torch
    items = small_items()
    b = GpuBatch(items)
    b.render(spp=3)
    ref = [a.clone() for a in b.accums]
    for a in b.accums:
        a.zero_()
    b.set_launch(*shape)
    b.render(spp=3)
    torch.cuda.synchronize()
    for a, r in zip(b.accums, ref):
        assert torch.equal(a, r)


def test_batch_graph_replay(cuda):
    import torch
    items = small_items()
    b = GpuBatch(items)
    b.render(spp=3)
    ref = [a.clone() for a in b.accums]
    for a in b.accums:
        a.zero_()
    g = b.capture(spp=3)
    g.replay()
    torch.cuda.synchronize()
    for a, r in zip(b.accums, ref):
        assert torch.equal(a, r)
    for a in b.accums:
        a.zero_()
    g.replay()
    torch.cuda.synchronize()
    for a, r in zip(b.accums, ref):
        assert torch.equal(a, r)


def test_autotuner_picks_shapes_caches_them_and_keeps_images(cuda, tmp_path, monkeypatch):
    import torch
    from barney_gb300 import autotune
    monkeypatch.setenv("GBV_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    items = small_items()
    ref = GpuBatch(items)
    ref.render(spp=3)
    bricks = [(3, 3, 3), (2, 2, 2), (4, 3, 2)]
    launches = [(5, 5, 8), (4, 30, 4)]
    b, rec = autotune.tuned_batch(items, 3, bricks=bricks, reps=1)
    assert not rec["cached"] and rec["brick"] in bricks
    assert (tmp_path / "tune.json").exists()
    b.render(spp=3)
    torch.cuda.synchronize()
    for a, r in zip(b.accums, ref.accums):
        assert torch.equal(a, r)
    b2, rec2 = autotune.tuned_batch(items, 3, bricks=bricks, reps=1)
    assert rec2["cached"] and rec2["brick"] == rec["brick"] and rec2["launch"] == rec["launch"]
    got = autotune.tune_batch(b2, 3, candidates=launches, reps=1, use_cache=False)
    assert got["launch"] in launches and len(got["timed"]) == 2
