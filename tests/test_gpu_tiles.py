"""gbv_render_tiles: each rank's share of the frame equals the full render
on the tiles it owns, leaves every other pixel alone, and the shares put
together are the frame."""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes, tiles
from barney_gb300.device import GpuScene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("R,multi", [(1, False), (3, False), (4, True), (200, False)])
def test_rank_shares_make_the_frame(cuda, R, multi):
    import torch
    if multi:
        s = scenes.frame_scene(dims=40, width=100, height=70, spp=3)
        s.env = scenes.env_sky(64, 32)
    else:
        s = scenes.small_scene(dims=40, spp=3, width=100, height=70)
    g = GpuScene(s)
    full = g.render()
    full2 = g.render(spp=2, accum=full.clone(), accum_id_start=3)
    cf = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    g.render(counters=cf)
    assembled = torch.full_like(full, float("nan"))
    csum = torch.zeros_like(cf)
    for r in range(R):
        mine = torch.full_like(full, -3.0)
        c = torch.zeros_like(cf)
        g.render_tiles(r, R, accum=mine, counters=c)
        g.render_tiles(r, R, spp=2, accum=mine, accum_id_start=3)
        csum += c
        low = tiles.tile_partition(s.width, s.height, r, R)
        owned = torch.zeros(full.shape[:2], dtype=torch.bool, device="cuda")
        for x, y in low:
            owned[y:y + 32, x:x + 32] = True
        assert torch.equal(mine[owned], full2[owned])
        assert bool((mine[~owned] == -3.0).all())
        tiles.unpack_tiles(assembled, tiles.pack_tiles(mine, low), low)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(assembled.cpu().numpy().view(np.uint32), full2.cpu().numpy().view(np.uint32))
    assert csum[:5].tolist() == cf[:5].tolist()


def test_render_tiles_rejects_bad_rank(cuda):
    import ctypes as C
    from barney_gb300.device import _ptr, _stream
    s = scenes.small_scene(dims=16, spp=1, width=8, height=8)
    g = GpuScene(s)
    acc = g.new_accum()
    rec = g.record()
    assert N.lib().gbv_render_tiles(C.byref(rec), _ptr(acc), 8, 8, 0, 1, 1, 1, None, _stream()) == 1
    assert N.lib().gbv_render_tiles(C.byref(rec), _ptr(acc), 8, 8, 0, 1, 0, 0, None, _stream()) == 1
