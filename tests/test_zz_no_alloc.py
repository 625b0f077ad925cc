"""gbv_render_noalloc: the frame render for callers that may not allocate.

Some applications cannot let a library allocate device memory while they
render (they hand out all HBM from their own pre-sized pool, or forbid
allocation calls on their frame path).  gbv_render_noalloc takes its one
word of scratch from a static device array instead of cudaMallocAsync; its
frames must equal gbv_render's bit for bit, call after call.

This file is collected last so that a run stopping at the first failure has
run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes
from barney_gb300.device import GpuScene, _ptr, _stream

pytestmark = pytest.mark.gpu


def _noalloc(g: GpuScene, accum, accum_id_start: int, spp: int, counters=None):
    rec = g.record()
    h, w, _ = accum.shape
    return N.lib().gbv_render_noalloc(C.byref(rec), _ptr(accum), w, h, accum_id_start, spp, _ptr(counters),
                                      _stream())


STORES = [
    (N.GBV_LAYOUT_BRICK_CORNERS, N.GBV_VOXEL_F32),
    (N.GBV_LAYOUT_BRICK_CORNERS, N.GBV_VOXEL_F16),
    (N.GBV_LAYOUT_BRICK_CORNERS, N.GBV_VOXEL_BF16),
    (N.GBV_LAYOUT_BRICK_CORNERS, N.GBV_VOXEL_U8_SCALED),
    (N.GBV_LAYOUT_LINEAR, N.GBV_VOXEL_F32),
]


@pytest.mark.parametrize("counted", [True, False], ids=["counted", "uncounted"])
@pytest.mark.parametrize("store", STORES, ids=["f32", "f16", "bf16", "u8", "linear"])
@pytest.mark.parametrize("multi", [False, True], ids=["single", "multi_env"])
def test_noalloc_matches_render_on_two_calls(cuda, multi, store, counted):
    """Both kernels (with and without event counters) of every voxel store:
    two calls in a row, a fresh frame and then progressive passes, each equal
    to gbv_render's frame bit for bit."""
    import torch
    if multi:
        s = scenes.frame_scene(dims=40, width=48, height=40, spp=4)
        s.env = scenes.env_sky(64, 32)
    else:
        s = scenes.small_scene(dims=48, spp=4, width=72, height=56)
    layout, fmt = store
    g = GpuScene(s, layout=layout, fmt=fmt)
    ref = g.new_accum()
    got = g.new_accum()
    c_ref = c_got = None
    if counted:
        c_ref = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
        c_got = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    # two calls in a row: a fresh frame, then 4 more progressive passes
    g.render(spp=4, accum=ref, accum_id_start=0, counters=c_ref)
    assert _noalloc(g, got, 0, 4, c_got) == N.GBV_OK, N.lib().gbv_last_error()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(got.cpu().numpy().view(np.uint32), ref.cpu().numpy().view(np.uint32))
    g.render(spp=4, accum=ref, accum_id_start=4, counters=c_ref)
    assert _noalloc(g, got, 4, 4, c_got) == N.GBV_OK, N.lib().gbv_last_error()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(got.cpu().numpy().view(np.uint32), ref.cpu().numpy().view(np.uint32))
    assert float(np.abs(got.cpu().numpy()).sum()) > 0
    if counted:
        assert c_got[:5].tolist() == c_ref[:5].tolist()
        assert c_got[0].item() > 0


def test_noalloc_rejects_oversized_frames(cuda):
    s = scenes.small_scene(dims=16, spp=1, width=8, height=8)
    g = GpuScene(s)
    acc = g.new_accum()
    rec = g.record()
    # 2^31-1 x 1 pixels is 2^28 tiles (accepted by the size rule, whose sums
    # are 64-bit); with 2^31-1 or 2^13 rows it is far beyond the 2^30 tiles
    # the counter holds (each case is rejected before any launch)
    for w, h in ((2 ** 31 - 1, 2 ** 31 - 1), (2 ** 31 - 1, 2 ** 13)):
        st = N.lib().gbv_render_noalloc(C.byref(rec), _ptr(acc), w, h, 0, 1, None, _stream())
        assert st == 1, (w, h)
        assert "2^30 tiles" in N.lib().gbv_last_error().decode()
