"""Brick shapes change only where cells sit in HBM: every shape renders the
same frame, bit for bit, and bounds the same macrocell ranges, in every
voxel format."""
import ctypes as C

import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes
from barney_gb300.device import GpuScene

pytestmark = pytest.mark.gpu

SHAPES = [(2, 2, 2), (4, 3, 2), (1, 5, 3), (5, 5, 5), (6, 1, 1)]


def _scene():
    # uneven sides so that every shape pads its last bricks
    s = scenes.frame_scene(dims=37, width=40, height=32, spp=2)
    s.scalars = np.ascontiguousarray(scenes.blob_volume((45, 37, 29), 8, seed=7, noise=0.05))
    s.env = scenes.env_sky(64, 32)
    return s


@pytest.mark.parametrize("fmt", [N.GBV_VOXEL_F32, N.GBV_VOXEL_F16, N.GBV_VOXEL_BF16, N.GBV_VOXEL_U8_SCALED])
def test_brick_shapes_render_identical_frames(cuda, fmt):
    import torch
    s = _scene()
    ref = GpuScene(s, fmt=fmt)
    img_ref = ref.render()
    torch.cuda.synchronize()
    for shape in SHAPES:
        g = GpuScene(s, fmt=fmt, brick=shape)
        assert torch.equal(g.majorants, ref.majorants), shape
        if fmt != N.GBV_VOXEL_F32:
            assert torch.equal(g.ranges, ref.ranges), shape
        if fmt == N.GBV_VOXEL_U8_SCALED:
            assert torch.equal(g.scale_offset, ref.scale_offset), shape
        img = g.render()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(img.cpu().numpy().view(np.uint32), img_ref.cpu().numpy().view(np.uint32),
                                      err_msg=str(shape))


def test_scene_with_out_of_range_brick_shape_is_rejected(cuda):
    s = scenes.small_scene(dims=16, spp=1, width=8, height=8)
    g = GpuScene(s)
    rec = g.record()
    rec.brick_log2[:] = [3, 3, 10]
    acc = g.new_accum()
    from barney_gb300.device import _ptr, _stream
    st = N.lib().gbv_render(C.byref(rec), _ptr(acc), 8, 8, 0, 1, None, _stream())
    assert st == N.GBV_ERROR_INVALID_ARGUMENT
