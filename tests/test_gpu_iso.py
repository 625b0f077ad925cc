"""Iso-surface ray queries (gbv_iso_intersect) against the oracle's
MCIsoSurfaceAccel::isProg restatement: identical hit flags, t, points and
normals, bit for bit, over every voxel store."""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes
from barney_gb300.device import GpuScene
import oracle

pytestmark = pytest.mark.gpu


def make_rays(n=3000, seed=3):
    rng = np.random.default_rng(seed)
    org = rng.normal(size=(n, 3))
    org = rng.uniform(0.9, 2.5, size=(n, 1)) * org / np.linalg.norm(org, axis=1, keepdims=True)
    org[: n // 6] = rng.uniform(-0.45, 0.45, size=(n // 6, 3))  # rays starting inside the volume
    tgt = rng.uniform(-0.35, 0.35, size=(n, 3))
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[n // 6: n // 6 + 60, rng.integers(0, 3, 60)] = 0.0  # zero direction components
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = org
    rays[:, 3] = 1e30
    rays[: n // 10, 3] = rng.uniform(0.5, 3.0, n // 10)  # short rays
    rays[:, 4:7] = d
    return rays


def _compare(got, ref):
    assert np.array_equal(got[:, 7], ref[:, 7])
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("layout,brick", [(N.GBV_LAYOUT_LINEAR, (3, 3, 3)), (N.GBV_LAYOUT_BRICK_CORNERS, (3, 3, 3)),
                                          (N.GBV_LAYOUT_BRICK_CORNERS, (4, 2, 2))])
@pytest.mark.parametrize("iso", [0.3, 0.55])
def test_iso_matches_oracle(cuda, layout, brick, iso):
    import torch
    s = scenes.small_scene(dims=48)
    g = GpuScene(s, layout=layout, brick=brick)
    rays = make_rays()
    got = g.iso_intersect(torch.from_numpy(rays).cuda(), iso).cpu().numpy()
    o = oracle.Oracle(s)
    ref = o.iso_intersect(rays, iso, ranges=o.mc_ranges())
    assert 0.2 < ref[:, 7].mean() < 0.9
    _compare(got, ref)
    hit = ref[:, 7] > 0
    assert np.allclose(np.linalg.norm(got[hit, 4:7], axis=1), 1.0, atol=1e-5)


def test_iso_half_store_matches_oracle_on_rounded_voxels(cuda):
    import torch, copy
    s = scenes.small_scene(dims=40)
    g = GpuScene(s, fmt=N.GBV_VOXEL_F16)
    rays = make_rays(1500, seed=5)
    got = g.iso_intersect(torch.from_numpy(rays).cuda(), 0.45).cpu().numpy()
    sr = copy.copy(s)
    sr.scalars = np.ascontiguousarray(s.scalars.astype(np.float16).astype(np.float32))
    o = oracle.Oracle(sr)
    ref = o.iso_intersect(rays, 0.45, ranges=o.mc_ranges())
    _compare(got, ref)


def test_iso_u8_store_matches_oracle_u8_form(cuda):
    import torch
    s = scenes.small_scene(dims=40)
    g = GpuScene(s, fmt=N.GBV_VOXEL_U8_SCALED)
    rays = make_rays(1500, seed=6)
    got = g.iso_intersect(torch.from_numpy(rays).cuda(), 0.45).cpu().numpy()
    o = oracle.Oracle(s, u8=True)
    ref = o.iso_intersect(rays, 0.45, ranges=o.mc_ranges())
    assert 0.2 < ref[:, 7].mean() < 0.9
    _compare(got, ref)


def test_iso_outside_the_data_range_never_hits(cuda):
    import torch
    s = scenes.small_scene(dims=32)
    g = GpuScene(s)
    got = g.iso_intersect(torch.from_numpy(make_rays(500)).cuda(), 7.0).cpu().numpy()
    assert not got.any()


def test_iso_rejects_bad_arguments(cuda):
    import ctypes as C
    from barney_gb300.device import _ptr, _stream
    s = scenes.small_scene(dims=16)
    g = GpuScene(s)
    rec = g.record()
    assert N.lib().gbv_iso_intersect(C.byref(rec), None, 0.5, None, 4, None, _stream()) == N.GBV_ERROR_INVALID_ARGUMENT
