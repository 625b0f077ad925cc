"""The input generator's NanoVDB writer (barney_gb300/scenegen/nanovdb_writer.cpp,
scenes.nanovdb_grid), which gives the NanoVDB field path workloads of any
size: its grids parse, hold the dense values at the voxels, and -- where the
reference checkout is, with its vendored NanoVDB library -- read exactly like
the library's own grid of the same volume (same header fields, samples and
macrocell ranges through the oracle's NanoVDB mode, which the reference pins)."""
import numpy as np
import pytest

import oracle
from oracle import refpin
from barney_gb300 import nanovdb, scenes


def _vol():
    vol = scenes.blob_volume((36, 30, 28), 6, seed=21, noise=0.0)
    return np.where(vol < 0.05, np.float32(0.0), vol).astype(np.float32)


@pytest.mark.parametrize("origin", [(0, 0, 0), (-5, 3, 7), (-4100, 4090, -3)])
def test_grid_holds_the_voxels(origin):
    vol = _vol()
    g = scenes.nanovdb_grid(vol, origin, 0.03, (-0.4, -0.55, -0.35))
    info = nanovdb.parse(g)
    act = np.argwhere(vol != 0)  # (z, y, x)
    assert list(info.index_lo) == [int(act[:, 2].min()) + origin[0], int(act[:, 1].min()) + origin[1],
                                   int(act[:, 0].min()) + origin[2]]
    assert list(info.index_hi) == [int(act[:, 2].max()) + origin[0], int(act[:, 1].max()) + origin[1],
                                   int(act[:, 0].max()) + origin[2]]
    # sampled at voxel centres (index i + 1/2 through the map) the grid gives the voxels back
    o = oracle.Oracle(scenes.Scene(scalars=vol, tf=scenes.tf_ramp(8)), nanovdb=g)
    rng = np.random.default_rng(0)
    ijk = np.stack([rng.integers(0, n, 500) for n in (vol.shape[2], vol.shape[1], vol.shape[0])], axis=1)
    P = (np.array([-0.4, -0.55, -0.35]) + 0.03 * (ijk + np.array(origin) + 0.5)).astype(np.float32)
    got = o.sample(P)
    want = vol[ijk[:, 2], ijk[:, 1], ijk[:, 0]]
    # far from the index origin the float world coordinates (|P| ~ 123 at
    # index 4100: one ulp is 7.6e-6) move the sample off the voxel centre by
    # up to ~3e-4 voxel, so the value moves by up to that times the gradient
    far = max(abs(c) for c in origin) > 1000
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-4 if far else 2e-6)


def test_scene_grid_is_the_structured_field():
    s = scenes.small_scene(dims=24, spp=1, width=8, height=8)
    g = scenes.nanovdb_of_scene(s)
    o_n = oracle.Oracle(s, nanovdb=g)
    o_s = oracle.Oracle(s)
    rng = np.random.default_rng(3)
    P = (rng.random((2000, 3)) * 0.96 - 0.48).astype(np.float32)
    np.testing.assert_allclose(o_n.sample(P), o_s.sample(P), rtol=0, atol=1e-5)


@pytest.mark.skipif(not refpin.reference_present(), reason="reference checkout absent")
@pytest.mark.parametrize("origin", [(0, 0, 0), (-5, 3, 7), (-4100, 4090, -3)])
def test_grid_reads_like_the_vendored_library(origin):
    import importlib.util
    from pathlib import Path
    path = Path(__file__).resolve().parent / "golden" / "make_nanovdb_golden.py"
    spec = importlib.util.spec_from_file_location("make_nanovdb_golden", path)
    G = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(G)
    vol = _vol()
    kw = dict(voxel_size=0.03, translation=(-0.4, -0.55, -0.35))
    a = scenes.nanovdb_grid(vol, origin, **kw)
    b = G.make_grid(vol, index_origin=origin, **kw)
    ia, ib = nanovdb.parse(a), nanovdb.parse(b)
    for f in ("background", "inv_map", "map_offset", "index_lo", "index_hi", "world_lo", "world_hi", "voxel_size",
              "mc_dims"):
        va, vb = getattr(ia, f), getattr(ib, f)
        assert (list(va) if hasattr(va, "__len__") else va) == (list(vb) if hasattr(vb, "__len__") else vb), f
    s = scenes.Scene(scalars=vol, tf=scenes.tf_ramp(8))
    oa, ob = oracle.Oracle(s, nanovdb=a), oracle.Oracle(s, nanovdb=b)
    lo, hi = np.array(ia.world_lo), np.array(ia.world_hi)
    P = (lo - 0.1 + (hi - lo + 0.2) * np.random.default_rng(1).random((20000, 3))).astype(np.float32)
    assert np.array_equal(oa.sample(P).view(np.uint32), ob.sample(P).view(np.uint32))
    assert np.array_equal(oa.mc_ranges().view(np.uint32), ob.mc_ranges().view(np.uint32))
