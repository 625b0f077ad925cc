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


# quantized grids: nanovdb::GridType and the largest decode error per value
# relative to the leaf's value range (half a quantum of 2^bits - 1 steps)
QUANTIZED = {"fp4": (13, 0.5 / 15), "fp8": (14, 0.5 / 255), "fp16": (15, 0.5 / 65535)}


@pytest.mark.parametrize("name", ["fp4", "fp8", "fp16", "fpn"])
def test_quantized_grid_holds_the_voxels(name):
    """A quantized grid parses with its type, and at voxel centres gives the
    voxels back within half a quantum of their leaf's range (FpN: within the
    tolerance its bit widths are chosen for)."""
    vol = _vol()
    tol = 0.004
    g = scenes.nanovdb_grid(vol, (-5, 3, 7), 0.03, (-0.4, -0.55, -0.35), grid_type=name, tolerance=tol)
    info = nanovdb.parse(g)
    assert info.grid_type == scenes.NANOVDB_TYPES[name]
    o = oracle.Oracle(scenes.Scene(scalars=vol, tf=scenes.tf_ramp(8)), nanovdb=g)
    rng = np.random.default_rng(0)
    # voxels inside the active index bbox (the sampler clamps to it)
    lo = np.array(info.index_lo) - np.array((-5, 3, 7))
    hi = np.array(info.index_hi) - np.array((-5, 3, 7))
    ijk = np.stack([rng.integers(lo[a], hi[a] + 1, 800) for a in range(3)], axis=1)
    P = (np.array([-0.4, -0.55, -0.35]) + 0.03 * (ijk + np.array((-5, 3, 7)) + 0.5)).astype(np.float32)
    got = o.sample(P)
    want = vol[ijk[:, 2], ijk[:, 1], ijk[:, 0]]
    # a leaf's range is at most the volume's (the background 0 included)
    bound = tol if name == "fpn" else QUANTIZED[name][1] * float(vol.max())
    assert np.abs(got - want).max() <= bound * 1.001 + 2e-6
    assert np.abs(got - want).max() > 0 or name == "fp16"


@pytest.mark.skipif(not refpin.reference_present(), reason="reference checkout absent")
@pytest.mark.parametrize("name,tol", [("fp4", -1.0), ("fp8", -1.0), ("fp16", -1.0), ("fpn", -1.0), ("fpn", 0.001),
                                      ("fpn", 0.05)])
def test_quantized_grid_reads_like_the_vendored_library(name, tol):
    """The writer quantizes as the library's builder does (dithering off;
    FpN's per-leaf bit widths for the same tolerance): the two grids of one
    volume sample and build macrocells bit-identically."""
    import importlib.util
    from pathlib import Path
    path = Path(__file__).resolve().parent / "golden" / "make_nanovdb_golden.py"
    spec = importlib.util.spec_from_file_location("make_nanovdb_golden", path)
    G = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(G)
    vol = _vol()
    kw = dict(voxel_size=0.03, translation=(-0.4, -0.55, -0.35))
    a = scenes.nanovdb_grid(vol, (-5, 3, 7), grid_type=name, tolerance=tol, **kw)
    b = G.make_grid(vol, index_origin=(-5, 3, 7), grid_type=scenes.NANOVDB_TYPES[name], tolerance=tol, fog=True, **kw)
    assert nanovdb.parse(a).grid_type == nanovdb.parse(b).grid_type
    s = scenes.Scene(scalars=vol, tf=scenes.tf_ramp(8))
    oa, ob = oracle.Oracle(s, nanovdb=a), oracle.Oracle(s, nanovdb=b)
    ia = nanovdb.parse(a)
    lo, hi = np.array(ia.world_lo), np.array(ia.world_hi)
    P = (lo - 0.1 + (hi - lo + 0.2) * np.random.default_rng(1).random((20000, 3))).astype(np.float32)
    assert np.array_equal(oa.sample(P).view(np.uint32), ob.sample(P).view(np.uint32))
    assert np.array_equal(oa.mc_ranges().view(np.uint32), ob.mc_ranges().view(np.uint32))


def _corrupt(grid: bytes, at: int, value: bytes) -> bytes:
    b = bytearray(grid)
    b[at:at + len(value)] = value
    return bytes(b)


def test_parser_rejects_bad_quantized_grids():
    """gbv_nanovdb_parse (host code; the device follows the tree unchecked):
    an FpN leaf with a bit width above 16, a child offset off NanoVDB's
    32-byte node alignment, and a value type the reference does not read are
    refused before any device work."""
    import struct
    from barney_gb300 import _native as N
    vol = _vol()
    g = scenes.nanovdb_grid(vol, (0, 0, 0), 0.03, (-0.4, -0.55, -0.35), grid_type="fpn", tolerance=0.01)
    nanovdb.parse(g)
    leaf0 = 672 + struct.unpack_from("<Q", g, 672)[0]
    bad = _corrupt(g, leaf0 + 15, bytes([5 << 5]))  # 32-bit codes
    with pytest.raises(RuntimeError, match="bit width"):
        nanovdb.parse(bad)
    lower0 = 672 + struct.unpack_from("<Q", g, 680)[0]
    # the first child of the first lower node, moved off its 32-byte alignment
    mask = np.frombuffer(g, np.uint8, 512, lower0 + 544)
    k = int(np.flatnonzero(np.unpackbits(mask, bitorder="little"))[0])
    off = struct.unpack_from("<q", g, lower0 + 1088 + 8 * k)[0]
    with pytest.raises(RuntimeError, match="bad leaf"):
        nanovdb.parse(_corrupt(g, lower0 + 1088 + 8 * k, struct.pack("<q", off + 8)))
    with pytest.raises(RuntimeError, match="value type"):
        nanovdb.parse(_corrupt(g, 636, struct.pack("<I", 2)))  # Double
    assert N.GBV_ERROR_UNSUPPORTED != N.GBV_ERROR_INVALID_ARGUMENT
