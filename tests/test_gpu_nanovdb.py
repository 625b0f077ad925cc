"""NanoVDB float-grid fields on the GPU: the library's grid reader, sampler
and macrocell build against the reference's own NanoVDB field code (the
pinned vectors of tests/golden/nanovdb_pin.npz), and frames of a NanoVDB
field against the oracle, through gbv_* and through bn*."""
from pathlib import Path

import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import bn, scenes
from barney_gb300.nanovdb import GpuNanoVDBScene
import oracle

pytestmark = pytest.mark.gpu

PIN = Path(__file__).resolve().parent / "golden" / "nanovdb_pin.npz"


@pytest.fixture(scope="module")
def pin():
    z = np.load(PIN)
    return {k: z[k] for k in z.files}


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _scene(spp=4, w=56, h=40, multi=False):
    if multi:
        s = scenes.frame_scene(dims=8, width=w, height=h, spp=spp)
        s.env = scenes.env_sky(64, 32)
    else:
        s = scenes.small_scene(dims=8, spp=spp, width=w, height=h)
        s.tf = scenes.tf_ramp(128, 0.9)
    return s


def test_sampler_and_macrocells_match_the_reference(cuda, pin):
    import torch
    g = GpuNanoVDBScene(_scene(), pin["grid"].tobytes())
    pts = torch.from_numpy(pin["points"]).cuda()
    got = g.sample(pts).cpu().numpy()
    np.testing.assert_array_equal(bits(got), bits(pin["samples"]))
    assert list(g.mc) == pin["mc_dims"].tolist()
    np.testing.assert_array_equal(bits(g.ranges.cpu().numpy().reshape(-1, 2)), bits(pin["ranges"]))


@pytest.mark.parametrize("multi", [False, True], ids=["single", "multi_env"])
def test_frames_match_the_oracle(cuda, pin, multi):
    """Single scattering bit-exact against the oracle; multiple scattering
    with the env map bit-exact against the oracle's bounded-math mode; event
    counts equal; the wavefront mode gives the same frame."""
    import torch
    s = _scene(multi=multi)
    grid = pin["grid"].tobytes()
    g = GpuNanoVDBScene(s, grid)
    c = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    acc = g.render(spp=4, accum_id_start=2, counters=c)
    wf = g.render(spp=4, accum_id_start=2, config={"mode": N.GBV_RENDER_WAVEFRONT})
    torch.cuda.synchronize()
    o = oracle.Oracle(s, nanovdb=grid, bounded_math=multi)
    ref = o.render(spp=4, accum_id_start=2)
    np.testing.assert_array_equal(bits(acc.cpu().numpy()), bits(ref))
    np.testing.assert_array_equal(bits(wf.cpu().numpy()), bits(ref))
    cc = c.cpu().tolist()
    assert cc[0] == o.stats["density_samples"] and cc[1] == o.stats["mc_visits"] and cc[2] == o.stats["rays"]
    assert cc[0] > 100


def test_bn_nanovdb_field(cuda, pin):
    """A "NanoVDB" scalar field made from a BN_UINT8 data array, as the
    reference's ANARI device makes it, renders the gbv path's frame."""
    import torch
    s = _scene()
    grid = pin["grid"].tobytes()
    with bn.BarneySession() as ses:
        err = ses.build_scene(s, 0, nanovdb=grid)
        assert err == "", err
        ses.render()
        img = ses.read()
    g = GpuNanoVDBScene(s, grid)
    ref = g.tonemap(g.render(), s.spp).cpu().numpy()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bits(img), bits(ref))
    assert float(img[..., :3].sum()) > 0


# ---- quantized grids (Fp4, Fp8, Fp16, FpN) ----------------------------------

PIN_FP = Path(__file__).resolve().parent / "golden" / "nanovdb_fp_pin.npz"
FP_NAMES = ["fp4", "fp8", "fp16", "fpn_fine", "fpn_coarse"]


@pytest.fixture(scope="module")
def pin_fp():
    z = np.load(PIN_FP)
    return {k: z[k] for k in z.files}


@pytest.mark.parametrize("name", FP_NAMES)
def test_quantized_sampler_and_macrocells_match_the_reference(cuda, pin_fp, name):
    """The reference's NanoVDBDataSampler and NanoVDBData_computeMCs on
    grids the vendored library quantized (FpN leaves of every bit width from
    1 to 16 across the two FpN grids): samples and ranges bit for bit."""
    import torch
    g = GpuNanoVDBScene(_scene(), pin_fp[f"grid_{name}"].tobytes())
    assert g.info.grid_type in (13, 14, 15, 16)
    got = g.sample(torch.from_numpy(pin_fp["points"]).cuda()).cpu().numpy()
    np.testing.assert_array_equal(bits(got), bits(pin_fp[f"samples_{name}"]))
    assert list(g.mc) == pin_fp[f"mc_dims_{name}"].tolist()
    np.testing.assert_array_equal(bits(g.ranges.cpu().numpy().reshape(-1, 2)), bits(pin_fp[f"ranges_{name}"]))


@pytest.mark.parametrize("name,multi", [("fp4", False), ("fp8", False), ("fp16", False), ("fpn_coarse", False),
                                        ("fpn_fine", True)])
def test_quantized_frames_match_the_oracle(cuda, pin_fp, name, multi):
    """Frames of a quantized grid: bit-exact against the oracle (its
    bounded-math mode with multiple scattering and the env map), event counts
    equal."""
    import torch
    s = _scene(multi=multi)
    grid = pin_fp[f"grid_{name}"].tobytes()
    g = GpuNanoVDBScene(s, grid)
    c = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    acc = g.render(spp=4, accum_id_start=1, counters=c)
    torch.cuda.synchronize()
    o = oracle.Oracle(s, nanovdb=grid, bounded_math=multi)
    ref = o.render(spp=4, accum_id_start=1)
    np.testing.assert_array_equal(bits(acc.cpu().numpy()), bits(ref))
    cc = c.cpu().tolist()
    assert cc[0] == o.stats["density_samples"] and cc[1] == o.stats["mc_visits"] and cc[2] == o.stats["rays"]
    assert cc[0] > 100


def test_bn_quantized_nanovdb_field(cuda):
    """A "NanoVDB" scalar field holding an Fp16 grid of the frame volume,
    made by the input generator, renders through bn* the frame the gbv path
    renders from the same grid."""
    import torch
    s = scenes.frame_scene(dims=40, width=48, height=32, spp=2)
    grid = scenes.nanovdb_of_scene(s, grid_type="fp16")
    with bn.BarneySession() as ses:
        err = ses.build_scene(s, 0, nanovdb=grid)
        assert err == "", err
        ses.render()
        img = ses.read()
    g = GpuNanoVDBScene(s, grid)
    ref = g.tonemap(g.render(), s.spp).cpu().numpy()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bits(img), bits(ref))
    assert float(img[..., :3].sum()) > 0


@pytest.mark.parametrize("kind", ["iso-only", "iso-first", "volume-first"])
def test_iso_world_on_a_nanovdb_field(cuda, pin, pin_fp, kind):
    """An iso-surface of a NanoVDB field (MCIsoSurfaceAccel over
    NanoVDBDataSampler, barney/volume/NanoVDB.cu), alone or beside the
    field's volume in either instance order: bit-exact against the oracle in
    its bounded-math mode, for a Float and an Fp8 grid."""
    import torch
    inst, vol_inst, no_vol = {"iso-only": (0, 0, True), "iso-first": (0, 1, False),
                              "volume-first": (1, 0, False)}[kind]
    for grid in (pin["grid"].tobytes(), pin_fp["grid_fp8"].tobytes()):
        s = _scene(multi=True)
        s.iso = scenes.IsoSurface(0.3, (0.9, 0.6, 0.3, 1.0), 1.0, inst)
        s.volume_instance, s.no_volume = vol_inst, no_vol
        g = GpuNanoVDBScene(s, grid)
        acc = g.render(spp=4)
        torch.cuda.synchronize()
        o = oracle.Oracle(s, nanovdb=grid, bounded_math=True)
        ref = o.render(spp=4)
        np.testing.assert_array_equal(bits(acc.cpu().numpy()), bits(ref))
        assert float(ref[..., :3].sum()) > 0


def test_bn_iso_surface_of_a_nanovdb_field(cuda, pin_fp):
    """bn*: an "iso_surface" geometry whose "scalarField" is a "NanoVDB"
    field (an FpN grid), beside the field's volume: the frame the gbv path
    renders from the same grid."""
    import torch
    s = _scene(multi=True)
    s.iso = scenes.IsoSurface(0.3, (0.9, 0.6, 0.3, 1.0), 1.0, 0)
    s.volume_instance, s.no_volume = 1, False
    grid = pin_fp["grid_fpn_coarse"].tobytes()
    with bn.BarneySession() as ses:
        err = ses.build_scene(s, 0, nanovdb=grid)
        assert err == "", err
        ses.render()
        img = ses.read()
    g = GpuNanoVDBScene(s, grid)
    ref = g.tonemap(g.render(), s.spp).cpu().numpy()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bits(img), bits(ref))
    assert float(img[..., :3].sum()) > 0


@pytest.mark.parametrize("origin", [(-5, 3, 7), (-1, 0, -2), (3_000_000, -2_500_000, 40)])
def test_sampler_index_arithmetic_edge_cases(cuda, origin):
    """The sampler's index position (the reference computes it in double;
    the device in exact fixed point where that is exact, else in double):
    points whose index coordinates fall on and one float step either side of
    voxel centres, within 2^-17 of index 0 (the double path), outside the
    grid (clamped), and a grid placed beyond +-2^21 (the double path
    throughout) sample bit-identically to the oracle."""
    import torch
    vol = scenes.blob_volume((24, 20, 18), 4, seed=7, noise=0.02)
    vs, tr = 0.03, (-0.4, -0.55, -0.35)
    grid = scenes.nanovdb_grid(vol, origin, vs, tr, background=-1.0)
    g = GpuNanoVDBScene(_scene(), grid)
    o = oracle.Oracle(_scene(), nanovdb=grid)
    rng = np.random.default_rng(11)
    n = 20000
    lo = np.array(origin, np.float64)
    hi = lo + np.array([24, 20, 18]) - 1
    idx = lo - 3 + rng.random((n, 3)) * (hi - lo + 6)      # inside and around the grid
    idx[: n // 4] = np.round(idx[: n // 4]) + 0.5          # voxel centres (u = 0)
    idx[n // 4: n // 2] = np.round(idx[n // 4: n // 2])    # voxel corners
    tiny = rng.standard_normal((n // 8, 3)) * 1e-6          # around index 0 on one axis
    idx[n // 2: n // 2 + n // 8, 0] = tiny[:, 0]
    P = (idx * vs + np.array(tr)).astype(np.float32)
    P[: n // 2] = np.nextafter(P[: n // 2], np.float32(rng.choice([-np.inf, np.inf])))  # one float step off
    got = g.sample(torch.from_numpy(P).cuda()).cpu().numpy()
    np.testing.assert_array_equal(bits(got), bits(o.sample(P)))
