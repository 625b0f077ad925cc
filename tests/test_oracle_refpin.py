"""The CPU oracle against the reference's own code (CPU only).

The reference renderer's sources for the structured-volume path compile
unchanged here (oracle/refpin, `make -C oracle ref`): its RNG and hash,
fastLog, the float/half conversions of its CPU backend, the transfer
function's map and majorant, the structured field's sampler with the CPU
backend's trilinear texture, sampleAndMap, the macrocell range build, the
macrocell DDA and the whole per-ray volume intersection program MCVolumeAccel::isProg (box test, RNG
stream, DDA over the majorant grid, Woodcock tracking, hit record), the
iso-surface intersection program MCIsoSurfaceAccel::isProg with an AnariMatte
material (hit search, normal, opacity test, Ray::setHit), the material's
Lambertian BSDF, the camera commit and ray generation, the shading step
bounce() of the default and the multi-scatter build with the env map's
importance tables (tests/golden/shade_pin.npz, make_shade_golden.py), and
the frame buffer's 8-bit and sRGB packing.  Their outputs on fixed inputs are
stored in tests/golden/ref_pin.npz (tests/golden/make_ref_golden.py); the
oracle must reproduce every one bit for bit.  Where the reference checkout
is present the live library is also compared on fresh random inputs.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from oracle import refpin

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_pin.npz"
SHADE = GOLDEN.parent / "shade_pin.npz"


@pytest.fixture(scope="module")
def pin():
    z = np.load(GOLDEN)
    c = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    o = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return c, o


def bits(a):
    a = np.ascontiguousarray(a, np.float32)
    return a.view(np.uint32)


def same_or_both_nan(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(bits(a)[~na], bits(b)[~nb])


def _scene(c, tf, domain, bd, cells_per_mc=8):
    from barney_gb300 import scenes
    s = scenes.Scene(scalars=c["vol"], tf=tf, base_density=bd, cells_per_mc=cells_per_mc)
    s.domain = tuple(domain)
    o = oracle.Oracle(s)
    o.rec.origin[:] = list(c["vol_origin"])
    o.rec.spacing[:] = list(c["vol_spacing"])
    return o


# ---- the oracle against the stored reference outputs ----------------------

def test_rng_streams(pin):
    c, o = pin
    got = np.stack([oracle.rng_sequence(int(a), int(b), 16) for a, b in c["rng_ab"]])
    assert np.array_equal(bits(got), bits(o["rng_seq"]))
    L = oracle.lib()
    seqs, states = [], []
    for u64 in (0, 1):
        for st, h in zip(c["seed_states"], c["seed_hashes"]):
            out = np.empty(8, np.float32)
            ns = oracle.C.c_uint64()
            L.orc_rng_from_seed(int(st), int(h), u64, 8, oracle._p(out), oracle.C.byref(ns))
            seqs.append(out)
            states.append(ns.value)
    assert np.array_equal(bits(np.stack(seqs)), bits(o["rng_seed_seq"]))
    assert np.array_equal(np.array(states, np.uint64), o["rng_seed_state"])
    seeded = np.array([L.orc_rng_seed_state(int(a), int(b)) for a, b in c["rng_ab"]], np.uint64)
    assert np.array_equal(seeded, o["rng_seeded"])
    h = np.array([L.orc_hash3(int(a), int(b), int(x)) for a, b, x in c["hash_abc"]], np.uint64)
    assert np.array_equal(h, o["hash3"])


def test_fast_log(pin):
    c, o = pin
    got = np.array([oracle.fast_log(float(v)) for v in c["log_x"]], np.float32)
    assert np.array_equal(bits(got), bits(o["log"]))


def test_half_conversions(pin):
    c, o = pin
    L = oracle.lib()
    got = np.array([L.orc_float_to_half(float(v)) for v in c["half_x"]], np.uint16)
    assert np.array_equal(got, o["half"])
    back = np.array([L.orc_half_to_float(h) for h in range(65536)], np.float32)
    assert same_or_both_nan(back, o["half_all"].view(np.float32))


@pytest.mark.parametrize("k,domain,bd", [("a", (0.0, 1.0), 50.0), ("b", (0.0, 1.0), 20.0), ("c", (0.15, 0.85), 3.5)])
def test_transfer_function_map_and_majorant(pin, k, domain, bd):
    c, o = pin
    orc = _scene(c, c[f"tf_{k}"], domain, bd)
    assert np.array_equal(bits(orc.tf_map(c["tf_s"])), bits(o[f"map_{k}"]))
    assert np.array_equal(bits(orc.majorants_of(c["tf_ranges"])), bits(o[f"maj_{k}"]))


def test_field_sampler(pin):
    c, o = pin
    orc = _scene(c, c["tf_a"], (0.0, 1.0), 40.0)
    got = orc.sample(c["pts"])
    assert same_or_both_nan(got, o["sample"])
    assert np.isnan(got).sum() > 100 and (~np.isnan(got)).sum() > 1000
    # sampleAndMap: NaN (outside) maps to zero
    s = np.nan_to_num(got, nan=0.0)
    m = orc.tf_map(s)
    m[np.isnan(got)] = 0.0
    assert np.array_equal(bits(m), bits(o["sample_map"]))


def test_macrocell_ranges(pin):
    """StructuredData::buildMCs / StructuredData_computeMCs: the scalar range
    of every 8-cell macrocell (9^3 voxels each, clipped at the field's edge)
    through the field's nearest-neighbour texture."""
    c, o = pin
    got = _scene(c, c["tf_a"], (0.0, 1.0), 40.0, cells_per_mc=8).mc_ranges()
    assert np.array_equal(bits(got), bits(o["mc_ranges_8"]))


def test_volume_intersection_program(pin):
    """MCVolumeAccel::isProg: hit flag, t, hit point, the phase function's
    albedo (the default build's Phase(color) keeps 0.7 x the sampled
    colour, packedBSDF/Phase.h:121-145) and the ray's RNG seed afterwards."""
    c, o = pin
    cpm = int(c["trace_cpm"][0])
    orc = _scene(c, c["tf_a"], (0.0, 1.0), 40.0, cells_per_mc=cpm)
    maj = orc.majorants_of(orc.mc_ranges())
    assert np.array_equal(bits(maj), bits(o["trace_majorants"]))
    orc.majorants = np.ascontiguousarray(maj)
    orc.rec.majorants = orc.majorants.ctypes.data
    L = oracle.lib()
    C = oracle.C
    nhit = 0
    for i in range(c["ray_org"].shape[0]):
        org, d = c["ray_org"][i].copy(), c["ray_dir"][i].copy()
        st = C.c_uint64(int(c["ray_seed"][i]))
        t = C.c_float(0.0)
        rgb = np.zeros(3, np.float32)
        h = L.orc_trace_ray(C.byref(orc.rec), oracle._p(org), oracle._p(d), float(c["ray_tmax"][i]), C.byref(st),
                            C.byref(t), oracle._p(rgb))
        assert bool(h) == bool(o["trace_hit"][i]), i
        assert st.value == int(o["trace_state"][i]), i
        if h:
            nhit += 1
            tt = np.float32(t.value)
            assert bits(tt) == bits(o["trace_t"][i]), i
            P = org + tt * d
            assert np.array_equal(bits(P), bits(o["trace_P"][i])), i
            assert np.array_equal(bits(np.float32(0.7) * rgb), bits(o["trace_albedo"][i])), i
    assert nhit > 100


def test_iso_surface_intersection_program(pin):
    """MCIsoSurfaceAccel::isProg with an AnariMatte material: hit flag, t,
    hit point, the normal in half precision, the Lambertian's albedo
    (0.85 color / pi) and alpha, the opacity test's stream (opacity 0.7)
    and the ray's RNG seed afterwards, for instance indices 0, 1 and 3."""
    c, o = pin
    cpm = int(c["iso_cpm"][0])
    orc = _scene(c, c["tf_a"], (0.0, 1.0), 40.0, cells_per_mc=cpm)
    rg = orc.mc_ranges()
    assert np.array_equal(bits(rg), bits(o["iso_ranges"]))
    k = 0
    hits = 0
    for iv in c["iso_values"]:
        for m in range(c["iso_colors"].shape[0]):
            for org, d, tm, sd in zip(c["ray_org"], c["ray_dir"], c["ray_tmax"], c["ray_seed"]):
                h, st, t, P, Nh, alb = orc.iso_hit(org, d, float(tm), int(sd), float(iv), c["iso_colors"][m],
                                                   float(c["iso_opacity"][m]), int(c["iso_inst"][m]), ranges=rg)
                assert h == bool(o["iso_hit"][k]), k
                assert st == int(o["iso_state"][k]), k
                if h:
                    hits += 1
                    assert bits(np.float32(t)) == bits(o["iso_t"][k]), k
                    assert np.array_equal(bits(P), bits(o["iso_P"][k])), k
                    assert np.array_equal(Nh, o["iso_N"][k]), k
                    assert np.array_equal(bits(alb), bits(o["iso_albedo"][k])), k
                k += 1
    assert hits > 1000
    # the opacity test let some rays through that the opaque material stops
    per = len(c["ray_org"])
    assert o["iso_hit"][2 * per:3 * per].sum() < o["iso_hit"][0:per].sum()


def test_lambertian_bsdf(pin):
    """The AnariMatte Lambertian: eval (value, pdf), pdf, and a scatter
    (direction, pdf, f_r).  The scatter takes its two draws in the order the
    reference's gcc build evaluates vec2f s(random(), random()): the second
    argument first.  The direction goes through owl's frame(), which the
    reference pin restates (the owl source is absent)."""
    c, o = pin
    got = np.stack([oracle.lambertian(col, ng, wo, wi, int(a), int(b)) for col, ng, wo, wi, (a, b) in
                    zip(c["lam_color"], c["lam_Ng"], c["lam_wo"], c["lam_wi"], c["lam_ab"])])
    assert np.array_equal(bits(got), bits(o["lambertian"]))
    assert (o["lambertian"][:, 3] == 0).sum() > 500  # light below the surface: pdf 0


def _shade_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_shade_golden", SHADE.parent / "make_shade_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def shade():
    z = np.load(SHADE)
    c = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    o = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return c, o


def test_env_importance_tables(shade):
    """EnvMapLight::computeCDFs (EnvMap.cu:181-238): per-texel weights from
    the 3x3 texture taps, row CDFs, the row weights and their CDF, for the
    sky map and a random map under every address mode."""
    c, o = shade
    mod = _shade_module()
    for t, tex in enumerate(mod.env_textures()):
        for a, addr in enumerate(c["addrs"]):
            cy, cx = oracle.env_cdfs(tex, tuple(int(v) for v in addr))
            assert np.array_equal(bits(cy), bits(o[f"cdf_y_{t}_{a}"])), (t, addr)
            assert np.array_equal(bits(cx), bits(o[f"cdf_x_{t}_{a}"])), (t, addr)


def test_shading_step(shade):
    """bounce() (shadeRays.cu:477-878) of the default and the multi-scatter
    build: misses (background and env light), shadow rays, volume hits
    (Phase) and matte-surface hits (Lambertian) at depths 0..10, on worlds
    with directional lights, an env map and ambient light -- light
    selection, env-map importance sampling, MIS weights, the phase and
    Lambertian scatter, bounce limits and the path's random streams, all bit
    for bit."""
    c, o = shade
    mod = _shade_module()
    got = mod.run(c, oracle.bounce, (o["cdf_y_0_0"], o["cdf_x_0_0"]))
    ref = o["bounce"]
    assert np.array_equal(got, ref)
    # what the cases cover
    recs = (oracle.OrcShadePath * len(c["depth"])).from_buffer_copy(c["paths"].tobytes())
    hits = np.array([p.hit for p in recs])
    shadows = ref[:, 22] != 0
    alive = ref[:, 6] != np.float32(-1).view(np.uint32)
    for m in (0, 1):
        for h in (0, 1, 2):
            sel = (c["multi"] == m) & (hits == h)
            assert sel.sum() > 100
            if h:
                assert shadows[sel].sum() > 20
    assert alive[(c["multi"] == 1) & (hits == 1)].sum() > 20   # volume bounces of the multi-scatter build
    assert alive[hits == 2].sum() > 20                          # diffuse surface bounces


def test_camera_and_ray_generation(shade):
    """PerspectiveCamera::commit and _generateRays: per pixel the origin,
    direction, tMax, background colour and the ray's seed state, for frames
    with partial 32x32 tiles, pass 0 (pixel centres) and jittered passes,
    a constant background and the gradient; the path state starts at
    throughput 1, MIS weight 0."""
    c, o = shade
    mod = _shade_module()
    got = mod.run_cameras(c, oracle.camera_commit, oracle.generate)
    assert np.array_equal(bits(got["commit"]), bits(o["commit"]))
    assert np.array_equal(bits(got["rays"]), bits(o["rays"]))
    assert np.array_equal(got["seeds"], o["seeds"])
    assert not got["gen_bad"].any() and not o["gen_bad"].any()


def test_frame_buffer_packing(pin):
    c, o = pin
    acc = c["rgba"].reshape(1, -1, 4)
    assert np.array_equal(oracle.Oracle.tonemap(None, acc, 1, 1).reshape(-1), o["rgba8"])
    assert np.array_equal(oracle.Oracle.tonemap(None, acc, 1, 2).reshape(-1), o["srgb8"])


# ---- the live reference library (where the reference checkout is) --------

live = pytest.mark.skipif(not refpin.reference_present(), reason="reference checkout absent")


@live
def test_live_library_reproduces_the_fixtures(pin):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_ref_golden", GOLDEN.parent / "make_ref_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    c, o = pin
    fresh = mod.cases()
    for k, v in c.items():
        assert np.array_equal(np.asarray(v), np.asarray(fresh[k])), k
    out = mod.reference_outputs(c)
    for k, v in o.items():
        a, b = np.asarray(v), np.asarray(out[k])
        if a.dtype == np.float32:
            assert same_or_both_nan(a, b), k
        else:
            assert np.array_equal(a, b), k


@live
def test_live_shading_reproduces_the_fixtures(shade):
    c, o = shade
    mod = _shade_module()
    fresh = mod.cases()
    for k, v in c.items():
        assert np.array_equal(np.asarray(v), np.asarray(fresh[k])), k
    out = mod.reference_outputs(c)
    for k, v in o.items():
        assert np.array_equal(np.asarray(v).view(np.uint32) if np.asarray(v).dtype == np.float32 else v,
                              np.asarray(out[k]).view(np.uint32) if np.asarray(out[k]).dtype == np.float32
                              else out[k]), k


@live
def test_live_random_rays_and_samples():
    """Fresh random inputs (other seeds, a bench-like TF and macrocells of 8
    and 16 cells): the live reference and the oracle agree bit for bit."""
    from barney_gb300 import scenes
    rng = np.random.default_rng(77)
    vol = scenes.blob_volume((48, 40, 36), 10, seed=99, noise=0.05, fbm_octaves=2, fbm_amplitude=0.1)
    origin = np.array([-0.5, -0.5, -0.5], np.float32)
    spacing = np.array([1 / 47, 1 / 39, 1 / 35], np.float32)
    tf = scenes.tf_two_peaks(256)
    c = {"vol": vol, "vol_origin": origin, "vol_spacing": spacing}
    pts = ((rng.random((3000, 3)) * 1.2) - 0.6).astype(np.float32)
    orc = _scene(c, tf, (0.0, 1.0), 50.0)
    assert same_or_both_nan(orc.sample(pts), refpin.sample_points(vol, origin, spacing, pts))
    for cpm in (8, 16):
        orc = _scene(c, tf, (0.0, 1.0), 50.0, cells_per_mc=cpm)
        maj = np.ascontiguousarray(orc.majorants_of(orc.mc_ranges()))
        orc.majorants = maj
        orc.rec.majorants = maj.ctypes.data
        C = oracle.C
        hits = 0
        for i in range(400):
            d = rng.standard_normal(3)
            d /= np.linalg.norm(d)
            org = (2.5 * d).astype(np.float32)
            dirv = ((rng.random(3) - 0.5) * 0.8 - org)
            dirv = (dirv / np.linalg.norm(dirv)).astype(np.float32)
            seed = int(rng.integers(0, 2 ** 63))
            h, t, P, alb, ns = refpin.trace_ray(vol, origin, spacing, cpm, maj, tf, (0.0, 1.0), 50.0, org, dirv,
                                                1e30, seed)
            st = C.c_uint64(seed)
            tt = C.c_float(0.0)
            rgb = np.zeros(3, np.float32)
            h2 = oracle.lib().orc_trace_ray(C.byref(orc.rec), oracle._p(org), oracle._p(dirv), 1e30, C.byref(st),
                                            C.byref(tt), oracle._p(rgb))
            assert h == bool(h2) and ns == st.value, (cpm, i)
            if h:
                hits += 1
                assert bits(np.float32(t)) == bits(np.float32(tt.value)), (cpm, i)
                assert np.array_equal(bits(np.float32(0.7) * rgb), bits(alb)), (cpm, i)
        assert hits > 50


# ---- NanoVDB fields ---------------------------------------------------------

NVDB = Path(__file__).resolve().parent / "golden" / "nanovdb_pin.npz"
# the byte offsets of the NanoVDB float-grid layout the library and the
# oracle read (grid header, map, bboxes, tree header, root, tiles, internal
# nodes, leaves and their sizes)
NVDB_LAYOUT = [672, 296, 560, 608, 636, 36, 72, 64, 24, 64, 32, 8, 20, 24, 28, 4128, 8256, 544, 1088, 96,
               270400, 33856, 2144]


@pytest.fixture(scope="module")
def nvdb():
    z = np.load(NVDB)
    return {k: z[k] for k in z.files}


def test_nanovdb_layout_is_the_vendored_library_layout(nvdb):
    assert nvdb["layout"].tolist() == NVDB_LAYOUT


def _nvdb_oracle(grid):
    from barney_gb300 import scenes
    s = scenes.Scene(scalars=np.zeros((2, 2, 2), np.float32), tf=scenes.tf_ramp(128), base_density=20.0)
    return oracle.Oracle(s, nanovdb=grid)


def test_oracle_nanovdb_field_against_the_reference(nvdb):
    """NanoVDBDataSampler::DD::sample and NanoVDBData_computeMCs of the
    reference (with the vendored NanoVDB library) against the oracle's
    restatement: samples, macrocell grid and ranges bit for bit."""
    o = _nvdb_oracle(nvdb["grid"].tobytes())
    assert same_or_both_nan(o.sample(nvdb["points"]), nvdb["samples"])
    assert (o.sample(nvdb["points"]) > 0).sum() > 500
    mc, world = o.mc_grid()
    assert list(mc) == nvdb["mc_dims"].tolist()
    assert np.array_equal(np.array(world, np.float32).view(np.uint32), nvdb["world"].view(np.uint32))
    assert np.array_equal(o.mc_ranges().view(np.uint32), nvdb["ranges"].view(np.uint32))


@live
def test_live_nanovdb_grids():
    """Fresh grids (another volume, index origin, voxel size and
    translation): the live reference and the oracle agree."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_nanovdb_golden", NVDB.parent / "make_nanovdb_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    from barney_gb300 import scenes
    rng = np.random.default_rng(5)
    for seed, origin, vs, tr in ((31, (0, 0, 0), 0.05, (-0.5, -0.5, -0.5)), (32, (-40, 17, -3), 0.021, (0.1, -0.3, 0.2))):
        vol = scenes.blob_volume((45, 21, 33), 5, seed=seed, noise=0.02)
        vol = np.where(vol < 0.03, np.float32(0.0), vol).astype(np.float32)
        grid = mod.make_grid(vol, origin, vs, tr)
        pts = (rng.random((2000, 3)) * 2.4 - 1.2).astype(np.float32)
        o = _nvdb_oracle(grid)
        assert same_or_both_nan(o.sample(pts), mod.reference_samples(grid, pts))
        mc, world, ranges = mod.reference_mc(grid)
        assert list(o.mc_grid()[0]) == mc.tolist()
        assert np.array_equal(o.mc_ranges().view(np.uint32), ranges.view(np.uint32))


# ---- quantized NanoVDB grids (Fp4, Fp8, Fp16, FpN) ---------------------------

NVDB_FP = Path(__file__).resolve().parent / "golden" / "nanovdb_fp_pin.npz"
FP_NAMES = ["fp4", "fp8", "fp16", "fpn_fine", "fpn_coarse"]
# LeafFnBase's flags, minimum and quantum offsets and size; the codes' offset
# in Fp4/Fp8/Fp16 leaves and their sizes; LeafData<FpN>'s size and its
# 8-bit memUsage; the upper and lower node sizes of the four types; the
# GridType values of Float, Fp4, Fp8, Fp16, FpN
NVDB_FP_LAYOUT = [15, 80, 84, 96, 96, 96, 96, 352, 608, 1120, 96, 608] + [270400] * 4 + [33856] * 4 + \
    [1, 13, 14, 15, 16]


@pytest.fixture(scope="module")
def nvdb_fp():
    z = np.load(NVDB_FP)
    return {k: z[k] for k in z.files}


def test_nanovdb_quantized_layout_is_the_vendored_library_layout(nvdb_fp):
    assert nvdb_fp["fp_layout"].tolist() == NVDB_FP_LAYOUT


def _fpn_widths(grid: bytes):
    """Bit widths of an FpN grid's leaves, walked in storage order."""
    import struct
    leaf0 = 672 + struct.unpack_from("<Q", grid, 672)[0]
    count = struct.unpack_from("<I", grid, 672 + 32)[0]
    off, widths = leaf0, set()
    for _ in range(count):
        w = 1 << (grid[off + 15] >> 5)
        widths.add(w)
        off += 96 + 64 * w
    return widths


@pytest.mark.parametrize("name", FP_NAMES)
def test_oracle_quantized_nanovdb_against_the_reference(nvdb_fp, name):
    """The reference's NanoVDBDataSampler<Fp4|Fp8|Fp16|FpN> and
    NanoVDBData_computeMCs<...> on grids the vendored library quantized,
    against the oracle: samples and macrocell ranges bit for bit."""
    grid = nvdb_fp[f"grid_{name}"].tobytes()
    o = _nvdb_oracle(grid)
    got = o.sample(nvdb_fp["points"])
    assert same_or_both_nan(got, nvdb_fp[f"samples_{name}"])
    assert (got > 0).sum() > 500
    assert list(o.mc_grid()[0]) == nvdb_fp[f"mc_dims_{name}"].tolist()
    assert np.array_equal(o.mc_ranges().view(np.uint32), nvdb_fp[f"ranges_{name}"].view(np.uint32))


def test_fpn_fixtures_cover_every_bit_width(nvdb_fp):
    widths = _fpn_widths(nvdb_fp["grid_fpn_fine"].tobytes()) | _fpn_widths(nvdb_fp["grid_fpn_coarse"].tobytes())
    assert widths == {1, 2, 4, 8, 16}


@live
def test_live_quantized_nanovdb_grids():
    """Fresh quantized grids of another volume and placement: the live
    reference and the oracle agree for every type."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_nanovdb_golden", NVDB.parent / "make_nanovdb_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    from barney_gb300 import scenes
    rng = np.random.default_rng(6)
    vol = scenes.blob_volume((33, 25, 41), 5, seed=33, noise=0.02)
    vol = np.where(vol < 0.03, np.float32(0.0), vol).astype(np.float32)
    pts = (rng.random((2000, 3)) * 2.4 - 1.2).astype(np.float32)
    for gtype, tol in ((13, -1.0), (14, -1.0), (15, -1.0), (16, 0.002), (16, 0.02), (16, -1.0)):
        grid = mod.make_grid(vol, (-12, 40, 5), 0.027, (0.2, -0.4, 0.1), grid_type=gtype, tolerance=tol, fog=True)
        o = _nvdb_oracle(grid)
        assert same_or_both_nan(o.sample(pts), mod.reference_samples(grid, pts)), (gtype, tol)
        mc, world, ranges = mod.reference_mc(grid)
        assert list(o.mc_grid()[0]) == mc.tolist()
        assert np.array_equal(o.mc_ranges().view(np.uint32), ranges.view(np.uint32)), (gtype, tol)
