"""Generates tests/golden/ref_pin.npz: inputs and the reference's own outputs.

The outputs come from the reference renderer's code compiled unchanged
(oracle/_ref/libbarney_ref.so, built by `make -C oracle ref` from the
reference checkout; see oracle/refpin/ref_harness.cpp for what it compiles).
tests/test_oracle_refpin.py checks the CPU oracle against these vectors on
any machine, and against the live library where the reference checkout is.

  python tests/golden/make_ref_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "ref_pin.npz"


def cases(seed: int = 2024) -> dict:
    """Deterministic inputs of every pinned function."""
    rng = np.random.default_rng(seed)
    c = {}
    c["rng_ab"] = rng.integers(0, 2 ** 32, size=(64, 2), dtype=np.uint64).astype(np.uint32)
    c["rng_ab"][:4] = [[0, 0], [1, 0], [0xFFFFFFFF, 0xFFFFFFFF], [1920 * 63 + 5, 7]]
    c["seed_states"] = rng.integers(0, 2 ** 63, size=64, dtype=np.uint64) * np.uint64(2) + np.uint64(1)
    c["seed_hashes"] = rng.integers(0, 2 ** 63, size=64, dtype=np.uint64)
    c["seed_hashes"][:2] = [0, 1]
    c["hash_abc"] = rng.integers(0, 2 ** 32, size=(64, 3), dtype=np.uint64).astype(np.uint32)
    c["hash_abc"][0] = [0, 0, 0]
    c["log_x"] = np.concatenate([rng.random(4000).astype(np.float32),
                                 np.array([1.0, 0.5, 2 ** -24, 1 - 2 ** -24, 1e-30], np.float32)])
    f = rng.standard_normal(3000).astype(np.float32) * np.float32(100.0)
    small = (rng.random(500).astype(np.float32) - np.float32(.5)) * np.float32(2e-4)
    tiny = (rng.random(200).astype(np.float32) - np.float32(.5)) * np.float32(1e-7)
    special = np.array([0.0, -0.0, 65504.0, 65519.99, 65520.0, 1e6, -1e6, np.inf, -np.inf, 6.1035156e-05,
                        5.9604645e-08, 2.9802322e-08, 1.0009766, 1.0004883, 1.0014648, 0.33333334], np.float32)
    c["half_x"] = np.concatenate([f, small, tiny, special]).astype(np.float32)
    # transfer functions: the bench's two-peak TF, a ramp, and a random one
    from barney_gb300 import scenes
    c["tf_a"] = scenes.tf_two_peaks(256)
    c["tf_b"] = scenes.tf_ramp(128, 0.8)
    c["tf_c"] = rng.random((37, 4)).astype(np.float32)
    c["tf_s"] = ((rng.random(3000) * 1.4) - 0.2).astype(np.float32)
    lo = rng.random(2000).astype(np.float32) * np.float32(1.2) - np.float32(.1)
    hi = lo + rng.random(2000).astype(np.float32) * np.float32(.3) - np.float32(.02)
    c["tf_ranges"] = np.stack([lo, hi], axis=1).astype(np.float32)
    # a small structured field and points inside and around it
    vol = scenes.blob_volume((33, 29, 25), 6, seed=11, noise=0.05)
    c["vol"] = vol
    c["vol_origin"] = np.array([-0.5, -0.45, -0.4], np.float32)
    c["vol_spacing"] = np.array([1 / 32, 0.9 / 28, 0.8 / 24], np.float32)
    c["pts"] = ((rng.random((4000, 3)) * 1.3) - 0.65).astype(np.float32)
    # rays through the field (trace): origins on a sphere, aimed into the box
    n = 768
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    org = (2.5 * d).astype(np.float32)
    tgt = (rng.random((n, 3)) - 0.5) * 0.9
    dirs = (tgt - org)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    dirs = dirs.astype(np.float32)
    dirs[dirs == 0.0] = np.float32(1e-6)
    c["ray_org"], c["ray_dir"] = org, dirs
    c["ray_tmax"] = np.where(rng.random(n) < 0.8, np.float32(1e30), (rng.random(n) * 3 + 1.5)).astype(np.float32)
    c["ray_seed"] = rng.integers(0, 2 ** 63, size=n, dtype=np.uint64)
    c["trace_cpm"] = np.array([4], np.int32)
    c["rgba"] = np.concatenate([rng.random((1000, 4)).astype(np.float32) * np.float32(1.3),
                                np.array([[0.0031308, 0.0031309, 1.0, 0.0], [0.5, 0.999, 1.001, 1.0]],
                                         np.float32)])
    c.update(surface_cases())
    return c


def surface_cases(seed: int = 2025) -> dict:
    """Inputs of the iso-surface intersection program (the trace rays above
    against two iso values, three materials and instance indices) and of the
    AnariMatte Lambertian (random normals, view and light directions)."""
    rng = np.random.default_rng(seed)
    c = {}
    c["iso_cpm"] = np.array([4], np.int32)
    c["iso_values"] = np.array([0.25, 0.45], np.float32)
    c["iso_colors"] = np.array([[0.8, 0.8, 0.8, 1.0], [0.2, 0.7, 0.4, 1.0], [1.0, 0.5, 0.25, 0.9]], np.float32)
    c["iso_opacity"] = np.array([1.0, 1.0, 0.7], np.float32)
    c["iso_inst"] = np.array([0, 1, 3], np.int32)
    n = 2000
    unit = lambda v: (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    c["lam_Ng"] = unit(rng.standard_normal((n, 3)))
    c["lam_wo"] = unit(rng.standard_normal((n, 3)))
    c["lam_wi"] = unit(rng.standard_normal((n, 3)))
    c["lam_ab"] = rng.integers(0, 2 ** 32, size=(n, 2), dtype=np.uint64).astype(np.uint32)
    c["lam_color"] = rng.random((n, 4)).astype(np.float32)
    c["lam_color"][:, 3] = 1.0
    c["lam_Ng"][:3] = np.eye(3, dtype=np.float32)  # axis-aligned normals
    return c


def iso_ranges(c: dict) -> np.ndarray:
    """Macrocell scalar ranges of the trace field at the iso macrocell size,
    from the oracle's range build."""
    import oracle
    from barney_gb300 import scenes
    s = scenes.Scene(scalars=c["vol"], tf=c["tf_a"], base_density=40.0, cells_per_mc=int(c["iso_cpm"][0]))
    o = oracle.Oracle(s)
    o.rec.origin[:] = list(c["vol_origin"])
    o.rec.spacing[:] = list(c["vol_spacing"])
    return o.mc_ranges()


def trace_majorants(c: dict) -> np.ndarray:
    """Majorants of the trace field's macrocells, from the oracle's range build
    (the pinned majorant function is checked separately)."""
    import oracle
    from barney_gb300 import scenes
    s = scenes.Scene(scalars=c["vol"], tf=c["tf_a"], base_density=40.0, cells_per_mc=int(c["trace_cpm"][0]))
    o = oracle.Oracle(s)
    o.rec.origin[:] = list(c["vol_origin"])
    o.rec.spacing[:] = list(c["vol_spacing"])
    return o.majorants_of(o.mc_ranges())


def reference_outputs(c: dict) -> dict:
    from oracle import refpin as R
    out = {}
    out["rng_seq"] = np.stack([R.rng_sequence(int(a), int(b), 16) for a, b in c["rng_ab"]])
    seqs, states = [], []
    for u64 in (0, 1):
        for st, h in zip(c["seed_states"], c["seed_hashes"]):
            v, ns = R.rng_from_seed(int(st), int(h), bool(u64), 8)
            seqs.append(v)
            states.append(ns)
    out["rng_seed_seq"] = np.stack(seqs)
    out["rng_seed_state"] = np.array(states, np.uint64)
    out["rng_seeded"] = np.array([R.lib().ref_rng_seed_state(int(a), int(b)) for a, b in c["rng_ab"]], np.uint64)
    out["hash3"] = np.array([R.lib().ref_hash3(int(a), int(b), int(x)) for a, b, x in c["hash_abc"]], np.uint64)
    out["log"] = R.fast_log(c["log_x"])
    out["half"] = R.float_to_half(c["half_x"])
    out["half_all"] = R.half_to_float(np.arange(65536, dtype=np.uint32).astype(np.uint16)).view(np.uint32)
    for k, dom, bd in (("a", (0.0, 1.0), 50.0), ("b", (0.0, 1.0), 20.0), ("c", (0.15, 0.85), 3.5)):
        out[f"map_{k}"] = R.tf_map(c[f"tf_{k}"], dom, bd, c["tf_s"])
        out[f"maj_{k}"] = R.tf_majorant(c[f"tf_{k}"], dom, bd, c["tf_ranges"])
    out["sample"] = R.sample_points(c["vol"], c["vol_origin"], c["vol_spacing"], c["pts"])
    out["sample_map"] = R.sample_and_map(c["vol"], c["vol_origin"], c["vol_spacing"], c["tf_a"], (0.0, 1.0), 40.0,
                                         c["pts"])
    maj = trace_majorants(c)
    hits, ts, Ps, albs, states = [], [], [], [], []
    for o, d, tm, sd in zip(c["ray_org"], c["ray_dir"], c["ray_tmax"], c["ray_seed"]):
        h, t, P, a, ns = R.trace_ray(c["vol"], c["vol_origin"], c["vol_spacing"], int(c["trace_cpm"][0]), maj,
                                     c["tf_a"], (0.0, 1.0), 40.0, o, d, float(tm), int(sd))
        hits.append(h)
        ts.append(t if h else 0.0)
        Ps.append(P)
        albs.append(a)
        states.append(ns)
    out["trace_hit"] = np.array(hits, np.int32)
    out["trace_t"] = np.array(ts, np.float32)
    out["trace_P"] = np.stack(Ps).astype(np.float32)
    out["trace_albedo"] = np.stack(albs).astype(np.float32)
    out["trace_state"] = np.array(states, np.uint64)
    out["trace_majorants"] = maj
    out["rgba8"] = R.rgba8(c["rgba"], False)
    out["srgb8"] = R.rgba8(c["rgba"], True)
    out["mc_ranges_8"] = R.mc_ranges(c["vol"])
    rg = iso_ranges(c)
    out["iso_ranges"] = rg
    hit, st, t, P, Nh, alb = [], [], [], [], [], []
    for iv in c["iso_values"]:
        for m in range(c["iso_colors"].shape[0]):
            for o, d, tm, sd in zip(c["ray_org"], c["ray_dir"], c["ray_tmax"], c["ray_seed"]):
                h, ns, tt, PP, NN, aa = R.iso_hit(c["vol"], c["vol_origin"], c["vol_spacing"], int(c["iso_cpm"][0]),
                                                  rg, float(iv), c["iso_colors"][m], float(c["iso_opacity"][m]),
                                                  int(c["iso_inst"][m]), o, d, float(tm), int(sd))
                hit.append(h)
                st.append(ns)
                t.append(tt if h else 0.0)
                P.append(PP)
                Nh.append(NN)
                alb.append(aa)
    out["iso_hit"] = np.array(hit, np.int32)
    out["iso_state"] = np.array(st, np.uint64)
    out["iso_t"] = np.array(t, np.float32)
    out["iso_P"] = np.stack(P).astype(np.float32)
    out["iso_N"] = np.stack(Nh).astype(np.uint16)
    out["iso_albedo"] = np.stack(alb).astype(np.float32)
    out["lambertian"] = np.stack([R.lambertian(col, ng, wo, wi, int(a), int(b)) for col, ng, wo, wi, (a, b) in
                                  zip(c["lam_color"], c["lam_Ng"], c["lam_wo"], c["lam_wi"], c["lam_ab"])])
    return out


def main() -> None:
    from oracle import refpin
    if not refpin.available():
        raise SystemExit("the reference checkout is needed to build oracle/_ref (make -C oracle ref)")
    c = cases()
    out = reference_outputs(c)
    np.savez_compressed(OUT, **{f"in_{k}": v for k, v in c.items()}, **{f"out_{k}": v for k, v in out.items()})
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes): {int(out['trace_hit'].sum())} of {len(out['trace_hit'])} "
          f"rays hit the volume, {int(out['iso_hit'].sum())} of {len(out['iso_hit'])} the iso-surfaces")


if __name__ == "__main__":
    main()
