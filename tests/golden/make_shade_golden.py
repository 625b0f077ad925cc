"""Generates tests/golden/shade_pin.npz: the reference's per-pixel path steps
on fixed inputs -- ray generation and the shading step.

The outputs come from the reference renderer's code compiled unchanged
(oracle/refpin/ref_shade.cpp, built by `make -C oracle ref` into
oracle/_ref/libbarney_ref.so for the default build and
oracle/_ref/libbarney_ref_ms.so for the multi-scatter build):

* EnvMapLight's importance tables (EnvMap.cu:181-238) of two env maps under
  every address mode;
* PerspectiveCamera::commit (Camera.cu:83-97) and _generateRays
  (generateRays.cu:44-243) for random cameras, frame sizes and passes;
* bounce() (shadeRays.cu:477-878) of both builds on four worlds --
  directional light and ambient; env map and two directional lights; env
  map alone; ambient alone -- for random paths: misses, shadow rays, volume
  hits and matte-surface hits at path depths 0..10.

tests/test_oracle_refpin.py checks the CPU oracle against these vectors on
any machine, and against the live libraries where the reference checkout is.

  python tests/golden/make_shade_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "shade_pin.npz"
WORLDS = ("dir", "env+dir", "env", "ambient")
ADDRS = ((0, 1), (1, 1), (0, 0), (3, 3), (2, 1))
PATHS_PER_WORLD = 300


def env_textures() -> list:
    """The bench's sky map at 64x32 and a random 40x17 map."""
    from barney_gb300 import scenes
    sky = np.ascontiguousarray(scenes.env_sky(64, 32).texels, np.float32)
    rnd = (np.random.default_rng(31).random((17, 40, 4)) * 5).astype(np.float32)
    return [sky, rnd]


def env_frame() -> tuple:
    """toWorld and toLocal of the sky map's frame (EnvMap.cu:164-179), columns
    vx, vy, vz, as 9 floats each."""
    from barney_gb300 import scenes
    e = scenes.env_sky(64, 32)
    up, d = np.array(e.up, np.float64), np.array(e.direction, np.float64)
    vz = -up / np.linalg.norm(up)
    vy = -np.cross(vz, d)
    vy /= np.linalg.norm(vy)
    vx = np.cross(vy, vz)
    to_world = np.stack([vx, vy, vz])          # rows = columns vx, vy, vz
    to_local = np.linalg.inv(to_world.T).T     # the inverse, in the same layout
    return to_world.astype(np.float32).reshape(-1), to_local.astype(np.float32).reshape(-1), tuple(e.addr)


def make_world(kind: str, cdf_y=None, cdf_x=None, keep=None):
    """The orc_shade_world of one of WORLDS (deterministic lights); cdf_y and
    cdf_x: the sky map's importance tables for the env worlds."""
    import oracle
    rng = np.random.default_rng(101 + WORLDS.index(kind))
    w = oracle.OrcShadeWorld()
    w.ambient_radiance = 0.3
    nd = {"dir": 1, "env+dir": 2, "env": 0, "ambient": 0}[kind]
    w.num_dir_lights = nd
    for i in range(nd):
        d = rng.standard_normal(3)
        w.dir_light_dir[i][:] = list((d / np.linalg.norm(d)).astype(np.float32))
        w.dir_light_color[i][:] = list(rng.random(3).astype(np.float32))
        w.dir_light_radiance[i] = float(np.float32(1.0 + 2.0 * rng.random()))
    if kind.startswith("env"):
        tex = env_textures()[0]
        tw, tl, addr = env_frame()
        if keep is not None:
            keep += [tex, cdf_y, cdf_x]
        w.env_texels = tex.ctypes.data
        w.env_dims[:] = [tex.shape[1], tex.shape[0]]
        w.env_addr[:] = list(addr)
        w.env_to_world[:] = list(tw)
        w.env_to_local[:] = list(tl)
        w.env_scale = 1.0
        w.env_cdf_y = cdf_y.ctypes.data
        w.env_cdf_x = cdf_x.ctypes.data
    w.volume_multi_scatter = 1
    w.max_volume_bounces = 4
    return w


def make_paths(seed: int, n: int) -> np.ndarray:
    """n random orc_shade_path records (as bytes): origins, directions, seeds,
    misses / volume hits / surface hits, some shadow rays, random path state."""
    import oracle
    rng = np.random.default_rng(seed)
    recs = (oracle.OrcShadePath * n)()
    for p in recs:
        d = rng.standard_normal(3)
        p.org[:] = list((rng.random(3) * 4 - 2).astype(np.float32))
        p.dir[:] = list((d / np.linalg.norm(d)).astype(np.float32))
        p.hit = int(rng.integers(0, 3))
        p.tmax = float(np.float32(rng.random() * 3)) if p.hit else float(np.float32(1e30))
        p.seed = int(rng.integers(0, 2 ** 63, dtype=np.uint64))
        p.P[:] = list((rng.random(3) - .5).astype(np.float32))
        p.rgb[:] = list(rng.random(3).astype(np.float32))
        p.g = float(np.float32(rng.choice([0.0, 0.6, -0.3])))
        p.scattering_albedo = 0.9
        nn = rng.standard_normal(3)
        p.N[:] = list((nn / np.linalg.norm(nn)).astype(np.float32))
        p.color[:] = list(np.append(rng.random(3), 1.0).astype(np.float32))
        p.opacity = 1.0
        p.shadow = int(rng.random() < 0.15)
        p.tp[:] = [int(x) for x in np.float16(rng.random(3) * 2).view(np.uint16)]
        p.mis = float(np.float32(rng.random()))
        p.diffuse_bounces = int(rng.integers(0, 2))
        p.volume_bounces = int(rng.integers(0, 5))
        p.miss_color[:] = list(rng.random(4).astype(np.float32))
    return np.frombuffer(bytes(recs), np.uint8).copy()


def cases(seed: int = 2027) -> dict:
    rng = np.random.default_rng(seed)
    c = {"addrs": np.array(ADDRS, np.int32)}
    n = len(WORLDS) * 2 * PATHS_PER_WORLD
    c["paths"] = make_paths(seed + 1, n)
    c["depth"] = rng.integers(0, 11, size=n).astype(np.int32)
    c["world"] = np.repeat(np.arange(len(WORLDS), dtype=np.int32), 2 * PATHS_PER_WORLD)
    c["multi"] = np.tile(np.repeat(np.array([0, 1], np.int32), PATHS_PER_WORLD), len(WORLDS))
    c.update(camera_cases(seed + 2))
    return c


def camera_cases(seed: int, n: int = 12) -> dict:
    """Random cameras (position, direction, up, fovy), frame sizes up to
    24x20 (partial 32x32 tiles), passes (0, 1 and large accumIDs) and
    background colours (a constant, or w < 0: the gradient)."""
    rng = np.random.default_rng(seed)
    cam = np.concatenate([rng.standard_normal((n, 9)) * np.array([3] * 3 + [1] * 6),
                          20 + 80 * rng.random((n, 1))], axis=1).astype(np.float32)
    frame = np.stack([rng.integers(1, 25, n), rng.integers(1, 21, n), rng.choice([0, 1, 7, 123456], n)],
                     axis=1).astype(np.int32)
    bg = np.where(rng.random((n, 1)) < .5, np.array([[0.1, 0.2, 0.3, 1.0]]), np.array([[0, 0, 0, -1.0]]))
    return {"cam": cam, "frame": frame, "bg": bg.astype(np.float32)}


def run_cameras(c: dict, commit, generate) -> dict:
    """Camera commits and generated rays of every camera case with the
    given implementation (oracle or refpin functions)."""
    out = {"commit": [], "rays": [], "seeds": [], "bad": []}
    for cm, fr, bg in zip(c["cam"], c["frame"], c["bg"]):
        args = (cm[0:3], cm[3:6], cm[6:9], float(cm[9]))
        out["commit"].append(commit(*args))
        rays, seeds, bad = generate(*args, int(fr[0]), int(fr[1]), int(fr[2]), bg)
        out["rays"].append(rays.reshape(-1))
        out["seeds"].append(seeds.reshape(-1))
        out["bad"].append(bad)
    return {"commit": np.stack(out["commit"]), "rays": np.concatenate(out["rays"]),
            "seeds": np.concatenate(out["seeds"]), "gen_bad": np.array(out["bad"], np.int32)}


def summary(io, sh, frag) -> np.ndarray:
    """The compared results of one bounce as uint32 words: the path (origin,
    direction, tmax, seed, hit, throughput, MIS weight, bounce counts), the
    shadow ray (the same, zero when there is none) and the fragment."""
    def words(p, valid=True):
        if not valid:
            return [0] * 16
        f = lambda v: [int(x) for x in np.asarray(v, np.float32).view(np.uint32)]
        return (f(p.org[:]) + f(p.dir[:]) + f([p.tmax]) + [p.seed & 0xFFFFFFFF, p.seed >> 32, p.hit] +
                [int(t) for t in p.tp[:]] + f([p.mis]) + [p.diffuse_bounces, p.volume_bounces])
    return np.array(words(io) + words(sh, sh.tmax > 0) + [int(x) for x in np.asarray(frag, np.float32).view(np.uint32)],
                    np.uint32)


def run(c: dict, bounce, cdfs) -> np.ndarray:
    """summary() of every case with `bounce` (oracle.bounce or refpin.bounce)
    and the sky map's tables `cdfs`."""
    import oracle
    keep = []
    worlds = [make_world(k, cdfs[0], cdfs[1], keep) for k in WORLDS]
    recs = (oracle.OrcShadePath * len(c["depth"])).from_buffer_copy(c["paths"].tobytes())
    out = [summary(*bounce(worlds[int(wi)], bool(m), int(d), p))
           for p, d, wi, m in zip(recs, c["depth"], c["world"], c["multi"])]
    return np.stack(out)


def reference_outputs(c: dict) -> dict:
    from oracle import refpin as R
    out = {}
    tex = env_textures()
    for t, T in enumerate(tex):
        for a, addr in enumerate(c["addrs"]):
            cy, cx = R.env_cdfs(T, tuple(int(v) for v in addr))
            out[f"cdf_y_{t}_{a}"] = cy
            out[f"cdf_x_{t}_{a}"] = cx
    sky = (out["cdf_y_0_0"], out["cdf_x_0_0"])  # the sky map under (wrap, clamp), its address modes
    assert tuple(c["addrs"][0]) == env_frame()[2]
    out["bounce"] = run(c, R.bounce, sky)
    out.update(run_cameras(c, R.camera_commit, R.generate))
    return out


def main() -> None:
    from oracle import refpin
    if not refpin.available():
        raise SystemExit("the reference checkout is needed to build oracle/_ref (make -C oracle ref)")
    c = cases()
    out = reference_outputs(c)
    np.savez_compressed(OUT, **{f"in_{k}": v for k, v in c.items()}, **{f"out_{k}": v for k, v in out.items()})
    b = out["bounce"]
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes): {len(b)} bounces, {int((b[:, 22] != 0).sum())} shadow rays, "
          f"{int((b[:, 6] != np.float32(-1).view(np.uint32)).sum())} paths alive after the bounce")


if __name__ == "__main__":
    main()
