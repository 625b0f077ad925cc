"""Benchmark of the structured-volume frame on GB300.

Workload (the reference's headline metric): a 512^3 FP32 blob+fBm volume,
256-entry two-peak transfer function, 16^3-voxel macrocells, 1920x1080 at
64 spp, delta tracking with up to 4 isotropic volume bounces, one
directional light plus a 512x256 HDR sky env map.  One step = one full frame
(64 accumulation passes from a cleared frame buffer).  Inputs stay resident
in HBM for `value`; `e2e` goes through the barney-compatible bn* C-ABI with
host buffers (volume upload, macrocell and brick build, render, frame read).

  python bench.py [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank renders its own replica of the frame (replicas only:
the frame is one GPU's work; there is no data-path collective); `value` and
`e2e` take the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "Msamples/s & frame ms @512³ 1080p; fwd+adjoint ms/view; FP16 vs FP32 at RMSE"
UNIT = "Msamples/s"
BYTES_PER_VOXEL = {0: 4, 1: 2, 2: 2, 3: 1}
FMT_NAME = {0: "f32", 1: "f16", 2: "bf16", 3: "u8"}
WORKLOAD = ("512^3 blob+fBm volume, 256-entry two-peak TF, 16^3 macrocells, 1920x1080, 64 spp, "
            "<=4 isotropic volume bounces, dir light + 512x256 env map")


def bench_config(world: int, fmt: str = "f32") -> dict:
    """The workload description both arms print (identical dicts)."""
    return {"workload": WORKLOAD, "voxel_format": fmt,
            "l2": "inputs larger than L2 (512^3 FP32 volume: 0.5 GB; its brick store on the GPU: 4.3 GB)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def alg_bytes(samples, mcs, fmt):
    """Algorithmic bytes: 8 voxels per density sample, 4 B per macrocell
    entered, 8 B (scale, offset) per u8 sample."""
    b = samples * 8 * BYTES_PER_VOXEL[fmt] + 4 * mcs
    if fmt == 3:
        b += 8 * samples
    return b


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.f is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.f.flush()
        rows = [l.split(",") for l in Path(self.f.name).read_text().splitlines() if l.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _full_frame_passes(o, scene, threads, first_accum_id, target_s, max_passes):
    """Renders full 1-spp passes of the frame with the oracle (accumIDs
    first_accum_id, first_accum_id+1, ...) until target_s seconds or
    max_passes passes; returns (passes, density samples, seconds per pass)."""
    acc = np.zeros((scene.height, scene.width, 4), np.float32)
    times, samples = [], []
    while len(times) < max_passes and (not times or sum(times) < target_s):
        t0 = time.perf_counter()
        o.render(spp=1, accum=acc, accum_id_start=first_accum_id + len(times), nthreads=threads)
        times.append(time.perf_counter() - t0)
        samples.append(o.stats["density_samples"])
    return samples, times


def cpu_baseline(scene, majorants, target_s=10.0):
    """The oracle (FP32 restatement of the reference's CPU backend, one
    std::thread per host core) on full 1920x1080 frames at 1 spp (accumIDs
    1, 2, ...; accumID 0 has no pixel jitter), repeated for about target_s."""
    import oracle
    o = oracle.Oracle(scene, majorants=majorants)
    threads = os.cpu_count() or 1
    samples, times = _full_frame_passes(o, scene, threads, 1, target_s, 64)
    value = sum(samples) / sum(times) / 1e6
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(times)} full {scene.width}x{scene.height} passes at 1 spp (accumID 1..{len(times)}), "
                      f"{sum(samples)} density samples in {sum(times):.1f} s",
            "frame_ms_extrapolated": 1e3 * sum(times) / len(times) * scene.spp}


def run_reference(args):
    """The reference's CPU path (the oracle's restatement of the embree
    backend) on all host cores: one step = one full 1920x1080 pass at 1 spp
    of the 64-spp frame (accumID 1 + step)."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from barney_gb300 import scenes
    import oracle
    scene = scenes.frame_scene(dims=args.dims)
    o = oracle.Oracle(scene)
    threads = os.cpu_count() or 1
    samples, times = _full_frame_passes(o, scene, threads, 1, float("inf"), args.warmup + args.steps)
    samples, times = samples[args.warmup:], times[args.warmup:]
    value = sum(samples) / sum(times) / 1e6
    sample = (f"full {scene.width}x{scene.height} pass at 1 spp per step (accumID {1 + args.warmup}.."
              f"{args.warmup + args.steps}), {sum(samples) // len(samples)} density samples per step")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": bench_config(world, args.format), "sample": sample,
            "frame_ms_extrapolated": 1e3 * sum(times) / len(times) * scene.spp,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ea_timing(dims=128, nviews=32, size=256, reps=3):
    """Forward and forward+adjoint ms per view of the differentiable EA workload."""
    import torch
    from barney_gb300 import scenes
    from barney_gb300.ea import EAProblem
    gt = scenes.ea_scene(dims)
    views = scenes.fibonacci_views(nviews, 2.5, size)
    step = 0.5 / (dims - 1)
    tgt = EAProblem(gt, views, step).render()
    start = scenes.Scene(scalars=np.full_like(gt.scalars, 0.1), tf=gt.tf, base_density=gt.base_density)
    p = EAProblem(start, views, step)
    for _ in range(2):
        img = p.render()
        p.backward(img, 2 * (img - tgt))
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fw, fb = [], []
    for _ in range(reps):
        e[0].record()
        img = p.render()
        e[1].record()
        g = 2 * (img - tgt)
        p.backward(img, g)
        e[2].record()
        torch.cuda.synchronize()
        fw.append(e[0].elapsed_time(e[1]))
        fb.append(e[0].elapsed_time(e[2]))
    f, b = min(fw) / nviews, min(fb) / nviews
    return {"views": nviews, "view_px": f"{size}x{size}", "grid": f"{dims}^3", "fwd_ms_per_view": f,
            "fwd_adjoint_ms_per_view": b, "ratio": b / f}


def ea_steps(scene, view, step):
    """March steps of the EA views (pixel-centre rays, box test, n = ceil of
    the chord over the step), counted in float64 on the host."""
    W, H = view["width"], view["height"]
    pos = np.asarray(view["pos"], np.float64)
    d = np.asarray(view["dir"], np.float64)
    d = d / np.linalg.norm(d)
    up = np.asarray(view["up"], np.float64)
    du = np.cross(d, up)
    du /= np.linalg.norm(du)
    dv = np.cross(du, d)
    dv /= np.linalg.norm(dv)
    scale = 1.0 / (2.0 * math.tan(math.radians(view["fovy"]) / 2.0))
    u = ((np.arange(W) + 0.5) / W - 0.5) * (W / H)
    v = (np.arange(H) + 0.5) / H - 0.5
    dirs = d[None, None, :] * scale + u[None, :, None] * du + v[:, None, None] * dv
    dirs /= np.linalg.norm(dirs, axis=-1, keepdims=True)
    origin, spacing = scene.geometry()
    lo = np.asarray(origin, np.float64)
    hi = lo + np.asarray(spacing, np.float64) * (np.asarray(scene.dims, np.float64) - 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        a = (lo - pos) / dirs
        b = (hi - pos) / dirs
    t0 = np.maximum(np.nanmax(np.minimum(a, b), axis=-1), 0.0)
    t1 = np.nanmin(np.maximum(a, b), axis=-1)
    n = np.where(t1 > t0, np.ceil((t1 - t0) / step), 0.0)
    return int(n.sum())


def _bias(d):
    """Mean signed error over the crop and its standard error from the
    per-row means (rows as independent batches): a storage format that
    shifts the image shows a bias several sigma from zero, while paths that
    part (a flipped decision changes the rest of a path) average out."""
    per_row = d.reshape(d.shape[0], -1).mean(axis=1)
    return {"bias_vs_fp64": float(d.mean()), "bias_sigma": float(per_row.std(ddof=1) / math.sqrt(per_row.size))}


def precision_study(scene, g32, rows=(523, 557), reps=2):
    """Voxel storage precision, two ways.

    ea: the fixed-step emission-absorption march (deterministic) of the
    512^3 volume through the frame's camera, per format: samples/s at
    1920x1080 and the error of a 240x135 view against the oracle's FP64 march
    of the FP32 source voxels.  `linear_f32` is the plain form (the
    reference's x-fastest FP32 texels).

    delta_tracking: each format's full frame (samples/s, frame ms) and its
    error on a band of rows against the oracle's FP64 render from the FP32
    source voxels.  All formats and the oracle use the FP32 source's majorant
    grid, so every pixel draws the same random numbers, and the shading
    streams hash the hit distance truncated to an integer, so a small
    difference in a distance keeps the path's streams; only a decision that
    flips between precisions changes the rest of that path.
    `oracle_fp32_vs_fp64` is the floor of the FP32 arithmetic itself;
    `rmse_vs_f32` (the same store layout and streams, FP32 voxels against
    the format's) isolates the storage, and `bias_vs_fp64` with `bias_sigma`
    (the mean signed error over the crop and its standard error) tests for a
    systematic shift."""
    import torch
    import oracle
    from barney_gb300 import _native as N
    from barney_gb300.device import GpuScene
    from barney_gb300.ea import EAProblem
    maj = g32.majorants.cpu().numpy()
    o = oracle.Oracle(scene, majorants=maj)
    threads = os.cpu_count() or 1
    H, W, spp = scene.height, scene.width, scene.spp
    out = {"delta_tracking": {}, "ea": {}}
    # ---- EA march ----
    step = 0.5 / (scene.dims[0] - 1)
    cam = dict(pos=tuple(scene.cam_pos), dir=tuple(scene.cam_dir), up=tuple(scene.cam_up), fovy=scene.fovy)
    big = dict(cam, width=W, height=H)
    small = dict(cam, width=240, height=135)
    t0 = time.perf_counter()
    ea64 = o.ea_render([small], step, use_double=True, nthreads=threads)
    out["ea"] = {"step": "0.5 voxel", "timed_view": f"{W}x{H}", "error_view": "240x135 (same camera)",
                 "oracle_fp64_s": time.perf_counter() - t0, "samples_per_view": ea_steps(scene, big, step),
                 "formats": {}}
    nsamp = out["ea"]["samples_per_view"]
    stores = [("linear_f32", None)] + [(name, fmt) for fmt, name in FMT_NAME.items()]
    for name, fmt in stores:
        g = None if fmt is None else (g32 if fmt == 0 else GpuScene(scene, fmt=fmt, scalars_device=g32.scalars))
        pb = EAProblem(scene, [big], step, scalars=g32.scalars, store=g)
        ps = EAProblem(scene, [small], step, scalars=g32.scalars, store=g)
        pb.render()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            pb.render()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        d = ps.render().cpu().numpy() - ea64
        out["ea"]["formats"][name] = {"Msamples_s": nsamp / (ms / 1e3) / 1e6, "ms": ms,
                                      "rmse_vs_fp64": float(np.sqrt(np.mean(d ** 2))),
                                      "max_err_vs_fp64": float(np.abs(d).max())}
        if fmt not in (None, 0):
            del g
        del pb, ps
        torch.cuda.empty_cache()
    base = out["ea"]["formats"]["linear_f32"]["Msamples_s"]
    for v in out["ea"]["formats"].values():
        v["vs_linear_f32"] = v["Msamples_s"] / base
    # ---- delta tracking ----
    t0 = time.perf_counter()
    ref64 = o.render(spp=spp, use_double=True, nthreads=threads, rows=rows)[rows[0]:rows[1], :, :3] / spp
    t64 = time.perf_counter() - t0
    ref32 = o.render(spp=spp, use_double=False, nthreads=threads, rows=rows)[rows[0]:rows[1], :, :3] / spp
    dt = out["delta_tracking"]
    dt.update({"crop": f"rows {rows[0]}-{rows[1]} x {W} columns ({(rows[1] - rows[0]) * W} pixels), {spp} spp",
               "majorants": "FP32 source majorant grid for every format", "oracle_fp64_s": t64,
               "oracle_fp32_vs_fp64": dict({"rmse": float(np.sqrt(np.mean((ref32 - ref64) ** 2))),
                                            "max_err": float(np.abs(ref32 - ref64).max())}, **_bias(ref32 - ref64)),
               "formats": {}})
    cnt = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    img32 = None
    for fmt, name in FMT_NAME.items():
        g = g32 if fmt == 0 else GpuScene(scene, fmt=fmt, scalars_device=g32.scalars)
        if fmt != 0:
            g.majorants.copy_(g32.majorants)
        acc = g.new_accum()
        cnt.zero_()
        g.render(spp=spp, accum=acc, counters=cnt)
        torch.cuda.synchronize()
        samples = int(cnt[0].item())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            g.render(spp=spp, accum=acc)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        full = acc.cpu().numpy()
        img = full[rows[0]:rows[1], :, :3] / spp
        d = img - ref64
        rec = {"Msamples_s": samples / (ms / 1e3) / 1e6, "frame_ms": ms, "store_GB": g.voxels.numel() / 1e9,
               "rmse_vs_fp64": float(np.sqrt(np.mean(d ** 2))), "max_err_vs_fp64": float(np.abs(d).max())}
        rec.update(_bias(d))
        if img32 is None:
            img32 = full
        else:
            rec["pixels_identical_to_f32"] = float(np.mean(np.all(full == img32, axis=-1)))
            d32 = img - img32[rows[0]:rows[1], :, :3] / spp
            rec["rmse_vs_f32"] = float(np.sqrt(np.mean(d32 ** 2)))
        dt["formats"][name] = rec
        if fmt != 0:
            del g
        del acc
        torch.cuda.empty_cache()
    f32 = dt["formats"]["f32"]["Msamples_s"]
    for v in dt["formats"].values():
        v["vs_f32"] = v["Msamples_s"] / f32
    return out


def wavefront_timing(g, scene, persistent_ms, reps=3):
    """The same frame in the wavefront mode (a trace kernel over a ray queue
    and a shade kernel over the active pixels per step, path state in HBM)
    against the persistent kernel's time: an A/B of the two structures; the
    frames are identical."""
    import torch
    from barney_gb300 import _native as N
    acc = g.new_accum()
    cfg = {"mode": N.GBV_RENDER_WAVEFRONT}
    g.render(spp=scene.spp, accum=acc, config=cfg)
    ref = g.new_accum()
    g.render(spp=scene.spp, accum=ref)
    torch.cuda.synchronize()
    identical = bool(torch.equal(acc, ref))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ts = []
    for _ in range(reps):
        e0.record()
        g.render(spp=scene.spp, accum=acc, config=cfg)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    ms = min(ts)
    return {"frame_ms": ms, "persistent_frame_ms": persistent_ms, "vs_persistent": persistent_ms / ms,
            "frames_identical": identical}


def iso_timing(g, scene, persistent_ms, reps=2):
    """The frame with an iso-surface of the field (value 0.5, matte
    material 0.8 grey): beside the volume in one group (the iso-surface's
    instance first), and alone; frame times and rays per second (event
    counts of one counted frame each)."""
    import torch
    from barney_gb300 import _native as N, scenes
    out = {"iso_value": 0.5, "volume_only_frame_ms": persistent_ms}
    saved = (scene.iso, scene.volume_instance, scene.no_volume)
    try:
        for name, (vi, nv) in {"iso_and_volume": (1, False), "iso_only": (0, True)}.items():
            scene.iso = scenes.IsoSurface(0.5, (0.8, 0.8, 0.8, 1.0), 1.0, 0)
            scene.volume_instance, scene.no_volume = vi, nv
            acc = g.new_accum()
            cnt = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
            g.render(spp=scene.spp, accum=acc, counters=cnt)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ts = []
            for _ in range(reps):
                e0.record()
                g.render(spp=scene.spp, accum=acc)
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            c = [int(x) for x in cnt.cpu().tolist()]
            ms = min(ts)
            out[name] = {"frame_ms": ms, "rays": c[N.GBV_COUNTER_RAYS], "Mrays_s": c[N.GBV_COUNTER_RAYS] / ms / 1e3,
                         "density_samples": c[N.GBV_COUNTER_SAMPLES], "loop_caps": c[N.GBV_COUNTER_CAPS]}
    finally:
        scene.iso, scene.volume_instance, scene.no_volume = saved
    return out


def nanovdb_timing(scene, persistent_ms, reps=2, types=("float", "fp16", "fp8", "fp4", "fpn")):
    """The frame with its volume given as a NanoVDB grid (voxel centres where
    the structured field has its voxels; the grid made by the input
    generator), of each value type the NanoVDB field reads (FpN with the
    builder's default tolerance for a fog volume, 0.01): grid bytes, frame
    time and density samples per second against the FP32 brick store's
    frame.  The Float grid's figures stay at the top level."""
    import torch
    from barney_gb300 import _native as N, scenes
    from barney_gb300.nanovdb import GpuNanoVDBScene
    out = {"brick_f32_frame_ms": persistent_ms, "types": {}}
    for t in types:
        t0 = time.perf_counter()
        grid = scenes.nanovdb_of_scene(scene, grid_type=t)
        make_s = time.perf_counter() - t0
        g = GpuNanoVDBScene(scene, grid)
        acc = g.new_accum()
        cnt = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
        g.render(accum=acc, counters=cnt)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ts = []
        for _ in range(reps):
            e0.record()
            g.render(accum=acc)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        c = [int(x) for x in cnt.cpu().tolist()]
        ms = min(ts)
        r = {"grid_bytes": len(grid), "grid_make_s": make_s, "frame_ms": ms,
             "density_samples": c[N.GBV_COUNTER_SAMPLES], "Msamples_s": c[N.GBV_COUNTER_SAMPLES] / ms / 1e3,
             "loop_caps": c[N.GBV_COUNTER_CAPS]}
        if t == "float":
            out.update(r)
        else:
            out["types"][t] = r
        del g, grid
        torch.cuda.empty_cache()
    return out


def tiles_timing(g, scene, persistent_ms, worlds=(2, 4, 8)):
    """The frame partition of a multi-GPU frame measured on one GPU: for N
    ranks, each rank's share of the frame (the 32x32 tiles it owns,
    gbv_render_tiles) timed alone -- the slowest share is the frame time N
    GPUs would take, the sum the partition's overhead against the whole
    frame -- and the compressed tile codec of the gather (gbv_compress_tiles
    / gbv_unpack_tiles, 6144 bytes per tile) over the whole 1080p frame."""
    import torch
    from barney_gb300 import _native as N, tiles as T
    out = {"full_frame_ms": persistent_ms, "ranks": {}}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    acc = g.new_accum()
    for world in worlds:
        ms = []
        for rank in range(world):
            g.render_tiles(rank, world, accum=acc)  # warm
            e0.record()
            g.render_tiles(rank, world, accum=acc)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        out["ranks"][str(world)] = {"max_rank_ms": max(ms), "sum_ms": sum(ms),
                                    "speedup_vs_full": persistent_ms / max(ms)}
    g.render(accum=acc)
    torch.cuda.synchronize()
    tiles = T.compress_tiles(acc, scene.spp, 0, 1)
    frame = torch.zeros_like(acc)
    for _ in range(2):
        T.compress_tiles(acc, scene.spp, 0, 1)
        T.unpack_tiles_into(frame, tiles, 0, 1)
    torch.cuda.synchronize()
    e0.record()
    tiles = T.compress_tiles(acc, scene.spp, 0, 1)
    e1.record()
    torch.cuda.synchronize()
    enc = e0.elapsed_time(e1)
    e0.record()
    T.unpack_tiles_into(frame, tiles, 0, 1)
    e1.record()
    torch.cuda.synchronize()
    dec = e0.elapsed_time(e1)
    nb = tiles.numel()
    out["codec"] = {"tiles": int(tiles.shape[0]), "compressed_bytes": int(nb), "accum_bytes": int(acc.numel() * 4),
                    "encode_ms": enc, "decode_ms": dec,
                    "encode_GBps": (acc.numel() * 4 + nb) / enc / 1e6, "decode_GBps": (nb + acc.numel() * 4) / dec / 1e6}
    return out


def batch_timing(count=64, reps=3):
    """The batched uneven workload: `count` volumes (sides log-uniform in
    [32, 256] per axis), each with its own TF, camera and image size from
    {128^2, 256^2, 512^2}, 8 spp; one persistent launch replayed from a CUDA
    graph against one gbv_render launch per item on the same stream."""
    import torch
    from barney_gb300 import _native as N, scenes
    from barney_gb300.batch import GpuBatch
    from barney_gb300.autotune import tuned_batch
    items = scenes.batch_items(count)
    spp = items[0].spp
    b, tuned = tuned_batch(items, spp)
    cnt = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    b.render(spp, counters=cnt)
    torch.cuda.synchronize()
    samples = int(cnt[0].item())
    graph = b.capture(spp)
    stream = torch.cuda.current_stream()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    e[0].record(stream)
    for _ in range(reps):
        graph.replay()
    e[1].record(stream)
    torch.cuda.synchronize()
    batched = [a.clone() for a in b.accums]
    for _ in range(2):
        for g, a in zip(b.items, b.accums):
            g.render(spp=spp, accum=a)
    torch.cuda.synchronize()
    e[2].record(stream)
    for _ in range(reps):
        for g, a in zip(b.items, b.accums):
            g.render(spp=spp, accum=a)
    e[3].record(stream)
    torch.cuda.synchronize()
    identical = all(torch.equal(x, y) for x, y in zip(batched, b.accums))
    ms_b = e[0].elapsed_time(e[1]) / reps
    ms_s = e[2].elapsed_time(e[3]) / reps
    out = {"items": count, "spp": spp, "pixels": sum(s.width * s.height for s in items),
           "voxels": int(sum(s.scalars.size for s in items)), "density_samples": samples,
           "batch_graph_ms": ms_b, "separate_launches_ms": ms_s, "speedup": ms_s / ms_b,
           "batch_Msamples_s": samples / (ms_b / 1e3) / 1e6, "images_identical": identical}
    out["tuned"] = {"brick_log2": list(tuned["brick"]), "launch_blocks_threshold_skip": list(tuned["launch"]),
                    "cached": tuned["cached"], "brick_ms": tuned.get("brick_ms")}
    b.close()
    return out


def run_ours(args):
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from barney_gb300 import _native as N, scenes
    from barney_gb300.device import GpuScene

    fmt = {"f32": 0, "f16": 1, "bf16": 2, "u8": 3}[args.format]
    scene = scenes.frame_scene(dims=args.dims)
    g = GpuScene(scene, layout=N.GBV_LAYOUT_BRICK_CORNERS, fmt=fmt)
    counters = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    acc = g.new_accum()
    stream = torch.cuda.current_stream()

    def frame(cnt=None):
        g.render(spp=scene.spp, accum=acc, accum_id_start=0, counters=cnt)

    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    counters.zero_()
    frame(counters)  # counts of one frame (the frame is deterministic)
    torch.cuda.synchronize()
    cnt = counters.cpu().tolist()
    samples, mcs, rays, caps = cnt[:4]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        t_all0 = time.perf_counter()
        for i in range(args.steps):
            starts[i].record(stream)
            frame()
            ends[i].record(stream)
        torch.cuda.synchronize()
        t_all = time.perf_counter() - t_all0
    if world > 1:
        dist.barrier()
    ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(ms)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    frame_ms = total_ms / args.steps
    value = world * samples * args.steps / (total_ms / 1e3) / 1e6
    peak, peak_kind = peaks()
    bytes_launch = alg_bytes(samples, mcs, fmt)
    achieved = bytes_launch / (frame_ms / 1e3) / 1e9
    traffic = None
    tf_path = ROOT / "profiles" / "render_traffic.json"
    if tf_path.exists():
        t = json.loads(tf_path.read_text())
        # scale the captured launch's DRAM bytes by density samples processed
        if t.get("format") == args.format and t.get("samples"):
            traffic = t["dram_bytes"] * samples / t["samples"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": frame_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(world, args.format),
            "voxel_store": "8^3-cell brick corners, %.2f GB" % (g.voxels.numel() / 1e9),
            "frame_ms": frame_ms, "density_samples_per_frame": samples, "macrocells_per_frame": mcs,
            "rays_per_frame": rays, "loop_caps": caps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6800 GB/s",
                         "bytes_per_launch": bytes_launch, "kernel": "render_kernel"},
            # per frame: the majorant-bitmask kernel, then the render kernel
            # (profiles/launches_bench_512cube_1080p_64spp.md)
            "gpu_launches": 2 * args.steps, "clocks": clk.summary()}
    # ---- e2e through the bn* C-ABI with host buffers, on every rank; the
    # slowest rank's step time counts ----
    if world > 1:
        dist.barrier()
    e2e = e2e_timing(args, scene, g, acc, fmt, local)
    if world > 1:
        t = torch.tensor([e2e["dt"]], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e["dt"] = float(t.item())
    line["e2e"] = {"value": world * samples / e2e["dt"] / 1e6, "unit": UNIT, "h2d_bytes_per_step": e2e["h2d"],
                   "d2h_bytes_per_step": e2e["d2h"], "ms_per_step": 1e3 * e2e["dt"],
                   "path": "bnTextureData3DCreate(host) .. bnRender .. bnFrameBufferRead(host), pinned buffers",
                   "frame_identical_to_device_frame": e2e["same"], "phases_ms": e2e["phases_ms"],
                   "host_cpus": e2e["host_cpus"]}
    if rank != 0:
        if world > 1:
            dist.barrier()
        return
    # ---- extras on rank 0 ----
    extras_t0 = time.perf_counter()
    if not args.quick:
        # voxel storage formats against the FP64 oracle
        try:
            line["precision"] = precision_study(scene, g)
        except Exception as e:  # report, never hide
            line["precision"] = {"error": repr(e)}
        try:
            line["batch"] = batch_timing()
        except Exception as e:
            line["batch"] = {"error": str(e)}
        try:
            line["ea_adjoint"] = ea_timing()
        except Exception as e:
            line["ea_adjoint"] = {"error": str(e)}
        try:
            line["wavefront"] = wavefront_timing(g, scene, frame_ms)
        except Exception as e:
            line["wavefront"] = {"error": str(e)}
        try:
            line["iso_surface"] = iso_timing(g, scene, frame_ms)
        except Exception as e:
            line["iso_surface"] = {"error": str(e)}
        try:
            line["nanovdb"] = nanovdb_timing(scene, frame_ms)
        except Exception as e:
            line["nanovdb"] = {"error": str(e)}
        try:
            line["tiles"] = tiles_timing(g, scene, frame_ms)
        except Exception as e:
            line["tiles"] = {"error": str(e)}
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(scene, g.majorants.cpu().numpy())
    line["extras_s"] = time.perf_counter() - extras_t0
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()


def bind_to_gpu_numa_node(local: int) -> str:
    """Runs this process on the CPUs attached to GPU `local` (its PCI
    device's local_cpulist in sysfs), as numactl --cpunodebind would, so that
    host buffers pinned afterwards are first touched in the GPU's own host
    memory; returns the CPU list, or why it was left as it was."""
    try:
        import torch
        pr = torch.cuda.get_device_properties(local)
        dev = "%04x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
        text = Path("/sys/bus/pci/devices/%s/local_cpulist" % dev).read_text().strip()
        cpus = set()
        for part in text.split(","):
            lo, _, hi = part.partition("-")
            cpus.update(range(int(lo), int(hi or lo) + 1))
        if not cpus or cpus == set(range(os.cpu_count() or 0)):
            return "all CPUs are local"
        os.sched_setaffinity(0, cpus)
        return text
    except Exception as e:  # no sysfs entry, no permission: leave the process where it is
        return "not bound: %s" % e


def e2e_timing(args, scene, g, acc, fmt, local):
    """Steps through the public bn* API with host buffers: each uploads the
    volume from pinned host memory (bnTextureData3DCreate), builds the
    scene, renders the frame (bnRender) and reads it into pinned host memory
    (bnFrameBufferRead); one untimed step first.  Returns the mean step
    time, its three phases, the bytes copied each way, and whether the frame
    read equals the device-timed frame `acc`."""
    import torch
    from barney_gb300 import bn
    before = os.sched_getaffinity(0)
    cpus = bind_to_gpu_numa_node(local)
    host_vol = torch.from_numpy(np.ascontiguousarray(scene.scalars)).pin_memory()
    out = torch.empty((scene.height, scene.width, 4), dtype=torch.float32).pin_memory()
    e2e_times, phases = [], []
    with bn.BarneySession(local) as ses:
        for i in range(1 + args.e2e_steps):
            t0 = time.perf_counter()
            ses.build_scene(scene, host_vol.data_ptr(), voxel_format=fmt)
            t1 = time.perf_counter()
            ses.render()
            t2 = time.perf_counter()
            ses.read(out)
            dt = time.perf_counter() - t0
            ses.release_scene()
            if i > 0:
                e2e_times.append(dt)
                # the bn* calls return when their work is done (each upload
                # and build synchronizes, bnRender waits for its frame)
                phases.append((t1 - t0, t2 - t1, t0 + dt - t2))
    os.sched_setaffinity(0, before)  # the CPU baseline afterwards uses every core
    ph = [1e3 * sum(p[k] for p in phases) / len(phases) for k in range(3)]
    # the bn* frame is the device frame read out: same samples, same pixels
    same = bool(torch.equal(out.cuda(), g.tonemap(acc, scene.spp)))
    h2d = host_vol.numel() * 4 + scene.tf.nbytes + (scene.env.texels.nbytes if scene.env is not None else 0)
    return {"dt": sum(e2e_times) / len(e2e_times), "h2d": int(h2d), "d2h": int(out.numel() * 4), "same": same,
            "phases_ms": {"upload_and_build": ph[0], "render": ph[1], "read": ph[2]}, "host_cpus": cpus}


def profile_render_case(args):
    """Small, self-contained render launches for ncu captures: the frame
    scene (--dims, --width, --height, --spp, --format, --layout), --warmup
    untimed launches, then --launches launches as timed runs make them (no
    event counting), then one counted launch whose counters go to --out, so
    that ncu's DRAM bytes of the uncounted launches can be related to
    density samples (the frame is deterministic).  Capture the uncounted
    launches with
      ncu --clock-control none -k regex:render_kernel -s <warmup> -c <launches> ...
    With --mode wavefront a frame is a sequence of wf_trace_kernel and
    wf_shade_kernel launches (one of each per step).  Count=0 in the trace
    kernel's template arguments marks the uncounted frames.  --iso V adds the
    iso-surface of value V (matte, its instance first); --iso-only renders
    the surface alone (the kernel's last template argument is then 1)."""
    import torch
    from barney_gb300 import _native as N, scenes
    from barney_gb300.device import GpuScene
    s = scenes.frame_scene(dims=args.dims, width=args.width, height=args.height, spp=args.spp)
    if args.iso is not None:
        s.iso = scenes.IsoSurface(args.iso, (0.8, 0.8, 0.8, 1.0), 1.0, 0)
        s.volume_instance, s.no_volume = (0, True) if args.iso_only else (1, False)
    fmt = {"f32": 0, "f16": 1, "bf16": 2, "u8": 3}[args.format]
    layout = N.GBV_LAYOUT_BRICK_CORNERS if args.layout == "brick" else N.GBV_LAYOUT_LINEAR
    g = GpuScene(s, layout=layout, fmt=fmt)
    acc = g.new_accum()
    cfg = {"mode": N.GBV_RENDER_WAVEFRONT} if args.mode == "wavefront" else None
    for _ in range(args.warmup + args.launches):
        g.render(accum=acc, config=cfg)
    cnt = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    g.render(accum=acc, counters=cnt, config=cfg)
    torch.cuda.synchronize()
    c = [int(x) for x in cnt.cpu().tolist()]
    rec = dict(dims=args.dims, width=args.width, height=args.height, spp=args.spp, format=args.format,
               layout=args.layout, mode=args.mode, iso=args.iso, iso_only=bool(args.iso_only),
               samples_per_launch=c[0], mc_visits_per_launch=c[1], rays_per_launch=c[2])
    if args.out:
        Path(args.out).parent.mkdir(parents=True, exist_ok=True)
        Path(args.out).write_text(json.dumps(rec, indent=1))
    print(json.dumps(rec))


def profile_ea_case(args):
    """EA launches for ncu captures: the differentiable emission-absorption
    workload (--dims^3 density grid, 256-entry TF, --views views of --size^2
    on a sphere of radius 2.5, step 0.5 voxel): --warmup forward+adjoint
    passes, then --launches more.  Capture the forward with
    -k regex:ea_forward and the adjoint with -k regex:ea_backward, skipping
    the warm-up launches (-s <warmup>), with --clock-control none."""
    import torch
    from barney_gb300 import scenes
    from barney_gb300.ea import EAProblem
    gt = scenes.ea_scene(args.dims)
    views = scenes.fibonacci_views(args.views, 2.5, args.size)
    step = 0.5 / (args.dims - 1)
    tgt = EAProblem(gt, views, step).render()
    start = scenes.Scene(scalars=np.full_like(gt.scalars, 0.1), tf=gt.tf, base_density=gt.base_density)
    p = EAProblem(start, views, step)
    for _ in range(args.warmup + args.launches):
        img = p.render()
        p.backward(img, 2 * (img - tgt))
    torch.cuda.synchronize()
    print("ok")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--format", default="f32", choices=["f32", "f16", "bf16", "u8"])
    ap.add_argument("--dims", type=int, default=None, help="volume edge (default 512; 128 for --profile-case ea)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--quick", action="store_true", help="skip the FP16 and adjoint extras")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--profile-case", choices=["render", "ea"],
                    help="small launches for an ncu capture instead of the benchmark")
    ap.add_argument("--width", type=int, default=480, help="--profile-case render: frame width")
    ap.add_argument("--height", type=int, default=270, help="--profile-case render: frame height")
    ap.add_argument("--spp", type=int, default=1, help="--profile-case render: passes per launch")
    ap.add_argument("--layout", default="brick", choices=["brick", "linear"], help="--profile-case render")
    ap.add_argument("--mode", default="persistent", choices=["persistent", "wavefront"],
                    help="--profile-case render: the persistent kernel, or the trace/shade kernels per step "
                         "(a frame is then many launches of each)")
    ap.add_argument("--launches", type=int, default=1, help="--profile-case: launches after the warm-up")
    ap.add_argument("--views", type=int, default=32, help="--profile-case ea: views")
    ap.add_argument("--size", type=int, default=256, help="--profile-case ea: view edge in pixels")
    ap.add_argument("--out", default="", help="--profile-case render: counters JSON")
    ap.add_argument("--iso", type=float, default=None, help="--profile-case render: an iso-surface of this value")
    ap.add_argument("--iso-only", action="store_true", help="--profile-case render: the iso-surface alone")
    args = ap.parse_args()
    if args.dims is None:
        args.dims = 128 if args.profile_case == "ea" else 512
    if args.profile_case:
        import torch
        torch.cuda.set_device(0)
        if args.profile_case == "render":
            profile_render_case(args)
        else:
            profile_ea_case(args)
        return
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
