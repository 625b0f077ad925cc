"""Autotuner for the batched persistent render launch.

The batched launch has knobs that change its speed but never its images
(every lane still renders its own pixels in the reference's accumulation
order, and every brick shape stores the same cells; tests/test_gpu_batch.py
and tests/test_gpu_bricks.py check both bit for bit):

* brick         -- log2 of the brick edge in cells per axis of the voxel
  stores (where neighbouring cells sit in HBM);
* blocks_per_sm -- resident 288-thread blocks per SM (4, 5 or 6: the kernel
  is compiled for each register budget);
* threshold     -- a warp keeps traversing while at least this percentage of
  its busy lanes still traces, then shades together;
* skip          -- cell tests and distance draws a lane may make per traversal
  iteration to reach its next sample position.

tune_batch() times launch shapes of an existing batch; tuned_batch() also
rebuilds the stores with each candidate brick shape (coordinate descent:
launch shape at 8^3 bricks, then brick shape at that launch shape, then the
launch shape again at the chosen bricks).  Every timing is CUDA events on the
launching stream.  Choices are cached in a JSON file keyed by the GPU and a
signature of the workload, so a later process with the same workload applies
them without timing.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

LAUNCH_CANDIDATES = [(b, t, k) for b in (4, 5, 6) for t in (5, 12, 20) for k in (4, 6, 8)]
# What a launch shape means to the kernel (block size, traversal units); part
# of every cache key, so choices cached by a build where the same numbers
# meant another launch are not reused.
LAUNCH_SHAPE_REVISION = "288-thread blocks, seek units"
BRICK_CANDIDATES = [(3, 3, 3), (2, 2, 2), (4, 4, 4), (4, 4, 2), (5, 3, 2)]


def cache_path() -> Path:
    p = os.environ.get("GBV_AUTOTUNE_CACHE")
    if p:
        return Path(p)
    return Path(os.path.expanduser("~")) / ".cache" / "barney_gb300" / "autotune.json"


def workload_key(scenes, spp: int, fmt: int, what: str) -> str:
    """Launch-shape revision, GPU name and SM count, plus the items' frame
    sizes, field sizes, macrocell sizes, scattering mode, voxel format and
    passes."""
    import torch
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    items = [(s.width, s.height, list(s.scalars.shape), s.cells_per_mc, s.multi_scatter) for s in scenes]
    blob = json.dumps([LAUNCH_SHAPE_REVISION, what, props.name, props.multi_processor_count, spp, fmt, items])
    return what + ":" + hashlib.sha1(blob.encode()).hexdigest()[:20]


def _load(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def _store(path: Path, key: str, rec: dict) -> None:
    d = _load(path)
    d[key] = rec
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp%d" % os.getpid())
        tmp.write_text(json.dumps(d, indent=1))
        tmp.replace(path)
    except OSError:
        pass  # a read-only home only costs the re-tuning


def time_launch(batch, spp: int, shape, reps: int = 2) -> float:
    """Milliseconds of one batch render with launch shape `shape`."""
    import torch
    batch.set_launch(*shape)
    stream = torch.cuda.current_stream()
    batch.render(spp)  # warm
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        batch.render(spp)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _fastest(timed: dict):
    best = min(timed, key=timed.get)
    return tuple(int(x) for x in best.split(",")), timed[best]


def tune_batch(batch, spp: int, candidates=None, reps: int = 2, use_cache: bool = True) -> dict:
    """Picks the fastest launch shape for `batch` at `spp` passes, applies it
    with set_launch and returns {"launch": (blocks_per_sm, threshold, skip),
    "ms": ..., "timed": {...}, "cached": bool}."""
    cands = [tuple(c) for c in (candidates or LAUNCH_CANDIDATES)]
    path = cache_path()
    key = workload_key(batch.scenes, spp, batch.fmt, "launch%d%d%d" % batch.brick)
    if use_cache:
        rec = _load(path).get(key)
        if rec and tuple(rec["launch"]) in cands:
            batch.set_launch(*rec["launch"])
            return dict(rec, launch=tuple(rec["launch"]), cached=True)
    timed = {",".join(map(str, c)): time_launch(batch, spp, c, reps) for c in cands}
    shape, ms = _fastest(timed)
    batch.set_launch(*shape)
    rec = {"launch": list(shape), "ms": ms, "timed": timed}
    if use_cache:
        _store(path, key, rec)
    return dict(rec, launch=shape, cached=False)


def tuned_batch(scenes, spp: int, fmt: int = 0, bricks=None, reps: int = 2, use_cache: bool = True):
    """Builds the batch of `scenes` with the fastest brick shape and launch
    shape; returns (GpuBatch, record)."""
    from .batch import GpuBatch
    bricks = [tuple(b) for b in (bricks or BRICK_CANDIDATES)]
    path = cache_path()
    key = workload_key(scenes, spp, fmt, "brick")
    rec = _load(path).get(key) if use_cache else None
    if rec and tuple(rec["brick"]) in bricks:
        b = GpuBatch(scenes, fmt=fmt, brick=rec["brick"])
        launch = tune_batch(b, spp, reps=reps, use_cache=use_cache)
        return b, dict(rec, brick=tuple(rec["brick"]), launch=launch["launch"], cached=True)
    b = GpuBatch(scenes, fmt=fmt, brick=bricks[0])
    first = tune_batch(b, spp, reps=reps, use_cache=use_cache)
    timed = {",".join(map(str, bricks[0])): time_launch(b, spp, first["launch"], reps)}
    for shape in bricks[1:]:
        b.close()
        del b
        b = GpuBatch(scenes, fmt=fmt, brick=shape)
        timed[",".join(map(str, shape))] = time_launch(b, spp, first["launch"], reps)
    brick, _ = _fastest(timed)
    if b.brick != brick:
        b.close()
        del b
        b = GpuBatch(scenes, fmt=fmt, brick=brick)
    launch = tune_batch(b, spp, reps=reps, use_cache=use_cache)
    rec = {"brick": list(brick), "brick_ms": timed, "launch": list(launch["launch"]), "ms": launch["ms"]}
    if use_cache:
        _store(path, key, rec)
    return b, dict(rec, brick=brick, launch=launch["launch"], cached=False)
