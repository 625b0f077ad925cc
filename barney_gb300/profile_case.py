"""Small, self-contained render launches for ncu captures.

  python -m barney_gb300.profile_case --dims 512 --width 480 --height 270 --spp 1 --format f32

Builds the frame scene (512^3 volume by default), renders `--warmup` untimed
launches, then `--launches` launches of the render kernel as timed runs make
them (no event counting), then one launch with event counting, and writes its
counters to the --out JSON so that ncu DRAM bytes of the uncounted launches
can be related to density samples (the frame is deterministic, so every
launch processes the same samples).  To capture the uncounted launches:
ncu -k regex:render_kernel -s <warmup> -c <launches>.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, default=512)
    ap.add_argument("--width", type=int, default=480)
    ap.add_argument("--height", type=int, default=270)
    ap.add_argument("--spp", type=int, default=1)
    ap.add_argument("--format", default="f32", choices=["f32", "f16", "bf16", "u8"])
    ap.add_argument("--layout", default="brick", choices=["brick", "linear"])
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--launches", type=int, default=1)
    ap.add_argument("--out", default="profile_case.json")
    a = ap.parse_args()
    import torch
    from . import _native as N, scenes
    from .device import GpuScene
    s = scenes.frame_scene(dims=a.dims, width=a.width, height=a.height, spp=a.spp)
    fmt = {"f32": 0, "f16": 1, "bf16": 2, "u8": 3}[a.format]
    layout = N.GBV_LAYOUT_BRICK_CORNERS if a.layout == "brick" else N.GBV_LAYOUT_LINEAR
    g = GpuScene(s, layout=layout, fmt=fmt)
    acc = g.new_accum()
    for _ in range(a.warmup + a.launches):
        g.render(accum=acc)
    cnt = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    g.render(accum=acc, counters=cnt)
    torch.cuda.synchronize()
    c = [int(x) for x in cnt.cpu().tolist()]
    rec = dict(dims=a.dims, width=a.width, height=a.height, spp=a.spp, format=a.format, layout=a.layout,
               samples_per_launch=c[0], mc_visits_per_launch=c[1], rays_per_launch=c[2])
    Path(a.out).parent.mkdir(parents=True, exist_ok=True)
    Path(a.out).write_text(json.dumps(rec, indent=1))
    print(json.dumps(rec))


if __name__ == "__main__":
    sys.exit(main())
