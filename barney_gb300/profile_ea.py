"""EA launches for ncu captures: the differentiable emission-absorption
workload (128^3 density grid, 256-entry TF, 32 views of 256^2 on a sphere of
radius 2.5, step 0.5 voxel): `--warmup` forward+adjoint passes, then
`--passes` more.

  python -m barney_gb300.profile_ea --warmup 1 --passes 1

Capture the forward with -k regex:ea_forward and the adjoint with
-k regex:ea_backward, skipping the warm-up launches (-s <warmup>).
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, default=128)
    ap.add_argument("--views", type=int, default=32)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--passes", type=int, default=1)
    a = ap.parse_args()
    import torch
    from . import scenes
    from .ea import EAProblem
    gt = scenes.ea_scene(a.dims)
    views = scenes.fibonacci_views(a.views, 2.5, a.size)
    step = 0.5 / (a.dims - 1)
    tgt = EAProblem(gt, views, step).render()
    start = scenes.Scene(scalars=np.full_like(gt.scalars, 0.1), tf=gt.tf, base_density=gt.base_density)
    p = EAProblem(start, views, step)
    for _ in range(a.warmup + a.passes):
        img = p.render()
        p.backward(img, 2 * (img - tgt))
    torch.cuda.synchronize()
    print("ok")


if __name__ == "__main__":
    sys.exit(main())
