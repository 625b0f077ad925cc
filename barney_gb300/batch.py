"""Batched rendering of many scenes of uneven sizes in one persistent launch.

GpuBatch uploads each Scene (its own field, TF, camera, lights and frame),
creates the native batch (gbv_batch_create) and renders all items with one
kernel launch (gbv_batch_render), optionally captured once in a CUDA graph
and replayed.
"""
from __future__ import annotations

import ctypes as C

from . import _native as N
from .device import GpuScene, _ptr, _stream


class GpuBatch:
    def __init__(self, scenes, fmt: int = N.GBV_VOXEL_F32, layout: int = N.GBV_LAYOUT_BRICK_CORNERS,
                 brick=(3, 3, 3)):
        self.scenes = list(scenes)
        self.fmt, self.layout, self.brick = fmt, layout, tuple(brick)
        self.items = [GpuScene(s, layout=layout, fmt=fmt, brick=brick) for s in self.scenes]
        self.accums = [g.new_accum() for g in self.items]
        n = len(self.items)
        recs = (N.GbvScene * n)(*[g.record() for g in self.items])
        self._recs = recs
        ptrs = (C.c_void_p * n)(*[a.data_ptr() for a in self.accums])
        ws = (C.c_int * n)(*[g.s.width for g in self.items])
        hs = (C.c_int * n)(*[g.s.height for g in self.items])
        h = C.c_void_p()
        N.check(N.lib().gbv_batch_create(recs, ptrs, ws, hs, n, C.byref(h)), "gbv_batch_create")
        self.h = h
        self.graph = None

    def set_launch(self, blocks_per_sm: int, threshold: int, skip: int) -> None:
        N.check(N.lib().gbv_batch_set_launch(self.h, blocks_per_sm, threshold, skip), "gbv_batch_set_launch")

    def render(self, spp: int, accum_id_start: int = 0, counters=None) -> None:
        N.check(N.lib().gbv_batch_render(self.h, accum_id_start, spp, _ptr(counters), _stream()),
                "gbv_batch_render")

    def capture(self, spp: int, accum_id_start: int = 0, counters=None):
        """Captures one batch render in a CUDA graph (torch.cuda.CUDAGraph)."""
        import torch
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.render(spp, accum_id_start, counters)
        torch.cuda.current_stream().wait_stream(s)
        self.graph = g
        return g

    def close(self) -> None:
        if self.h:
            N.lib().gbv_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
