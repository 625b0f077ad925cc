"""NanoVDB grid fields of value type Float, Fp4, Fp8, Fp16 or FpN
(gbv_nanovdb_* in include/gbvol.h).

parse() checks a grid held in host memory; GpuNanoVDBScene renders a Scene
whose field is such a grid (its transfer function, camera, lights and
renderer settings come from the Scene)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .device import GpuScene, _ptr, _stream
from .scenes import Scene


class GbvNanovdbInfo(C.Structure):
    _fields_ = [("bytes", C.c_ulonglong), ("root_offset", C.c_longlong), ("root_tiles", C.c_uint),
                ("background", C.c_float), ("inv_map", C.c_float * 9), ("map_offset", C.c_float * 3),
                ("index_lo", C.c_int * 3), ("index_hi", C.c_int * 3), ("world_lo", C.c_float * 3),
                ("world_hi", C.c_float * 3), ("voxel_size", C.c_double * 3), ("mc_dims", C.c_int * 3),
                ("grid_type", C.c_int)]


_ready = False


def lib() -> C.CDLL:
    global _ready
    L = N.lib()
    if not _ready:
        vp = C.c_void_p
        ip = C.POINTER(GbvNanovdbInfo)
        for name, args in {"gbv_nanovdb_parse": [vp, C.c_size_t, ip],
                           "gbv_nanovdb_mc_ranges": [vp, ip, vp, vp],
                           "gbv_nanovdb_sample": [vp, ip, vp, C.c_longlong, vp, vp]}.items():
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = args
        _ready = True
    return L


def parse(grid: bytes) -> GbvNanovdbInfo:
    info = GbvNanovdbInfo()
    g = np.frombuffer(bytes(grid), np.uint8)
    N.check(lib().gbv_nanovdb_parse(g.ctypes.data_as(C.c_void_p), g.size, C.byref(info)), "gbv_nanovdb_parse")
    return info


class GpuNanoVDBScene(GpuScene):
    """A Scene whose field is a NanoVDB grid (bytes), on the device."""

    def __init__(self, scene: Scene, grid: bytes):
        import torch
        self.s = scene
        self.layout, self.fmt, self.brick = N.GBV_LAYOUT_NANOVDB, N.GBV_VOXEL_F32, (3, 3, 3)
        self.info = parse(grid)
        host = np.frombuffer(bytes(grid), np.uint8).copy()
        self.grid = torch.from_numpy(host).cuda()
        self.voxels, self.scale_offset = self.grid, None
        self.dims = scene.dims
        self.tf = torch.from_numpy(np.ascontiguousarray(scene.tf, dtype=np.float32)).cuda()
        self.mc = tuple(self.info.mc_dims)
        nmc = self.mc[0] * self.mc[1] * self.mc[2]
        self.ranges = torch.empty(2 * nmc, dtype=torch.float32, device="cuda")
        self.majorants = torch.empty(nmc, dtype=torch.float32, device="cuda")
        self.build_macrocells()
        self._init_env()

    def build_macrocells(self) -> None:
        N.check(lib().gbv_nanovdb_mc_ranges(_ptr(self.grid), C.byref(self.info), _ptr(self.ranges), _stream()),
                "gbv_nanovdb_mc_ranges")
        self.map_majorants()

    def sample(self, points):
        import torch
        p = points.contiguous().float()
        out = torch.empty(p.shape[0], dtype=torch.float32, device="cuda")
        N.check(lib().gbv_nanovdb_sample(_ptr(self.grid), C.byref(self.info), _ptr(p), p.shape[0], _ptr(out),
                                         _stream()), "gbv_nanovdb_sample")
        return out

    def record(self) -> N.GbvScene:
        r = super().record()
        r.layout = N.GBV_LAYOUT_NANOVDB
        r.format = N.GBV_VOXEL_F32
        r.d_voxels = self.grid.data_ptr()
        r.d_scale_offset = None
        r.cells_per_mc = 0
        r.nanovdb = C.addressof(self.info)
        return r
