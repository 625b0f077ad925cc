"""GPU-resident scene: uploads a Scene to HBM and drives the gbv_* C-ABI.

torch supplies device memory and the current stream only; every computation
runs in the native library's sm_103a kernels.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _native as N
from .scenes import Scene


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def mc_dims(dims, cells_per_mc: int) -> tuple:
    out = (C.c_int * 3)()
    N.check(N.lib().gbv_mc_dims(N.ivec(*dims), cells_per_mc, out), "gbv_mc_dims")
    return tuple(out)


class GpuScene:
    """A Scene resident on the current CUDA device.

    layout: GBV_LAYOUT_LINEAR (FP32 only) or GBV_LAYOUT_BRICK_CORNERS.
    fmt:    voxel format of the brick store.
    brick:  log2 of the brick edge in cells per axis (default (3, 3, 3)).
    """

    def __init__(self, scene: Scene, layout: int = N.GBV_LAYOUT_BRICK_CORNERS, fmt: int = N.GBV_VOXEL_F32,
                 scalars_device=None, brick=(3, 3, 3)):
        import torch
        self.s = scene
        self.layout, self.fmt = layout, fmt
        self.brick = tuple(int(b) for b in brick)
        dev = torch.device("cuda")
        if scalars_device is not None:
            self.scalars = scalars_device
        else:
            self.scalars = torch.from_numpy(np.ascontiguousarray(scene.scalars).reshape(-1)).to(dev)
        self.tf = torch.from_numpy(np.ascontiguousarray(scene.tf, dtype=np.float32)).to(dev)
        self.dims = scene.dims
        self.mc = mc_dims(self.dims, scene.cells_per_mc)
        nmc = self.mc[0] * self.mc[1] * self.mc[2]
        self.ranges = torch.empty(2 * max(nmc, 1), dtype=torch.float32, device=dev)
        self.majorants = torch.empty(max(nmc, 1), dtype=torch.float32, device=dev)
        self.voxels, self.scale_offset = self.scalars, None
        if layout == N.GBV_LAYOUT_BRICK_CORNERS:
            self.build_bricks(fmt)
        elif fmt != N.GBV_VOXEL_F32:
            raise ValueError("the linear layout holds FP32 voxels only")
        self.build_macrocells()
        self._init_env()

    def _init_env(self) -> None:
        import torch
        scene = self.s
        dev = torch.device("cuda")
        self.env_tex = self.cdf_y = self.cdf_x = None
        if scene.env is not None:
            e = scene.env
            H, W, _ = e.texels.shape
            self.env_tex = torch.from_numpy(np.ascontiguousarray(e.texels)).to(dev)
            self.cdf_y = torch.empty(H, dtype=torch.float32, device=dev)
            self.cdf_x = torch.empty(H * W, dtype=torch.float32, device=dev)
            N.check(N.lib().gbv_env_build_cdfs(_ptr(self.env_tex), W, H, N.ivec(*e.addr), _ptr(self.cdf_y),
                                               _ptr(self.cdf_x), _stream()), "gbv_env_build_cdfs")

    # -- macrocells ---------------------------------------------------------
    def build_macrocells(self) -> None:
        s = self.s
        nmc = self.mc[0] * self.mc[1] * self.mc[2]
        L = N.lib()
        if self.fmt == N.GBV_VOXEL_F32:
            N.check(L.gbv_build_mc_ranges(_ptr(self.scalars), N.ivec(*self.dims), s.cells_per_mc, _ptr(self.ranges),
                                          _stream()), "gbv_build_mc_ranges")
        else:  # quantized store: bound the stored values
            N.check(L.gbv_build_mc_ranges_from_store_shaped(_ptr(self.voxels), _ptr(self.scale_offset), self.fmt,
                                                            N.ivec(*self.dims), N.ivec(*self.brick), s.cells_per_mc,
                                                            _ptr(self.ranges), _stream()),
                    "gbv_build_mc_ranges_from_store_shaped")
        self.map_majorants()

    def map_majorants(self) -> None:
        s = self.s
        nmc = self.mc[0] * self.mc[1] * self.mc[2]
        N.check(N.lib().gbv_map_majorants(_ptr(self.ranges), nmc, _ptr(self.tf), self.tf.shape[0], s.domain[0],
                                          s.domain[1], s.base_density, _ptr(self.majorants), _stream()),
                "gbv_map_majorants")

    def build_bricks(self, fmt: int) -> None:
        import torch
        vb, sb = C.c_size_t(), C.c_size_t()
        N.check(N.lib().gbv_brick_store_bytes_shaped(N.ivec(*self.dims), fmt, N.ivec(*self.brick), C.byref(vb),
                                                     C.byref(sb)), "gbv_brick_store_bytes_shaped")
        # 32-byte aligned storage (torch allocations are 512-byte aligned)
        self.voxels = torch.empty(max(vb.value, 32), dtype=torch.uint8, device="cuda")
        self.scale_offset = torch.empty(max(sb.value, 8), dtype=torch.uint8, device="cuda") if sb.value else None
        N.check(N.lib().gbv_build_brick_store_shaped(_ptr(self.scalars), N.ivec(*self.dims), fmt,
                                                     N.ivec(*self.brick), _ptr(self.voxels), _ptr(self.scale_offset),
                                                     _stream()), "gbv_build_brick_store_shaped")
        self.fmt = fmt

    # -- scene record ---------------------------------------------------------
    def record(self) -> N.GbvScene:
        s = self.s
        r = N.GbvScene()
        r.d_voxels = self.voxels.data_ptr()
        r.d_scale_offset = self.scale_offset.data_ptr() if self.scale_offset is not None else None
        r.format, r.layout = self.fmt, self.layout
        r.dims[:] = list(self.dims)
        r.brick_log2[:] = list(self.brick)
        origin, spacing = s.geometry()
        r.origin[:] = list(origin)
        r.spacing[:] = list(spacing)
        r.d_majorants = self.majorants.data_ptr()
        r.cells_per_mc = s.cells_per_mc
        r.d_tf = self.tf.data_ptr()
        r.tf_n = self.tf.shape[0]
        r.domain[:] = list(s.domain)
        r.base_density = s.base_density
        r.anisotropy, r.scattering_albedo = s.anisotropy, s.scattering_albedo
        r.cam_pos[:] = list(s.cam_pos)
        r.cam_dir[:] = list(s.cam_dir)
        r.cam_up[:] = list(s.cam_up)
        r.fovy = s.fovy
        r.num_dir_lights = len(s.dir_lights)
        for i, (d, c, rad) in enumerate(s.dir_lights[:4]):
            r.dir_light_dir[i][:] = list(d)
            r.dir_light_color[i][:] = list(c)
            r.dir_light_radiance[i] = rad
        if s.env is not None:
            e = s.env
            H, W, _ = e.texels.shape
            r.d_env_texels = self.env_tex.data_ptr()
            r.d_env_cdf_y = self.cdf_y.data_ptr()
            r.d_env_cdf_x = self.cdf_x.data_ptr()
            r.env_dims[:] = [W, H]
            r.env_addr[:] = list(e.addr)
            r.env_dir[:] = list(e.direction)
            r.env_up[:] = list(e.up)
            r.env_scale = e.scale
        r.bg_color[:] = list(s.bg_color)
        r.ambient_radiance = s.ambient
        r.multi_scatter = s.multi_scatter
        r.volume_multi_scatter = s.volume_multi_scatter
        r.max_volume_bounces = s.max_volume_bounces
        r.volume_instance = s.volume_instance
        r.volume_user_id = getattr(s, "volume_user_id", 0)
        if s.iso is not None:
            iso = N.GbvIsoSurface()
            iso.iso_value = s.iso.value
            iso.d_ranges = self.ranges.data_ptr()
            iso.color[:] = [float(c) for c in s.iso.color]
            iso.opacity = s.iso.opacity
            iso.instance = s.iso.instance
            iso.user_id = s.iso.user_id
            self._iso_record = iso  # kept alive with the scene record's pointer to it
            r.iso = C.addressof(iso)
            if s.no_volume:
                r.d_majorants = None
        return r

    # -- rendering --------------------------------------------------------------
    def new_accum(self, width: Optional[int] = None, height: Optional[int] = None):
        import torch
        return torch.zeros(((height or self.s.height), (width or self.s.width), 4), dtype=torch.float32,
                           device="cuda")

    def render(self, spp: Optional[int] = None, accum=None, accum_id_start: int = 0, counters=None,
               width: Optional[int] = None, height: Optional[int] = None, config: Optional[dict] = None,
               aux: Optional[dict] = None):
        """Accumulates `spp` passes into accum (H, W, 4); returns accum.
        config: launch settings of gbv_render_ex (blocks_per_sm,
        threshold_pct, skip_cells, stage, profile); None = defaults.
        aux: auxiliary channels to write, CUDA tensors of (H, W) entries
        under "depth" (float32), "prim_id", "inst_id", "obj_id" (int32)."""
        w, h = width or self.s.width, height or self.s.height
        if accum is None:
            accum = self.new_accum(w, h)
        rec = self.record()
        if aux:
            for f, k in (("d_depth", "depth"), ("d_prim_id", "prim_id"), ("d_inst_id", "inst_id"),
                         ("d_obj_id", "obj_id")):
                t = aux.get(k)
                setattr(rec, f, t.data_ptr() if t is not None else None)
        n = self.s.spp if spp is None else spp
        if config is None:
            N.check(N.lib().gbv_render(C.byref(rec), _ptr(accum), w, h, accum_id_start, n, _ptr(counters),
                                       _stream()), "gbv_render")
        else:
            cfg = N.render_config(**config)
            N.check(N.lib().gbv_render_ex(C.byref(rec), _ptr(accum), w, h, accum_id_start, n, _ptr(counters),
                                          C.byref(cfg), _stream()), "gbv_render_ex")
        return accum

    def render_tiles(self, rank: int, world: int, spp: Optional[int] = None, accum=None, accum_id_start: int = 0,
                     counters=None):
        """render() of only the 32x32 tiles `rank` of `world` owns (the
        reference's round-robin partition); other pixels of accum are left
        as they are."""
        w, h = self.s.width, self.s.height
        if accum is None:
            accum = self.new_accum(w, h)
        rec = self.record()
        N.check(N.lib().gbv_render_tiles(C.byref(rec), _ptr(accum), w, h, accum_id_start,
                                         self.s.spp if spp is None else spp, rank, world, _ptr(counters),
                                         _stream()), "gbv_render_tiles")
        return accum

    def iso_intersect(self, rays, iso: float):
        """First crossings of the iso value by rays, a (n, 8) float32 CUDA
        tensor (org xyz, tmax, dir xyz, unused); returns (n, 8): t, P xyz,
        N xyz, hit (1/0)."""
        import torch
        rays = rays.contiguous().float()
        hits = torch.empty_like(rays)
        rec = self.record()
        N.check(N.lib().gbv_iso_intersect(C.byref(rec), _ptr(self.ranges), float(iso), _ptr(rays), rays.shape[0],
                                          _ptr(hits), _stream()), "gbv_iso_intersect")
        return hits

    def tonemap(self, accum, accum_id: int, fmt: int = N.GBV_FB_FLOAT4):
        import torch
        h, w, _ = accum.shape
        out = (torch.empty((h, w, 4), dtype=torch.float32, device="cuda") if fmt == N.GBV_FB_FLOAT4
               else torch.empty((h, w), dtype=torch.int32, device="cuda"))
        N.check(N.lib().gbv_tonemap(_ptr(accum), w, h, accum_id, fmt, _ptr(out), _stream()), "gbv_tonemap")
        return out


def ea_views(views) -> "C.Array":
    arr = (N.GbvEAView * len(views))()
    for a, v in zip(arr, views):
        a.pos[:] = list(v["pos"])
        a.dir[:] = list(v["dir"])
        a.up[:] = list(v["up"])
        a.fovy = v["fovy"]
        a.width, a.height = v["width"], v["height"]
    return arr
