"""Seeded synthetic scenes of the structured-volume workloads.

The reference's regression data is not available; these stand in for it with
the shapes, sizes and value distributions of the named workloads:

* ``small``   64^3 FP32 blob+noise volume (8 blobs, seed 1), 128-entry ramp TF,
  8^3-voxel macrocells, 256x256, 16 spp, one directional light plus ambient,
  single scatter (the reference's default build).
* ``frame``   512^3 volume (64 blobs + 4-octave fBm, seed 2), 256-entry
  two-peak TF, 16^3-voxel macrocells, 1920x1080, 64 spp, up to 4 isotropic
  volume bounces, directional light plus a 512x256 sky env map.
* ``ea``      128^3 ground-truth blob volume (16 blobs, seed 4), 256-entry TF,
  32 views of 256x256 on a Fibonacci sphere of radius 2.5.
* ``batch``   64 volumes with sides log-uniform in [32,256] per axis (seed 5).

A volume fills the unit cube centred at the origin: origin -0.5, spacing
1/(N-1) per axis.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _native as N


@dataclass
class EnvMap:
    texels: np.ndarray                 # (H, W, 4) float32, row 0 first
    addr: tuple = (N.GBV_ADDR_WRAP, N.GBV_ADDR_CLAMP)
    direction: tuple = (1.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    scale: float = 1.0


@dataclass
class IsoSurface:
    """An iso-surface of the scene's field (IsoSurface geometry) with a matte
    material (AnariMatte: constant color and opacity).  `instance` is the RTC
    instance index of the geometry's group in the world's instance list
    (0 when it shares a group with the volume: a group's user geometries
    come before its volumes)."""
    value: float
    color: tuple = (0.8, 0.8, 0.8, 1.0)  # AnariMatte default color (AnariMatte.h:43), alpha 1
    opacity: float = 1.0
    instance: int = 0
    user_id: int = 0  # the geometry's "userID": the object ID of its hits


@dataclass
class Scene:
    scalars: np.ndarray                # (nz, ny, nx) float32
    tf: np.ndarray                     # (n, 4) float32 RGBA
    domain: tuple = (0.0, 1.0)
    base_density: float = 20.0
    cells_per_mc: int = 8
    anisotropy: float = 0.0
    scattering_albedo: float = 0.9
    cam_pos: tuple = (0.0, 0.0, 2.5)
    cam_dir: tuple = (0.0, 0.0, -1.0)
    cam_up: tuple = (0.0, 1.0, 0.0)
    fovy: float = 60.0
    dir_lights: list = field(default_factory=list)   # [(direction, color, radiance)]
    env: Optional[EnvMap] = None
    bg_color: tuple = (0.0, 0.0, 0.0, 1.0)
    ambient: float = 1.0
    multi_scatter: int = 0
    volume_multi_scatter: int = 0
    max_volume_bounces: int = 0
    width: int = 256
    height: int = 256
    spp: int = 16
    origin: Optional[tuple] = None
    spacing: Optional[tuple] = None
    # an iso-surface over the same field; the volume's RTC instance index
    # (1 when the iso-surface shares its group); no_volume: the world holds
    # the iso-surface only
    iso: Optional[IsoSurface] = None
    volume_instance: int = 0
    volume_user_id: int = 0  # the volume's "userID": the object ID of its hits
    no_volume: bool = False

    @property
    def dims(self) -> tuple:
        nz, ny, nx = self.scalars.shape
        return (nx, ny, nz)

    def geometry(self) -> tuple:
        nx, ny, nz = self.dims
        origin = self.origin if self.origin is not None else (-0.5, -0.5, -0.5)
        spacing = self.spacing if self.spacing is not None else (
            1.0 / (nx - 1), 1.0 / (ny - 1), 1.0 / (nz - 1))
        return origin, spacing


_SCENEGEN = None


def _scenegen() -> C.CDLL:
    """The input generator library (barney_gb300/_lib/libgbv_scenegen.so,
    host code apart from the renderer); raises if it has not been built."""
    global _SCENEGEN
    if _SCENEGEN is None:
        from pathlib import Path
        path = Path(__file__).resolve().parent / "_lib" / "libgbv_scenegen.so"
        if not path.exists():
            raise RuntimeError(f"input generator missing: {path} (run __graft_entry__.build())")
        L = C.CDLL(str(path))
        L.sg_blob_volume.restype = C.c_int
        L.sg_blob_volume.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_uint64, C.c_float, C.c_int, C.c_float,
                                     C.c_int, C.c_void_p]
        _SCENEGEN = L
    return _SCENEGEN


def blob_volume(dims, num_blobs: int, seed: int, noise: float = 0.05, fbm_octaves: int = 0,
                fbm_amplitude: float = 0.0, nthreads: int = 0) -> np.ndarray:
    """FP32 (nz, ny, nx) blob+noise volume from the seeded generator."""
    nx, ny, nz = dims
    out = np.empty((nz, ny, nx), dtype=np.float32)
    dv = (C.c_int * 3)(int(nx), int(ny), int(nz))
    if _scenegen().sg_blob_volume(dv, num_blobs, seed, noise, fbm_octaves, fbm_amplitude, nthreads,
                                  out.ctypes.data_as(C.c_void_p)) != 0:
        raise ValueError(f"sg_blob_volume: bad arguments {dims}, {num_blobs}, {fbm_octaves}")
    return out


# nanovdb::GridType of the value types the NanoVDB field reads
NANOVDB_TYPES = {"float": 1, "fp4": 13, "fp8": 14, "fp16": 15, "fpn": 16}


def nanovdb_grid(values: np.ndarray, origin=(0, 0, 0), voxel_size: float = 1.0, translation=(0.0, 0.0, 0.0),
                 background: float = 0.0, grid_type: str = "float", tolerance: float = -1.0) -> bytes:
    """A NanoVDB grid (format 32.7 memory layout) of a dense (nz, ny, nx)
    array placed at index `origin`, world = voxel_size * index +
    translation; voxels equal to `background` are inactive.  grid_type: one
    of NANOVDB_TYPES (quantized as NanoVDB's builder does, dithering off);
    tolerance: the absolute error of an FpN leaf's bit width (negative: the
    builder's default for a fog volume)."""
    L = _scenegen()
    if not hasattr(L, "_nvdb_ready"):
        L.sg_nanovdb_from_dense_typed.restype = C.c_int
        L.sg_nanovdb_from_dense_typed.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_double,
                                                  C.c_void_p, C.c_int, C.c_float, C.POINTER(C.c_void_p),
                                                  C.POINTER(C.c_size_t)]
        L.sg_free.argtypes = [C.c_void_p]
        L._nvdb_ready = True
    v = np.ascontiguousarray(values, np.float32)
    nz, ny, nx = v.shape
    dims = np.array([nx, ny, nz], np.int32)
    org = np.array(origin, np.int32)
    tr = np.array(translation, np.float64)
    buf, n = C.c_void_p(), C.c_size_t()
    rc = L.sg_nanovdb_from_dense_typed(v.ctypes.data, dims.ctypes.data, org.ctypes.data, background, voxel_size,
                                       tr.ctypes.data, NANOVDB_TYPES[grid_type], tolerance, C.byref(buf),
                                       C.byref(n))
    if rc != 0:
        raise ValueError(f"sg_nanovdb_from_dense_typed failed ({rc})")
    try:
        return C.string_at(buf, n.value)
    finally:
        L.sg_free(buf)


def nanovdb_of_scene(scene: "Scene", grid_type: str = "float", tolerance: float = -1.0) -> bytes:
    """The scene's volume as a NanoVDB grid whose voxel centres lie where the
    structured field has its voxels (the NanoVDB sampler reads voxel i at
    index i + 1/2; needs the same spacing on every axis), of the given value
    type (see nanovdb_grid)."""
    origin, spacing = scene.geometry()
    if not (spacing[0] == spacing[1] == spacing[2]):
        raise ValueError("a NanoVDB grid has one voxel size")
    vs = float(spacing[0])
    return nanovdb_grid(scene.scalars, (0, 0, 0), vs, tuple(float(o) - 0.5 * vs for o in origin), background=-1.0,
                        grid_type=grid_type, tolerance=tolerance)


def tf_ramp(n: int = 128, max_opacity: float = 0.8) -> np.ndarray:
    """Opacity ramps linearly 0 -> max_opacity; colour ramps blue -> red."""
    t = np.linspace(0.0, 1.0, n, dtype=np.float64)
    tf = np.stack([t, np.full_like(t, 0.25), 1.0 - t, max_opacity * t], axis=1)
    return tf.astype(np.float32)


def tf_two_peaks(n: int = 256) -> np.ndarray:
    """Opacity peaks at s=0.35 (0.6, half-width 0.03) and s=0.70 (0.9, half-width 0.05)."""
    s = np.linspace(0.0, 1.0, n, dtype=np.float64)
    a = np.maximum(0.6 * np.clip(1.0 - np.abs(s - 0.35) / 0.03, 0, 1),
                   0.9 * np.clip(1.0 - np.abs(s - 0.70) / 0.05, 0, 1))
    tf = np.stack([0.9 - 0.5 * s, 0.4 + 0.4 * s, 0.2 + 0.8 * s, a], axis=1)
    return tf.astype(np.float32)


def tf_two_ramps(n: int, rng: np.random.Generator) -> np.ndarray:
    """Random two-ramp TF of the batched workload."""
    s = np.linspace(0.0, 1.0, n)
    c1, c2 = np.sort(rng.uniform(0.1, 0.9, 2))
    a = np.maximum(np.clip((s - c1) / 0.2, 0, 1) * 0.5, np.clip((s - c2) / 0.1, 0, 1) * rng.uniform(0.5, 1.0))
    col = rng.uniform(0.2, 1.0, 3)
    tf = np.stack([col[0] * (1 - s) + s, col[1] * np.ones_like(s), col[2] * s + 0.2, a], axis=1)
    return tf.astype(np.float32)


def env_sky(width: int = 512, height: int = 256) -> EnvMap:
    """Sky gradient (zenith (0.2,0.4,1.0) to horizon (0.9,0.9,1.0)) with a sun disk
    of radius 1.5 deg at elevation 35 deg, radiance 50.

    Texel row iy is polar angle theta = pi (iy+.5)/H of the map's local frame,
    whose z axis the env light maps to -up (EnvMapLight::commit), so the
    elevation above the horizon is theta - pi/2."""
    iy, ix = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    theta = math.pi * (iy + 0.5) / height
    phi = 2 * math.pi * (ix + 0.5) / width
    elev = theta - math.pi / 2
    zen = np.array([0.2, 0.4, 1.0])
    hor = np.array([0.9, 0.9, 1.0])
    gnd = np.array([0.25, 0.22, 0.2])
    w = np.clip(np.sin(elev), 0, 1)[..., None]
    sky = hor * (1 - w) + zen * w
    rgb = np.where((elev >= 0)[..., None], sky, gnd)
    # sun at elevation 35 deg, azimuth 45 deg
    se, sa = math.radians(35.0), math.radians(45.0)
    sun = np.array([math.cos(se) * math.cos(sa), math.cos(se) * math.sin(sa), math.sin(se)])
    d = np.stack([np.cos(elev) * np.cos(phi), np.cos(elev) * np.sin(phi), np.sin(elev)], axis=-1)
    ang = np.arccos(np.clip(d @ sun, -1, 1))
    disk = ang < math.radians(1.5)
    disk.flat[np.argmin(ang)] = True  # a coarse map still gets its sun texel
    rgb = np.where(disk[..., None], np.array([50.0, 47.0, 42.0]), rgb)
    tex = np.concatenate([rgb, np.ones_like(rgb[..., :1])], axis=-1).astype(np.float32)
    return EnvMap(texels=np.ascontiguousarray(tex))


def _look_at_origin(pos):
    p = np.asarray(pos, dtype=np.float64)
    return tuple(float(x) for x in p), tuple(float(x) for x in -p)


def small_scene(dims: int = 64, spp: int = 16, width: int = 256, height: int = 256) -> Scene:
    vol = blob_volume((dims, dims, dims), 8, seed=1, noise=0.05)
    pos = 2.5 * np.array([0.3, 0.4, 1.0]) / np.linalg.norm([0.3, 0.4, 1.0])
    cp, cd = _look_at_origin(pos)
    d = np.array([-1.0, -1.0, -1.0]) / math.sqrt(3.0)
    return Scene(scalars=vol, tf=tf_ramp(128), base_density=20.0, cells_per_mc=8,
                 cam_pos=cp, cam_dir=cd, dir_lights=[(tuple(d), (1.0, 1.0, 1.0), 2.0)],
                 ambient=0.3, width=width, height=height, spp=spp)


def frame_scene(dims: int = 512, width: int = 1920, height: int = 1080, spp: int = 64,
                with_env: bool = True) -> Scene:
    vol = blob_volume((dims, dims, dims), 64, seed=2, noise=0.05, fbm_octaves=4, fbm_amplitude=0.1)
    pos = 2.5 * np.array([0.3, 0.4, 1.0]) / np.linalg.norm([0.3, 0.4, 1.0])
    cp, cd = _look_at_origin(pos)
    d = np.array([-1.0, -1.0, -1.0]) / math.sqrt(3.0)
    return Scene(scalars=vol, tf=tf_two_peaks(256), base_density=50.0, cells_per_mc=16,
                 anisotropy=0.0, scattering_albedo=0.9, cam_pos=cp, cam_dir=cd,
                 dir_lights=[(tuple(d), (1.0, 1.0, 1.0), 2.0)], env=env_sky() if with_env else None,
                 ambient=0.3, multi_scatter=1, volume_multi_scatter=1, max_volume_bounces=4,
                 width=width, height=height, spp=spp)


def fibonacci_views(n: int = 32, radius: float = 2.5, size: int = 256, fovy: float = 60.0):
    """n views of size^2 placed on a Fibonacci sphere, looking at the origin."""
    views = []
    golden = math.pi * (3.0 - math.sqrt(5.0))
    for i in range(n):
        y = 1.0 - 2.0 * (i + 0.5) / n
        r = math.sqrt(max(0.0, 1.0 - y * y))
        th = golden * i
        p = np.array([math.cos(th) * r, y, math.sin(th) * r]) * radius
        up = (0.0, 1.0, 0.0) if abs(y) < 0.99 else (1.0, 0.0, 0.0)
        views.append(dict(pos=tuple(p), dir=tuple(-p), up=up, fovy=fovy, width=size, height=size))
    return views


def ea_scene(dims: int = 128) -> Scene:
    vol = blob_volume((dims, dims, dims), 16, seed=4, noise=0.0)
    return Scene(scalars=vol, tf=tf_two_peaks(256), base_density=20.0, cells_per_mc=8)


def batch_items(count: int = 64, seed: int = 5, lo: int = 32, hi: int = 256):
    """Batched workload: `count` (scene, view) items of uneven sizes."""
    rng = np.random.default_rng(seed)
    items = []
    for k in range(count):
        dims = tuple(int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(3))
        vol = blob_volume(dims, 8, seed=500 + k, noise=0.05)
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        size = int(rng.choice([128, 256, 512]))
        cp, cd = _look_at_origin(2.5 * v)
        up = (0.0, 1.0, 0.0) if abs(v[1]) < 0.99 else (1.0, 0.0, 0.0)
        d = np.array([-1.0, -1.0, -1.0]) / math.sqrt(3.0)
        items.append(Scene(scalars=vol, tf=tf_two_ramps(128, rng), base_density=20.0, cells_per_mc=8,
                           cam_pos=cp, cam_dir=cd, cam_up=up, dir_lights=[(tuple(d), (1.0, 1.0, 1.0), 2.0)],
                           ambient=0.3, width=size, height=size, spp=8))
    return items
