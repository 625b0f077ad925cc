"""Generates tests/golden/nanovdb_pin.npz and nanovdb_fp_pin.npz: NanoVDB
grids made by the NanoVDB library the reference vendors -- one of value type
Float, and grids of the quantized types Fp4, Fp8, Fp16 and FpN (FpN at two
tolerances, so that its leaves take every bit width from 1 to 16) -- and the
reference's own NanoVDB field code run on them (oracle/refpin/ref_nanovdb.cpp,
built by `make -C oracle ref`): samples of NanoVDBDataSampler at fixed
points, the macrocell grid and ranges of NanoVDBData_computeMCs, and the
NanoVDB layout offsets.  tests/test_oracle_refpin.py and
tests/test_gpu_nanovdb.py check the oracle and the library against these
vectors on any machine.

  python tests/golden/make_nanovdb_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "nanovdb_pin.npz"
OUT_FP = Path(__file__).resolve().parent / "nanovdb_fp_pin.npz"
# the quantized grids of the fixture: name -> (nanovdb::GridType, FpN tolerance)
FP_GRIDS = {"fp4": (13, -1.0), "fp8": (14, -1.0), "fp16": (15, -1.0), "fpn_fine": (16, 0.001),
            "fpn_coarse": (16, 0.05)}


def _lib():
    from oracle import refpin
    L = refpin.lib()
    vp = C.c_void_p
    L.ref_nanovdb_from_dense.restype = C.c_int
    L.ref_nanovdb_from_dense.argtypes = [vp, vp, vp, C.c_float, C.c_double, vp, C.POINTER(vp), C.POINTER(C.c_size_t)]
    L.ref_nanovdb_from_dense_typed.restype = C.c_int
    L.ref_nanovdb_from_dense_typed.argtypes = [vp, vp, vp, C.c_float, C.c_double, vp, C.c_int, C.c_float, C.c_int,
                                               C.POINTER(vp), C.POINTER(C.c_size_t)]
    L.ref_nanovdb_fp_layout.restype = C.c_int
    L.ref_nanovdb_fp_layout.argtypes = [vp]
    L.ref_nanovdb_sample.restype = C.c_int
    L.ref_nanovdb_sample.argtypes = [vp, C.c_size_t, vp, C.c_int, vp]
    L.ref_nanovdb_mc_ranges.restype = C.c_int
    L.ref_nanovdb_mc_ranges.argtypes = [vp, C.c_size_t, vp, vp, vp, C.c_longlong]
    L.ref_nanovdb_layout.restype = C.c_int
    L.ref_nanovdb_layout.argtypes = [vp]
    L.ref_free.argtypes = [vp]
    return L


def make_grid(values: np.ndarray, index_origin, voxel_size: float, translation, background: float = 0.0,
              grid_type: int = 1, tolerance: float = -1.0, fog: bool = False) -> bytes:
    """A NanoVDB grid of a dense (nz, ny, nx) array, voxels equal to the
    background left inactive, of nanovdb::GridType grid_type (1 Float, 13
    Fp4, 14 Fp8, 15 Fp16, 16 FpN with leaves within `tolerance`; dithering
    off), made by the library's builder; fog: a fog-volume grid."""
    L = _lib()
    v = np.ascontiguousarray(values, np.float32)
    nz, ny, nx = v.shape
    dims = np.array([nx, ny, nz], np.int32)
    org = np.array(index_origin, np.int32)
    tr = np.array(translation, np.float64)
    buf, n = C.c_void_p(), C.c_size_t()
    if L.ref_nanovdb_from_dense_typed(v.ctypes.data, dims.ctypes.data, org.ctypes.data, background, voxel_size,
                                      tr.ctypes.data, grid_type, tolerance, int(fog), C.byref(buf),
                                      C.byref(n)) != 0:
        raise RuntimeError("grid creation failed")
    out = C.string_at(buf, n.value)
    L.ref_free(buf)
    return out


def reference_samples(grid: bytes, points: np.ndarray) -> np.ndarray:
    L = _lib()
    g = np.frombuffer(grid, np.uint8).copy()
    p = np.ascontiguousarray(points, np.float32)
    out = np.empty(p.shape[0], np.float32)
    if L.ref_nanovdb_sample(g.ctypes.data, g.size, p.ctypes.data, p.shape[0], out.ctypes.data) != 0:
        raise RuntimeError("sampling failed")
    return out


def reference_mc(grid: bytes):
    L = _lib()
    g = np.frombuffer(grid, np.uint8).copy()
    mc = np.zeros(3, np.int32)
    world = np.zeros(6, np.float32)
    L.ref_nanovdb_mc_ranges(g.ctypes.data, g.size, mc.ctypes.data, world.ctypes.data, None, 0)
    ranges = np.empty((int(np.prod(mc)), 2), np.float32)
    if L.ref_nanovdb_mc_ranges(g.ctypes.data, g.size, mc.ctypes.data, world.ctypes.data, ranges.ctypes.data,
                               ranges.shape[0]) != 0:
        raise RuntimeError("macrocell build failed")
    return mc, world, ranges


def layout() -> np.ndarray:
    out = np.zeros(32, np.int64)
    n = _lib().ref_nanovdb_layout(out.ctypes.data)
    return out[:n]


def fp_layout() -> np.ndarray:
    out = np.zeros(32, np.int64)
    n = _lib().ref_nanovdb_fp_layout(out.ctypes.data)
    return out[:n]


def pin_volume() -> np.ndarray:
    """The pinned grid's dense values: a 36 x 30 x 28 blob volume whose
    values below 0.05 are left inactive (background 0)."""
    from barney_gb300 import scenes
    vol = scenes.blob_volume((36, 30, 28), 6, seed=21, noise=0.0)
    return np.where(vol < 0.05, np.float32(0.0), vol).astype(np.float32)


PIN = dict(index_origin=(-5, 3, 7), voxel_size=0.03, translation=(-0.4, -0.55, -0.35))


def main() -> None:
    from oracle import refpin
    if not refpin.available():
        raise SystemExit("the reference checkout is needed to build oracle/_ref (make -C oracle ref)")
    grid = make_grid(pin_volume(), **PIN)
    rng = np.random.default_rng(17)
    pts = (rng.random((4000, 3)) * 1.6 - 0.8).astype(np.float32)
    samples = reference_samples(grid, pts)
    mc, world, ranges = reference_mc(grid)
    np.savez_compressed(OUT, grid=np.frombuffer(grid, np.uint8), points=pts, samples=samples, mc_dims=mc,
                        world=world, ranges=ranges, layout=layout())
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes): grid {len(grid)} bytes, {int(np.prod(mc))} macrocells")
    fp = {"points": pts, "fp_layout": fp_layout()}
    for name, (gtype, tol) in FP_GRIDS.items():
        g = make_grid(pin_volume(), **PIN, grid_type=gtype, tolerance=tol, fog=True)
        mc, world, ranges = reference_mc(g)
        fp.update({f"grid_{name}": np.frombuffer(g, np.uint8), f"samples_{name}": reference_samples(g, pts),
                   f"mc_dims_{name}": mc, f"ranges_{name}": ranges})
    np.savez_compressed(OUT_FP, **fp)
    print(f"wrote {OUT_FP} ({OUT_FP.stat().st_size} bytes): grids {', '.join(FP_GRIDS)}")


if __name__ == "__main__":
    main()
