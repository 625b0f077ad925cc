"""TEST INFRASTRUCTURE ONLY: the reference pin.

ctypes binding of oracle/_ref/libbarney_ref.so, the reference renderer's own
sources for the structured-volume path compiled unchanged from the reference
tree (recipe: oracle/Makefile, target `ref`; harness: ref_harness.cpp).  The
reference tree exists only where the reference checkout does; elsewhere
`available()` is False and the pinned fixtures (tests/golden/ref_pin.npz)
stand in for the live library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
LIB = ORACLE / "_ref" / "libbarney_ref.so"
REF = Path(os.environ.get("BARNEY_REFERENCE_ROOT", "/root/reference"))

_lib = None


def reference_present() -> bool:
    return (REF / "barney" / "volume" / "DDA.h").exists()


def build() -> Path:
    """Compiles the pin library (needs the reference tree)."""
    subprocess.run(["make", "-s", "-C", str(ORACLE), "ref", f"REF={REF}"], check=True)
    return LIB


def available() -> bool:
    if LIB.exists():
        return True
    if not reference_present():
        return False
    build()
    return LIB.exists()


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("reference pin library unavailable (no reference tree to build it from)")
        L = C.CDLL(str(LIB))
        vp, i, f, u32, u64 = C.c_void_p, C.c_int, C.c_float, C.c_uint32, C.c_uint64
        sigs = {
            "ref_pin_version": (i, []),
            "ref_rng_sequence": (None, [u32, u32, i, vp]),
            "ref_rng_from_seed": (None, [u64, u64, i, i, vp, C.POINTER(u64)]),
            "ref_rng_seed_state": (u64, [u32, u32]),
            "ref_hash3": (u64, [u32, u32, u32]),
            "ref_fast_log": (f, [f]),
            "ref_float_to_half": (C.c_uint16, [f]),
            "ref_half_to_float": (f, [C.c_uint16]),
            "ref_tf_map": (None, [vp, i, f, f, f, vp, i, vp]),
            "ref_tf_majorant": (None, [vp, i, f, f, f, vp, i, vp]),
            "ref_dda": (i, [vp, vp, f, vp, i, vp, vp]),
            "ref_sample_points": (None, [vp, vp, vp, vp, vp, i, vp]),
            "ref_sample_and_map": (None, [vp, vp, vp, vp, vp, i, f, f, f, vp, i, vp]),
            "ref_trace_ray": (i, [vp, vp, vp, vp, i, vp, vp, i, f, f, f, vp, vp, f, C.POINTER(u64), C.POINTER(f),
                                  vp, vp]),
            "ref_rgba8": (None, [vp, i, i, vp]),
            "ref_iso_hit": (i, [vp, vp, vp, vp, i, vp, f, vp, f, i, vp, vp, f, C.POINTER(u64), C.POINTER(f), vp,
                                vp, vp]),
            "ref_lambertian": (None, [vp, vp, vp, vp, u32, u32, vp]),
            "ref_env_cdfs": (None, [vp, vp, vp, vp, vp]),
            "ref_shade_multi_scatter": (i, []),
            "ref_camera_commit": (None, [vp, vp, vp, f, vp]),
            "ref_mc_ranges": (None, [vp, vp, vp]),
            "ref_generate": (i, [vp, vp, vp, f, i, i, i, vp, vp, vp]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return a.ctypes.data_as(C.c_void_p)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, np.float32)


def rng_sequence(a: int, b: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float32)
    lib().ref_rng_sequence(a, b, n, _p(out))
    return out


def rng_from_seed(state: int, h: int, use_u64: bool, n: int):
    out = np.empty(n, np.float32)
    ns = C.c_uint64()
    lib().ref_rng_from_seed(state, h, 1 if use_u64 else 0, n, _p(out), C.byref(ns))
    return out, ns.value


def fast_log(x: np.ndarray) -> np.ndarray:
    return np.array([lib().ref_fast_log(float(v)) for v in _f32(x).reshape(-1)], np.float32)


def float_to_half(x: np.ndarray) -> np.ndarray:
    return np.array([lib().ref_float_to_half(float(v)) for v in _f32(x).reshape(-1)], np.uint16)


def half_to_float(h: np.ndarray) -> np.ndarray:
    return np.array([lib().ref_half_to_float(int(v)) for v in np.asarray(h, np.uint16).reshape(-1)], np.float32)


def tf_map(tf, domain, base_density, s) -> np.ndarray:
    tf, s = _f32(tf), _f32(s).reshape(-1)
    out = np.empty((s.size, 4), np.float32)
    lib().ref_tf_map(_p(tf), tf.shape[0], domain[0], domain[1], base_density, _p(s), s.size, _p(out))
    return out


def tf_majorant(tf, domain, base_density, ranges) -> np.ndarray:
    tf, r = _f32(tf), _f32(ranges).reshape(-1, 2)
    out = np.empty(r.shape[0], np.float32)
    lib().ref_tf_majorant(_p(tf), tf.shape[0], domain[0], domain[1], base_density, _p(r), r.shape[0], _p(out))
    return out


def dda(org, direction, t_max, grid, max_cells=4096):
    cells = np.zeros((max_cells, 3), np.int32)
    t01 = np.zeros((max_cells, 2), np.float32)
    n = lib().ref_dda(_p(_f32(org)), _p(_f32(direction)), t_max, _p(np.asarray(grid, np.int32)), max_cells,
                      _p(cells), _p(t01))
    return cells[:n], t01[:n]


def _geom(scalars, origin, spacing):
    nz, ny, nx = scalars.shape
    return np.array([nx, ny, nz], np.int32), _f32(origin), _f32(spacing)


def sample_points(scalars, origin, spacing, P) -> np.ndarray:
    scalars = _f32(scalars)
    dims, o, sp = _geom(scalars, origin, spacing)
    P = _f32(P).reshape(-1, 3)
    out = np.empty(P.shape[0], np.float32)
    lib().ref_sample_points(_p(scalars), _p(dims), _p(o), _p(sp), _p(P), P.shape[0], _p(out))
    return out


def sample_and_map(scalars, origin, spacing, tf, domain, base_density, P) -> np.ndarray:
    scalars, tf = _f32(scalars), _f32(tf)
    dims, o, sp = _geom(scalars, origin, spacing)
    P = _f32(P).reshape(-1, 3)
    out = np.empty((P.shape[0], 4), np.float32)
    lib().ref_sample_and_map(_p(scalars), _p(dims), _p(o), _p(sp), _p(tf), tf.shape[0], domain[0], domain[1],
                             base_density, _p(P), P.shape[0], _p(out))
    return out


def trace_ray(scalars, origin, spacing, cells_per_mc, majorants, tf, domain, base_density, org, direction, tmax,
              seed_state):
    """MCVolumeAccel::isProg for one ray: (hit, t, P, albedo, new seed state)."""
    scalars, tf, maj = _f32(scalars), _f32(tf), _f32(majorants)
    dims, o, sp = _geom(scalars, origin, spacing)
    st = C.c_uint64(seed_state)
    t = C.c_float(0.0)
    P = np.zeros(3, np.float32)
    alb = np.zeros(3, np.float32)
    h = lib().ref_trace_ray(_p(scalars), _p(dims), _p(o), _p(sp), cells_per_mc, _p(maj), _p(tf), tf.shape[0],
                            domain[0], domain[1], base_density, _p(_f32(org)), _p(_f32(direction)), tmax,
                            C.byref(st), C.byref(t), _p(P), _p(alb))
    return bool(h), t.value, P, alb, st.value


def iso_hit(scalars, origin, spacing, cells_per_mc, ranges, iso, color, opacity, inst, org, direction, tmax,
            seed_state):
    """MCIsoSurfaceAccel::isProg with an AnariMatte material for one ray:
    (hit, new seed state, t, P, N as 3 uint16 halfs, albedo + alpha)."""
    scalars = _f32(scalars)
    dims, o, sp = _geom(scalars, origin, spacing)
    st = C.c_uint64(seed_state)
    t = C.c_float(0.0)
    P = np.zeros(3, np.float32)
    Nh = np.zeros(3, np.uint16)
    alb = np.zeros(4, np.float32)
    h = lib().ref_iso_hit(_p(scalars), _p(dims), _p(o), _p(sp), cells_per_mc, _p(_f32(ranges)), iso,
                          _p(_f32(color)), opacity, inst, _p(_f32(org)), _p(_f32(direction)), tmax, C.byref(st),
                          C.byref(t), _p(P), _p(Nh), _p(alb))
    return bool(h), st.value, t.value, P, Nh, alb


def lambertian(color, Ng, wo, wi, a: int, b: int) -> np.ndarray:
    """The reference's AnariMatte Lambertian: eval value[3], eval pdf,
    pdf(wi), scatter dir[3], scatter pdf, f_r[3]."""
    out = np.zeros(12, np.float32)
    lib().ref_lambertian(_p(_f32(color)), _p(_f32(Ng)), _p(_f32(wo)), _p(_f32(wi)), a, b, _p(out))
    return out


_lib_ms = None


def _shade_lib(multi: bool) -> C.CDLL:
    """The default build's pin (lib()) or the multi-scatter build's
    (_ref/libbarney_ref_ms.so: the shading step compiled with
    BARNEY_USE_MULTI_SCATTERING=1)."""
    global _lib_ms
    from oracle import OrcShadePath, OrcShadeWorld
    L = lib()
    if multi:
        if _lib_ms is None:
            _lib_ms = C.CDLL(str(LIB.parent / "libbarney_ref_ms.so"))
            _lib_ms.ref_shade_multi_scatter.restype = C.c_int
        L = _lib_ms
    fn = L.ref_bounce
    fn.restype = None
    fn.argtypes = [C.POINTER(OrcShadeWorld), C.c_int, C.POINTER(OrcShadePath), C.POINTER(OrcShadePath), C.c_void_p]
    assert L.ref_shade_multi_scatter() == (1 if multi else 0)
    return L


def bounce(world, multi: bool, depth: int, path):
    """The reference's bounce() of the default or the multi-scatter build on
    oracle.OrcShadeWorld / OrcShadePath records: (path afterwards, shadow
    ray, fragment); the inputs are copied."""
    from oracle import OrcShadePath
    L = _shade_lib(multi)
    io = OrcShadePath.from_buffer_copy(path)
    sh = OrcShadePath()
    frag = np.zeros(3, np.float32)
    L.ref_bounce(C.byref(world), depth, C.byref(io), C.byref(sh), _p(frag))
    return io, sh, frag


def mc_ranges(scalars) -> np.ndarray:
    """StructuredData::buildMCs' scalar ranges (8-cell macrocells), as an
    (nmc, 2) array."""
    scalars = _f32(scalars)
    nz, ny, nx = scalars.shape
    m = [(d - 1 + 7) // 8 for d in (nx, ny, nz)]
    out = np.zeros((m[0] * m[1] * m[2], 2), np.float32)
    lib().ref_mc_ranges(_p(scalars), _p(np.array([nx, ny, nz], np.int32)), _p(out))
    return out


def camera_commit(pos, direction, up, fovy) -> np.ndarray:
    """The reference's PerspectiveCamera::commit: dir_00, dir_du, dir_dv,
    lens_00 as a (4, 3) array."""
    out = np.zeros(12, np.float32)
    lib().ref_camera_commit(_p(_f32(pos)), _p(_f32(direction)), _p(_f32(up)), fovy, _p(out))
    return out.reshape(4, 3)


def generate(pos, direction, up, fovy, W, H, accum_id, bg):
    """The reference's _generateRays: (H, W, 11) rays, (H, W) seed states
    and the count of pixels with a path state other than (1, 0)."""
    out = np.zeros((H, W, 11), np.float32)
    seeds = np.zeros((H, W), np.uint64)
    bad = lib().ref_generate(_p(_f32(pos)), _p(_f32(direction)), _p(_f32(up)), fovy, W, H, accum_id,
                             _p(_f32(bg)), _p(out), _p(seeds))
    return out, seeds, bad


def env_cdfs(texels, addr) -> tuple:
    """EnvMapLight::computeCDFs' tables: cdf_y (H), cdf_x (H*W)."""
    texels = _f32(texels)
    H, W, _ = texels.shape
    cy, cx = np.empty(H, np.float32), np.empty(H * W, np.float32)
    lib().ref_env_cdfs(_p(texels), _p(np.array([W, H], np.int32)), _p(np.asarray(addr, np.int32)), _p(cy), _p(cx))
    C.CDLL(None).fflush(None)  # the border address mode prints a line per lookup (Texture.cpp:79)
    return cy, cx


def rgba8(rgba, srgb: bool) -> np.ndarray:
    rgba = _f32(rgba).reshape(-1, 4)
    out = np.empty(rgba.shape[0], np.uint32)
    lib().ref_rgba8(_p(rgba), rgba.shape[0], 1 if srgb else 0, _p(out))
    return out
