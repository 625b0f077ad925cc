"""ctypes binding of the native library (include/gbvol.h, include/barney_gb300.h).

The library is built in-tree by barney_gb300.build (or __graft_entry__.build()).
Loading fails loudly when it is missing: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB = Path(__file__).resolve().parent / "_lib" / "libbarney_gb300.so"

GBV_OK = 0
GBV_ERROR_INVALID_ARGUMENT, GBV_ERROR_CUDA, GBV_ERROR_OUT_OF_MEMORY, GBV_ERROR_LIMIT, GBV_ERROR_UNSUPPORTED = 1, 2, 3, 4, 5
GBV_VOXEL_F32, GBV_VOXEL_F16, GBV_VOXEL_BF16, GBV_VOXEL_U8_SCALED = 0, 1, 2, 3
GBV_LAYOUT_LINEAR, GBV_LAYOUT_BRICK_CORNERS, GBV_LAYOUT_NANOVDB = 0, 1, 2
GBV_FB_FLOAT4, GBV_FB_RGBA8, GBV_FB_RGBA8_SRGB = 0, 1, 2
GBV_ADDR_WRAP, GBV_ADDR_CLAMP, GBV_ADDR_BORDER, GBV_ADDR_MIRROR = 0, 1, 2, 3
GBV_NUM_COUNTERS = 12
(GBV_COUNTER_SAMPLES, GBV_COUNTER_MC_VISITS, GBV_COUNTER_RAYS, GBV_COUNTER_CAPS,
 GBV_COUNTER_CELLS) = 0, 1, 2, 3, 4

_f3 = C.c_float * 3
_i3 = C.c_int * 3


class GbvIsoSurface(C.Structure):
    """gbv_iso_surface: an iso-surface of the field with a matte material."""
    _fields_ = [("iso_value", C.c_float), ("d_ranges", C.c_void_p), ("color", C.c_float * 4),
                ("opacity", C.c_float), ("instance", C.c_int), ("user_id", C.c_int)]


class GbvScene(C.Structure):
    _fields_ = [
        ("d_voxels", C.c_void_p), ("d_scale_offset", C.c_void_p),
        ("format", C.c_int), ("layout", C.c_int),
        ("dims", _i3), ("origin", _f3), ("spacing", _f3),
        ("d_majorants", C.c_void_p), ("cells_per_mc", C.c_int),
        ("d_tf", C.c_void_p), ("tf_n", C.c_int), ("domain", C.c_float * 2), ("base_density", C.c_float),
        ("anisotropy", C.c_float), ("scattering_albedo", C.c_float),
        ("cam_pos", _f3), ("cam_dir", _f3), ("cam_up", _f3), ("fovy", C.c_float),
        ("num_dir_lights", C.c_int), ("dir_light_dir", _f3 * 4), ("dir_light_color", _f3 * 4),
        ("dir_light_radiance", C.c_float * 4),
        ("d_env_texels", C.c_void_p), ("d_env_cdf_y", C.c_void_p), ("d_env_cdf_x", C.c_void_p),
        ("env_dims", C.c_int * 2), ("env_addr", C.c_int * 2), ("env_dir", _f3), ("env_up", _f3),
        ("env_scale", C.c_float),
        ("bg_color", C.c_float * 4), ("ambient_radiance", C.c_float),
        ("multi_scatter", C.c_int), ("volume_multi_scatter", C.c_int), ("max_volume_bounces", C.c_int),
        ("brick_log2", _i3),
        ("nanovdb", C.c_void_p),
        ("iso", C.c_void_p), ("volume_instance", C.c_int), ("volume_user_id", C.c_int),
        ("d_depth", C.c_void_p), ("d_prim_id", C.c_void_p), ("d_inst_id", C.c_void_p), ("d_obj_id", C.c_void_p),
    ]


GBV_STAGE_DEFAULT, GBV_STAGE_NONE, GBV_STAGE_ALL, GBV_STAGE_BALLOT = 0, 1, 2, 3
GBV_RENDER_PERSISTENT, GBV_RENDER_WAVEFRONT = 0, 1


class GbvRenderConfig(C.Structure):
    """gbv_render_config: launch settings (zero fields take the defaults)."""
    _fields_ = [("blocks_per_sm", C.c_int), ("threshold_pct", C.c_int), ("skip_cells", C.c_int),
                ("stage", C.c_int), ("profile", C.c_int), ("mode", C.c_int),
                ("reserved", C.c_int * 2)]


def render_config(**kw) -> GbvRenderConfig:
    c = GbvRenderConfig()
    for k, v in kw.items():
        setattr(c, k, int(v))
    return c


class GbvEAView(C.Structure):
    _fields_ = [("pos", _f3), ("dir", _f3), ("up", _f3), ("fovy", C.c_float),
                ("width", C.c_int), ("height", C.c_int)]


_lib = None


def lib() -> C.CDLL:
    """The loaded native library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not _LIB.exists():
            raise RuntimeError(f"native library missing: {_LIB} (run __graft_entry__.build())")
        L = C.CDLL(str(_LIB))
        vp, st, i, f = C.c_void_p, C.c_int, C.c_int, C.c_float
        ip = C.POINTER(C.c_int)
        sig = {
            "gbv_last_error": (C.c_char_p, []),
            "gbv_version": (i, []),
            "gbv_mc_dims": (st, [ip, i, ip]),
            "gbv_build_mc_ranges": (st, [vp, ip, i, vp, vp]),
            "gbv_build_mc_ranges_from_store": (st, [vp, vp, i, ip, i, vp, vp]),
            "gbv_map_majorants": (st, [vp, i, vp, i, f, f, f, vp, vp]),
            "gbv_brick_store_bytes": (st, [ip, i, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
            "gbv_build_brick_store": (st, [vp, ip, i, vp, vp, vp]),
            "gbv_brick_store_bytes_shaped": (st, [ip, i, ip, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
            "gbv_build_brick_store_shaped": (st, [vp, ip, i, ip, vp, vp, vp]),
            "gbv_build_mc_ranges_from_store_shaped": (st, [vp, vp, i, ip, ip, i, vp, vp]),
            "gbv_env_build_cdfs": (st, [vp, i, i, ip, vp, vp, vp]),
            "gbv_render": (st, [C.POINTER(GbvScene), vp, i, i, i, i, vp, vp]),
            "gbv_render_ex": (st, [C.POINTER(GbvScene), vp, i, i, i, i, vp, C.POINTER(GbvRenderConfig), vp]),
            "gbv_render_noalloc": (st, [C.POINTER(GbvScene), vp, i, i, i, i, vp, vp]),
            "gbv_render_tiles": (st, [C.POINTER(GbvScene), vp, i, i, i, i, i, i, vp, vp]),
            "gbv_tile_partition": (st, [i, i, i, i, ip, ip]),
            "gbv_selftest_sincos": (st, [vp, C.c_longlong, vp, vp, i, vp]),
            "gbv_selftest_angles": (st, [vp, vp, C.c_longlong, vp, vp, i, vp]),
            "gbv_normalize_texels": (st, [vp, i, C.c_longlong, vp, vp]),
            "gbv_compressed_tile_bytes": (C.c_size_t, []),
            "gbv_compress_tiles": (st, [vp, i, i, i, i, i, vp, vp]),
            "gbv_unpack_tiles": (st, [vp, i, i, i, i, i, vp, vp]),
            "gbv_iso_intersect": (st, [C.POINTER(GbvScene), vp, C.c_float, vp, C.c_longlong, vp, vp]),
            "gbv_batch_create": (st, [C.POINTER(GbvScene), vp, ip, ip, i, C.POINTER(vp)]),
            "gbv_batch_set_launch": (st, [vp, i, i, i]),
            "gbv_batch_render": (st, [vp, i, i, vp, vp]),
            "gbv_batch_destroy": (st, [vp]),
            "gbv_tonemap": (st, [vp, i, i, i, i, vp, vp]),
            "gbv_ea_render": (st, [C.POINTER(GbvScene), C.POINTER(GbvEAView), i, f, vp, vp]),
            "gbv_ea_render_f64": (st, [C.POINTER(GbvScene), C.POINTER(GbvEAView), i, f, vp, vp]),
            "gbv_ea_backward": (st, [C.POINTER(GbvScene), C.POINTER(GbvEAView), i, f, vp, vp, vp, vp, vp]),
            "gbv_ea_backward_ex": (st, [C.POINTER(GbvScene), C.POINTER(GbvEAView), i, f, vp, vp, vp, vp, i, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class GbvError(RuntimeError):
    pass


def check(status: int, what: str = "") -> None:
    if status != GBV_OK:
        msg = lib().gbv_last_error().decode(errors="replace")
        raise GbvError(f"{what} failed with status {status}: {msg}")


def ivec(*v) -> C.Array:
    return (C.c_int * len(v))(*[int(x) for x in v])
