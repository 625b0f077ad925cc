"""Python binding of the ANARI parameter translation (include/gbv_anari.h).

The reference's ANARI device turns a `structuredRegular` spatial field and a
`transferFunction1D` volume into barney objects; these helpers make the same
bn* objects from the same ANARI parameters, without the ANARI SDK.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _native as N

GBV_ANARI_FLOAT32, GBV_ANARI_UFIXED8, GBV_ANARI_UINT8 = 0, 1, 2
# frame channel element types
(GBV_ANARI_UNKNOWN, GBV_ANARI_UFIXED8_VEC4, GBV_ANARI_UFIXED8_RGBA_SRGB, GBV_ANARI_FLOAT32_VEC3,
 GBV_ANARI_FLOAT32_VEC4, GBV_ANARI_UINT32) = -1, 10, 11, 12, 13, 14

_ready = False


def lib() -> C.CDLL:
    global _ready
    L = N.lib()
    if not _ready:
        vp, i, f, ll = C.c_void_p, C.c_int, C.c_float, C.c_longlong
        sig = {
            "gbv_anari_structured_regular": (i, [vp, i, i, vp, vp, vp, vp, C.POINTER(vp)]),
            "gbv_anari_structured_regular_bounds": (i, [vp, vp, vp, vp, vp]),
            "gbv_anari_tf1d_rgba_map": (i, [vp, i, ll, vp, ll, vp, f, vp, C.POINTER(ll)]),
            "gbv_anari_density_scale": (f, [f]),
            "gbv_anari_transfer_function_1d": (i, [vp, vp, i, ll, vp, ll, vp, f, vp, f, i]),
            "gbv_anari_frame_color_format": (i, [i]),
            "gbv_anari_frame_channels": (C.c_uint32, [i, i, i, i, i]),
            "gbv_anari_frame_resize": (i, [vp, i, i, i, i, i, i, i, i]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _ready = True
    return L


def _p(a) -> C.c_void_p:
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def tf1d_rgba_map(color: Optional[np.ndarray] = None, opacity: Optional[np.ndarray] = None,
                  uniform_color=None, opacity_param: float = 1.0) -> np.ndarray:
    """The transferFunction1D's RGBA map: color (n, 3) or (n, 4) float32 or
    None, opacity (m,) float32 or None."""
    col = None if color is None else np.ascontiguousarray(color, np.float32)
    op = None if opacity is None else np.ascontiguousarray(opacity, np.float32)
    uc = None if uniform_color is None else np.ascontiguousarray(uniform_color, np.float32)
    ch = 0 if col is None else col.shape[1]
    nc = 0 if col is None else col.shape[0]
    no = 0 if op is None else op.shape[0]
    n = C.c_longlong()
    N.check(lib().gbv_anari_tf1d_rgba_map(_p(col), ch, nc, _p(op), no, _p(uc), opacity_param, None, C.byref(n)),
            "gbv_anari_tf1d_rgba_map")
    out = np.empty((n.value, 4), np.float32)
    N.check(lib().gbv_anari_tf1d_rgba_map(_p(col), ch, nc, _p(op), no, _p(uc), opacity_param, _p(out), C.byref(n)),
            "gbv_anari_tf1d_rgba_map")
    return out


def density_scale(unit_distance: float) -> float:
    return lib().gbv_anari_density_scale(unit_distance)


def structured_regular_bounds(dims, origin=None, spacing=None):
    lo, hi = np.empty(3, np.float32), np.empty(3, np.float32)
    o = None if origin is None else np.ascontiguousarray(origin, np.float32)
    s = None if spacing is None else np.ascontiguousarray(spacing, np.float32)
    N.check(lib().gbv_anari_structured_regular_bounds(_p(np.asarray(dims, np.int32)), _p(o), _p(s), _p(lo),
                                                      _p(hi)), "gbv_anari_structured_regular_bounds")
    return lo, hi


def frame_color_format(color_type: int) -> int:
    """The bn color format of an ANARI "channel.color" type (toBarney)."""
    return int(lib().gbv_anari_frame_color_format(color_type))


def frame_channels(depth=GBV_ANARI_UNKNOWN, primitive_id=GBV_ANARI_UNKNOWN, object_id=GBV_ANARI_UNKNOWN,
                   instance_id=GBV_ANARI_UNKNOWN, normal=GBV_ANARI_UNKNOWN) -> int:
    """Frame::finalize's requiredChannels for the frame's channel types."""
    return int(lib().gbv_anari_frame_channels(depth, primitive_id, object_id, instance_id, normal))

