"""The ANARI parameter translation (include/gbv_anari.h) on the CPU: the
transferFunction1D RGBA map against a float32 restatement of the reference
device's loop (anari/Volume.cpp:129-170), the density scale, the
structuredRegular bounds and the rejected inputs."""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import anari as A

f32 = np.float32


def restated_map(color, opacity, uniform_color=(1, 1, 1, 1), opacity_param=1.0):
    uc = [f32(v) for v in uniform_color]
    uop = f32(opacity_param) * uc[3]
    nc = 1 if color is None else color.shape[0]
    no = 1 if opacity is None else opacity.shape[0]
    n = max(nc, no)
    out = np.empty((n, 4), np.float32)
    for i in range(n):
        cp = f32(f32(i) / f32(n - 1)) * f32(nc - 1) if n > 1 else f32(0)
        cf = cp - np.floor(cp)
        c0 = [uc[0], uc[1], uc[2], uop]
        c1 = list(c0)
        if color is not None:
            k0, k1 = int(np.floor(cp)), int(np.ceil(cp))
            if color.shape[1] == 3:
                c0 = [color[k0, 0], color[k0, 1], color[k0, 2], uop]
                c1 = [color[k1, 0], color[k1, 1], color[k1, 2], uop]
            else:
                c0 = list(color[k0])
                c1 = list(color[k1])
        c = [(f32(1) - cf) * f32(a) + cf * f32(b) for a, b in zip(c0, c1)]
        if opacity is not None:
            ap = f32(f32(i) / f32(n - 1)) * f32(no - 1) if n > 1 else f32(0)
            af = ap - np.floor(ap)
            a0, a1 = opacity[int(np.floor(ap))], opacity[int(np.ceil(ap))]
            c[3] = c[3] * ((f32(1) - af) * a0 + af * a1)
        out[i] = c
    return out


@pytest.mark.parametrize("case", ["vec3+opacity", "vec4", "opacity_only", "vec4+opacity", "single"])
def test_rgba_map_matches_the_reference_loop(case):
    rng = np.random.default_rng(3)
    col3 = rng.random((5, 3)).astype(np.float32)
    col4 = rng.random((7, 4)).astype(np.float32)
    op9 = rng.random(9).astype(np.float32)
    kw = {}
    if case == "vec3+opacity":
        color, opacity = col3, op9
    elif case == "vec4":
        color, opacity = col4, None
    elif case == "opacity_only":
        color, opacity = None, rng.random(3).astype(np.float32)
        kw = dict(uniform_color=(0.2, 0.4, 0.6, 0.8), opacity_param=0.5)
    elif case == "vec4+opacity":
        color, opacity = col4, rng.random(13).astype(np.float32)
    else:
        color, opacity = None, None
        kw = dict(uniform_color=(0.3, 0.5, 0.7, 1.0), opacity_param=0.25)
    got = A.tf1d_rgba_map(color, opacity, **kw)
    ref = restated_map(color, opacity, **kw)
    assert got.shape == ref.shape
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_identity_maps():
    """A vec4 color array alone, or its RGB with its alpha as the opacity
    array, reproduces the array exactly (the transfer function a bn* app
    would pass directly)."""
    from barney_gb300 import scenes
    tf = scenes.tf_two_peaks(256)
    np.testing.assert_array_equal(A.tf1d_rgba_map(tf).view(np.uint32), tf.view(np.uint32))
    np.testing.assert_array_equal(A.tf1d_rgba_map(np.ascontiguousarray(tf[:, :3]),
                                                  np.ascontiguousarray(tf[:, 3])).view(np.uint32), tf.view(np.uint32))


def test_density_scale_and_bounds():
    assert A.density_scale(0.5) == 2.0
    assert A.density_scale(0.0) == 1.0 and A.density_scale(-3.0) == 1.0
    assert A.density_scale(float(np.float32(1) / np.float32(20))) == 20.0
    lo, hi = A.structured_regular_bounds((65, 33, 9), (-0.5, 0.0, 1.0), (0.25, 0.5, 2.0))
    assert lo.tolist() == [-0.5, 0.0, 1.0] and hi.tolist() == [15.5, 16.0, 17.0]
    lo, hi = A.structured_regular_bounds((4, 4, 4))
    assert lo.tolist() == [0, 0, 0] and hi.tolist() == [3, 3, 3]


def test_rejected_inputs():
    L = A.lib()
    import ctypes as C
    n = C.c_longlong()
    col = np.zeros((4, 2), np.float32)
    assert L.gbv_anari_tf1d_rgba_map(A._p(col), 2, 4, None, 0, None, 1.0, None, C.byref(n)) == N.GBV_ERROR_UNSUPPORTED
    h = C.c_void_p(0)
    assert L.gbv_anari_structured_regular(C.c_void_p(16), 0, 7, C.c_void_p(16), N.ivec(4, 4, 4), None, None,
                                          C.byref(h)) == N.GBV_ERROR_UNSUPPORTED
    assert L.gbv_anari_structured_regular(C.c_void_p(16), 0, 0, None, N.ivec(4, 4, 4), None, None,
                                          C.byref(h)) == N.GBV_ERROR_INVALID_ARGUMENT
    assert "missing required parameter 'data'" in N.lib().gbv_last_error().decode()


# ---- the frame (anari/Frame.cpp) ---------------------------------------------

def test_frame_color_format_is_to_barney():
    from barney_gb300 import anari as A
    from barney_gb300 import bn
    assert A.frame_color_format(A.GBV_ANARI_UFIXED8_VEC4) == bn.BN_UFIXED8_RGBA
    assert A.frame_color_format(A.GBV_ANARI_UFIXED8_RGBA_SRGB) == bn.BN_UFIXED8_RGBA_SRGB
    assert A.frame_color_format(A.GBV_ANARI_FLOAT32) == bn.BN_FLOAT32
    assert A.frame_color_format(A.GBV_ANARI_FLOAT32_VEC3) == bn.BN_FLOAT32 + 2
    assert A.frame_color_format(A.GBV_ANARI_FLOAT32_VEC4) == bn.BN_FLOAT4
    assert A.frame_color_format(A.GBV_ANARI_UINT32) == 0 and A.frame_color_format(A.GBV_ANARI_UNKNOWN) == 0


def test_frame_required_channels():
    """Frame::finalize: color always; depth for a FLOAT32 depth channel, the
    IDs for UINT32 ones, the normal for FLOAT32_VEC3; other types add
    nothing."""
    from barney_gb300 import anari as A
    from barney_gb300 import bn
    assert A.frame_channels() == bn.BN_FB_COLOR
    assert A.frame_channels(depth=A.GBV_ANARI_FLOAT32) == bn.BN_FB_COLOR | bn.BN_FB_DEPTH
    assert A.frame_channels(depth=A.GBV_ANARI_UINT32, primitive_id=A.GBV_ANARI_FLOAT32) == bn.BN_FB_COLOR
    all_ids = A.frame_channels(primitive_id=A.GBV_ANARI_UINT32, object_id=A.GBV_ANARI_UINT32,
                               instance_id=A.GBV_ANARI_UINT32)
    assert all_ids == bn.BN_FB_COLOR | bn.BN_FB_PRIMID | bn.BN_FB_OBJID | bn.BN_FB_INSTID
    assert A.frame_channels(normal=A.GBV_ANARI_FLOAT32_VEC3) == bn.BN_FB_COLOR | 32
