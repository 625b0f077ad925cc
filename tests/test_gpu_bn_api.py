"""The barney-compatible bn* API on the GPU: host buffers in, host image out,
identical to the gbv path and to the oracle."""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import bn, scenes
from barney_gb300.device import GpuScene
import oracle

pytestmark = pytest.mark.gpu


def test_bn_render_matches_oracle(cuda):
    s = scenes.small_scene(dims=48, spp=4, width=64, height=48)
    with bn.BarneySession() as ses:
        err = ses.build_scene(s, s.scalars.ctypes.data, frame_stats=True)
        assert err == "", err
        ses.render()
        img = ses.read()
        assert ses.stats()[0] > 0
        o = oracle.Oracle(s)
        ref = o.tonemap(o.render(), 4)
        np.testing.assert_array_equal(img.view(np.uint32), ref.view(np.uint32))
        # a second bnRender accumulates 4 more passes, as the reference does
        ses.render()
        img2 = ses.read()
        acc = o.render()
        o.render(spp=4, accum=acc, accum_id_start=4)
        np.testing.assert_array_equal(img2.view(np.uint32), o.tonemap(acc, 8).view(np.uint32))


@pytest.mark.parametrize("fmt", [bn.BN_UFIXED8_RGBA, bn.BN_UFIXED8_RGBA_SRGB])
def test_bn_fixed8_formats(cuda, fmt):
    s = scenes.small_scene(dims=32, spp=2, width=40, height=30)
    with bn.BarneySession() as ses:
        ses.build_scene(s, s.scalars.ctypes.data, color_format=fmt)
        ses.render()
        img = ses.read()
        o = oracle.Oracle(s)
        ref = o.tonemap(o.render(), 2, fmt=1 if fmt == bn.BN_UFIXED8_RGBA else 2)
        d = np.abs(img.view(np.uint8).astype(int) - ref.view(np.uint8).astype(int))
        assert d.max() <= (0 if fmt == bn.BN_UFIXED8_RGBA else 1)


@pytest.mark.parametrize("brick", [None, (4, 4, 2)])
def test_bn_multi_scatter_env_matches_gbv_path(cuda, brick):
    import torch
    s = scenes.frame_scene(dims=40, width=48, height=32, spp=4)
    s.env = scenes.env_sky(64, 32)
    with bn.BarneySession() as ses:
        ses.build_scene(s, s.scalars.ctypes.data, voxel_format=N.GBV_VOXEL_F16, brick=brick)
        ses.render()
        img = ses.read()
    g = GpuScene(s, fmt=N.GBV_VOXEL_F16)
    ref = g.tonemap(g.render(), 4).cpu().numpy()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(img.view(np.uint32), ref.view(np.uint32))


def test_bn_errors_are_recorded(cuda):
    with bn.BarneySession() as ses:
        L = ses.L
        assert not L.bnScalarFieldCreate(ses.ctx, 0, b"unstructured")
        assert "not supported" in bn.last_error()
        assert not L.bnLightCreate(ses.ctx, 0, b"quad")
        fb = L.bnFrameBufferCreate(ses.ctx, 0)
        L.bnFrameBufferResize(fb, 123, 8, 8, 1)
        assert "unsupported color format" in bn.last_error()
    # a new context starts without a recorded failure
    with bn.BarneySession():
        assert bn.last_error() == ""


def test_bn_scene_rebuilds_reuse_context_memory(cuda):
    """Scenes built and released one after another on one context (as an app
    that uploads a new volume every frame does) render the same frame each
    time; their device buffers come from the context's memory pool."""
    s = scenes.small_scene(dims=24, spp=2, width=40, height=24)
    frames = []
    with bn.BarneySession() as ses:
        for _ in range(3):
            assert ses.build_scene(s, s.scalars.ctypes.data) == ""
            ses.render()
            frames.append(ses.read().copy())
            ses.release_scene()
    for f in frames[1:]:
        np.testing.assert_array_equal(f.view(np.uint32), frames[0].view(np.uint32))


@pytest.mark.parametrize("bits", [8, 16])
def test_bn_integer_texels_normalised_on_device(cuda, bits):
    """UFIXED8/UFIXED16 fields read v/255 or v/65535 (normalised texture
    reads): the frame equals the one of the FP32 field holding those values."""
    s = scenes.small_scene(dims=40, spp=2, width=48, height=40)
    top = 255 if bits == 8 else 65535
    q = np.round(s.scalars * top).astype(np.uint8 if bits == 8 else np.uint16)
    f = (q.astype(np.float32) / np.float32(top)).astype(np.float32)
    fmt = bn.BN_UFIXED8 if bits == 8 else bn.BN_UFIXED16
    with bn.BarneySession() as ses:
        ses.build_scene(s, q.ctypes.data, texel_format=fmt)
        ses.render()
        got = ses.read()
        ses.release_scene()
        ses.build_scene(s, np.ascontiguousarray(f).ctypes.data)
        ses.render()
        ref = ses.read()
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_bn_progressive_accumulation_and_reset(cuda):
    """Two bnRender calls of 3 paths each accumulate like one 6-pass frame
    (accumIDs 0..5); bnAccumReset starts over (the reference's
    FrameBuffer::accumID bookkeeping)."""
    import torch
    s = scenes.small_scene(dims=40, spp=3, width=48, height=40)
    with bn.BarneySession() as ses:
        ses.build_scene(s, s.scalars.ctypes.data)
        ses.render()
        ses.render()
        two = ses.read()
        ses.L.bnAccumReset(ses.handles["fb"])
        ses.render()
        one = ses.read()
    g = GpuScene(s)
    acc = g.render(spp=3)
    g.render(spp=3, accum=acc, accum_id_start=3)
    ref6 = g.tonemap(acc, 6).cpu().numpy()
    ref3 = g.tonemap(g.render(spp=3), 3).cpu().numpy()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(two.view(np.uint32), ref6.view(np.uint32))
    np.testing.assert_array_equal(one.view(np.uint32), ref3.view(np.uint32))


@pytest.mark.parametrize("anari", ["vec4", "vec3+opacity"])
def test_anari_translation_renders_the_bn_frame(cuda, anari):
    """A structuredRegular field and a transferFunction1D volume made by the
    ANARI parameter translation (include/gbv_anari.h) from the scene's data,
    colors (and opacities) and unitDistance = 1 / base density render the
    frame the direct bn* calls render, bit for bit (single and multiple
    scattering)."""
    for s in (scenes.small_scene(dims=40, spp=3, width=48, height=40),
              scenes.frame_scene(dims=40, width=48, height=32, spp=3)):
        frames = []
        for via in (None, anari):
            with bn.BarneySession() as ses:
                err = ses.build_scene(s, s.scalars.ctypes.data, anari=via)
                assert err == "", err
                ses.render()
                frames.append(ses.read())
        np.testing.assert_array_equal(frames[0].view(np.uint32), frames[1].view(np.uint32))
        assert float(frames[0][..., :3].sum()) > 0
