"""Iso-surface worlds on the GPU: an iso_surface geometry with a matte
material, alone or beside the volume in either instance order, rendered
through gbv_render, gbv_render_noalloc and bn*, bit for bit with the oracle.

The surface's diffuse scatter takes a sine and cosine of its azimuth, so the
oracle runs in its bounded-math mode (the library's routines restated);
everything else on the surface path is float arithmetic shared with the
reference (tests/test_oracle_refpin.py pins the iso intersection program and
the Lambertian against the reference's own code).
"""
import ctypes as C

import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import bn, scenes
from barney_gb300.device import GpuScene, _ptr, _stream
import oracle

pytestmark = pytest.mark.gpu

ISO = 0.3
KINDS = {
    "iso-only": dict(instance=0, volume_instance=0, no_volume=True),
    "iso-first": dict(instance=0, volume_instance=1, no_volume=False),
    "volume-first": dict(instance=1, volume_instance=0, no_volume=False),
}


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def iso_scene(kind, multi=False, env=False, dims=48, w=64, h=48, spp=4, color=(0.9, 0.6, 0.3, 1.0), opacity=1.0):
    k = KINDS[kind]
    if multi:
        s = scenes.frame_scene(dims=dims, width=w, height=h, spp=spp, with_env=False)
        if env:
            s.env = scenes.env_sky(64, 32)
    else:
        s = scenes.small_scene(dims=dims, spp=spp, width=w, height=h)
    s.iso = scenes.IsoSurface(ISO, color, opacity, k["instance"])
    s.volume_instance = k["volume_instance"]
    s.no_volume = k["no_volume"]
    return s


def gpu_render(s, layout=N.GBV_LAYOUT_BRICK_CORNERS, fmt=N.GBV_VOXEL_F32, spp=None, start=0, acc=None):
    import torch
    g = GpuScene(s, layout=layout, fmt=fmt)
    counters = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    acc = g.new_accum() if acc is None else torch.from_numpy(acc).cuda()
    g.render(spp=spp, accum=acc, accum_id_start=start, counters=counters)
    torch.cuda.synchronize()
    return acc.cpu().numpy(), counters.cpu().numpy()


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("build", ["single", "multi-env"])
def test_iso_world_bit_exact(cuda, kind, build):
    s = iso_scene(kind, multi=build != "single", env=build != "single")
    got, c = gpu_render(s)
    o = oracle.Oracle(s, bounded_math=True)
    ref = o.render()
    np.testing.assert_array_equal(bits(got), bits(ref))
    assert c[N.GBV_COUNTER_CAPS] == 0
    assert c[N.GBV_COUNTER_RAYS] == o.stats["rays"]
    if kind == "iso-first":
        # the kernel traces the volume before searching the surface (same
        # hits and streams), so it takes the samples past the surface that
        # the oracle, bounding the volume by the surface first, does not;
        # macrocell counts differ either way (the oracle's bounded tracking
        # walks on to the grid's exit, the kernel's stops at its collision)
        assert c[N.GBV_COUNTER_SAMPLES] >= o.stats["density_samples"]
    else:
        assert c[N.GBV_COUNTER_SAMPLES] == o.stats["density_samples"]
        assert c[N.GBV_COUNTER_MC_VISITS] == o.stats["mc_visits"]
    if kind == "iso-only":
        assert c[N.GBV_COUNTER_SAMPLES] == 0
    # the surface is in the picture: frames differ from the volume-only world
    plain = iso_scene(kind, multi=build != "single", env=build != "single")
    plain.iso, plain.no_volume, plain.volume_instance = None, False, 0
    base, _ = gpu_render(plain)
    assert (np.abs(got - base).max(axis=2) > 1e-3).mean() > 0.05


def test_iso_instance_order_changes_the_streams(cuda):
    a, _ = gpu_render(iso_scene("iso-first"))
    b, _ = gpu_render(iso_scene("volume-first"))
    assert not np.array_equal(bits(a), bits(b))


@pytest.mark.parametrize("opacity,alpha", [(0.7, 1.0), (1.0, 0.5)])
def test_translucent_matte(cuda, opacity, alpha):
    s = iso_scene("iso-first", color=(0.2, 0.7, 0.4, alpha), opacity=opacity)
    got, _ = gpu_render(s)
    ref = oracle.Oracle(s, bounded_math=True).render()
    np.testing.assert_array_equal(bits(got), bits(ref))


@pytest.mark.parametrize("layout,fmt,u8", [(N.GBV_LAYOUT_LINEAR, N.GBV_VOXEL_F32, False),
                                           (N.GBV_LAYOUT_BRICK_CORNERS, N.GBV_VOXEL_U8_SCALED, True)])
def test_iso_world_other_stores(cuda, layout, fmt, u8):
    s = iso_scene("iso-first")
    got, _ = gpu_render(s, layout=layout, fmt=fmt)
    ref = oracle.Oracle(s, bounded_math=True, u8=u8).render()
    np.testing.assert_array_equal(bits(got), bits(ref))


def test_iso_world_progressive(cuda):
    s = iso_scene("volume-first", multi=True, env=True)
    got, _ = gpu_render(s, spp=3)
    got, _ = gpu_render(s, spp=2, start=3, acc=got)
    o = oracle.Oracle(s, bounded_math=True)
    ref = o.render(spp=3)
    o.render(spp=2, accum=ref, accum_id_start=3)
    np.testing.assert_array_equal(bits(got), bits(ref))


def test_iso_world_noalloc(cuda):
    import torch
    s = iso_scene("iso-first", multi=True, env=True)
    want, _ = gpu_render(s)
    g = GpuScene(s)
    acc = g.new_accum()
    rec = g.record()
    st = N.lib().gbv_render_noalloc(C.byref(rec), _ptr(acc), s.width, s.height, 0, s.spp, None, _stream())
    assert st == N.GBV_OK, N.lib().gbv_last_error()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bits(acc.cpu().numpy()), bits(want))


def test_iso_world_rejected_where_unsupported(cuda):
    s = iso_scene("iso-first")
    g = GpuScene(s)
    acc = g.new_accum()
    rec = g.record()
    cfg = N.render_config(mode=N.GBV_RENDER_WAVEFRONT)
    st = N.lib().gbv_render_ex(C.byref(rec), _ptr(acc), s.width, s.height, 0, 1, None, C.byref(cfg), _stream())
    assert st == N.GBV_ERROR_UNSUPPORTED and "wavefront" in N.lib().gbv_last_error().decode()
    # the iso-surface and the volume need distinct instances
    rec.volume_instance = 0
    N.GbvIsoSurface.from_address(rec.iso).instance = 0
    st = N.lib().gbv_render(C.byref(rec), _ptr(acc), s.width, s.height, 0, 1, None, _stream())
    assert st == N.GBV_ERROR_INVALID_ARGUMENT


@pytest.mark.parametrize("kind", list(KINDS))
def test_bn_iso_surface_matches_oracle(cuda, kind):
    """bnGeometryCreate("iso_surface") + bnMaterialCreate("matte") through
    bn*: the same frame as the oracle's, including the instance order the
    groups give (one group: the iso-surface first; its own later group:
    the volume first)."""
    s = iso_scene(kind, multi=True, env=True)
    with bn.BarneySession() as ses:
        err = ses.build_scene(s, s.scalars.ctypes.data)
        assert err == "", err
        ses.render()
        img = ses.read()
        o = oracle.Oracle(s, bounded_math=True)
        ref = o.tonemap(o.render(), s.spp)
        np.testing.assert_array_equal(img.view(np.uint32), ref.view(np.uint32))


def test_bn_iso_surface_needs_a_committed_material(cuda):
    s = iso_scene("iso-only")
    with bn.BarneySession() as ses:
        L = ses.L
        ses.build_scene(s, s.scalars.ctypes.data)
        geom = ses.handles["geom"]
        mat = L.bnMaterialCreate(ses.ctx, 0, b"matte")  # never committed
        L.bnSetObject(geom, b"material", mat)
        ses.render()
        assert "committed material" in bn.last_error()
        assert not L.bnMaterialCreate(ses.ctx, 0, b"physicallyBased")
        assert not L.bnGeometryCreate(ses.ctx, 0, b"triangles")
