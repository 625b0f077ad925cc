"""Auxiliary frame channels on the GPU (gbv_scene.d_depth, d_prim_id,
d_inst_id, d_obj_id): depth and hit IDs of each pixel's primary ray, as the
reference's shading step writes its aux tiles (barney/kernels/shadeRays.cu:
1003-1023) from the closest hit's IDs (barney/volume/MCAccelerator.h:
552-565, 685-700), bit for bit with the oracle -- volume-only worlds,
iso-surface worlds in both instance orders, progressive accumulation."""
import numpy as np
import pytest

from barney_gb300 import scenes
from barney_gb300.device import GpuScene
import oracle

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _aux_gpu(W, H):
    import torch
    return {"depth": torch.full((H, W), -7.0, dtype=torch.float32, device="cuda"),
            "prim_id": torch.full((H, W), 99, dtype=torch.int32, device="cuda"),
            "inst_id": torch.full((H, W), 99, dtype=torch.int32, device="cuda"),
            "obj_id": torch.full((H, W), 99, dtype=torch.int32, device="cuda")}


def _aux_cpu(W, H):
    return {"depth": np.full((H, W), -7.0, np.float32), "prim_id": np.full((H, W), 99, np.int32),
            "inst_id": np.full((H, W), 99, np.int32), "obj_id": np.full((H, W), 99, np.int32)}


def _check(s, chunks, bounded=False):
    """Renders the passes in `chunks` ((start, count) pairs) on both sides and
    compares the frame and the four channels bit for bit."""
    import torch
    g = GpuScene(s)
    acc = g.new_accum()
    ag = _aux_gpu(s.width, s.height)
    o = oracle.Oracle(s, bounded_math=bounded)
    ref = np.zeros((s.height, s.width, 4), np.float32)
    ac = _aux_cpu(s.width, s.height)
    for start, n in chunks:
        g.render(spp=n, accum=acc, accum_id_start=start, aux=ag)
        o.render(spp=n, accum=ref, accum_id_start=start, aux=ac)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bits(acc.cpu().numpy()), bits(ref))
    for k in ac:
        np.testing.assert_array_equal(bits(ag[k].cpu().numpy()), bits(ac[k]), err_msg=k)
    return ac


def test_volume_world_channels():
    s = scenes.frame_scene(dims=40, width=64, height=48, spp=4, with_env=False)
    s.volume_user_id = 11
    ac = _check(s, [(0, 4)])
    hit = ac["prim_id"] == 0
    assert hit.any() and (~hit).any()
    assert np.all(ac["inst_id"][hit] == 0) and np.all(ac["obj_id"][hit] == 11)
    assert np.all(ac["inst_id"][~hit] == -1) and np.all(ac["obj_id"][~hit] == -1)
    assert np.all(ac["depth"] <= np.float32(1e30)) and np.all(ac["depth"][hit] < 1e3)


def test_progressive_keeps_the_nearest_depth_and_the_first_pass_ids():
    s = scenes.frame_scene(dims=40, width=48, height=40, spp=6, with_env=True)
    s.env = scenes.env_sky(64, 32)
    _check(s, [(0, 2), (2, 3), (5, 1)], bounded=True)


@pytest.mark.parametrize("order", ["iso-first", "volume-first"])
def test_iso_world_channels(order):
    s = scenes.small_scene(dims=40, spp=3, width=56, height=40)
    inst = 0 if order == "iso-first" else 1
    s.iso = scenes.IsoSurface(0.3, (0.9, 0.6, 0.3, 1.0), 1.0, inst, user_id=5)
    s.volume_instance = 1 - inst
    s.volume_user_id = 8
    ac = _check(s, [(0, 3)], bounded=True)
    assert set(np.unique(ac["obj_id"])) <= {-1, 5, 8} and (ac["obj_id"] == 5).any()


def test_bn_frame_buffer_channels():
    """bn*: a frame buffer resized with BN_FB_DEPTH | PRIMID | INSTID | OBJID
    gives, after two progressive bnRender calls, the channels of the gbv
    path (the volume's and the iso-surface's "userID" as object IDs); a
    channel not asked for is refused."""
    import torch
    from barney_gb300 import bn
    s = scenes.small_scene(dims=40, spp=2, width=48, height=40)
    s.iso = scenes.IsoSurface(0.3, (0.9, 0.6, 0.3, 1.0), 1.0, 0, user_id=21)
    s.volume_instance, s.volume_user_id = 1, 34
    chans = bn.BN_FB_DEPTH | bn.BN_FB_PRIMID | bn.BN_FB_INSTID | bn.BN_FB_OBJID
    vol = np.ascontiguousarray(s.scalars)
    with bn.BarneySession() as ses:
        assert ses.build_scene(s, vol.ctypes.data, channels=chans) == ""
        ses.render()
        ses.render()
        got = {k: ses.read_channel(c) for k, c in (("depth", bn.BN_FB_DEPTH), ("prim_id", bn.BN_FB_PRIMID),
                                                   ("inst_id", bn.BN_FB_INSTID), ("obj_id", bn.BN_FB_OBJID))}
        assert bn.last_error() == ""
    with bn.BarneySession() as ses:
        assert ses.build_scene(s, vol.ctypes.data) == ""
        ses.render()
        ses.read_channel(bn.BN_FB_DEPTH)
        assert "not requested" in bn.last_error()
    g = GpuScene(s)
    acc = g.new_accum()
    ag = _aux_gpu(s.width, s.height)
    g.render(spp=2, accum=acc, accum_id_start=0, aux=ag)
    g.render(spp=2, accum=acc, accum_id_start=2, aux=ag)
    torch.cuda.synchronize()
    for k in got:
        np.testing.assert_array_equal(bits(got[k]), bits(ag[k].cpu().numpy()), err_msg=k)
    assert set(np.unique(got["obj_id"])) <= {-1, 21, 34} and (got["obj_id"] == 21).any()


def test_anari_frame_resize_and_map():
    """The ANARI frame's channel set-up (gbv_anari_frame_resize: sRGB color,
    FLOAT32 depth, UINT32 object IDs) on a bn* frame buffer, then the
    frame's maps: the color and the two channels asked for read back, the
    instance-ID channel (not asked for) is refused, and a normal channel is
    refused at the resize."""
    from barney_gb300 import anari as A
    from barney_gb300 import bn
    s = scenes.small_scene(dims=32, spp=2, width=40, height=32)
    s.volume_user_id = 9
    vol = np.ascontiguousarray(s.scalars)
    L = A.lib()
    with bn.BarneySession() as ses:
        assert ses.build_scene(s, vol.ctypes.data, color_format=bn.BN_UFIXED8_RGBA_SRGB) == ""
        fb = ses.handles["fb"]
        st = L.gbv_anari_frame_resize(fb, A.GBV_ANARI_UFIXED8_RGBA_SRGB, A.GBV_ANARI_FLOAT32, A.GBV_ANARI_UNKNOWN,
                                      A.GBV_ANARI_UINT32, A.GBV_ANARI_UNKNOWN, A.GBV_ANARI_UNKNOWN, 40, 32)
        assert st == 0
        ses.render()
        img = ses.read()
        depth = ses.read_channel(bn.BN_FB_DEPTH)
        obj = ses.read_channel(bn.BN_FB_OBJID)
        assert bn.last_error() == ""
        ses.read_channel(bn.BN_FB_INSTID)
        assert "not requested" in bn.last_error()
        st = L.gbv_anari_frame_resize(fb, A.GBV_ANARI_FLOAT32_VEC4, A.GBV_ANARI_UNKNOWN, A.GBV_ANARI_UNKNOWN,
                                      A.GBV_ANARI_UNKNOWN, A.GBV_ANARI_UNKNOWN, A.GBV_ANARI_FLOAT32_VEC3, 40, 32)
        assert st != 0
    assert img.shape == (32, 40) and depth.shape == (32, 40)
    hit = obj == 9
    assert hit.any() and (obj[~hit] == -1).all() and (depth[hit] < 1e3).all()
    # a pixel whose first pass missed keeps IDs -1; its depth is 1e30 unless a later pass hit
    assert ((depth[~hit] == np.float32(1e30)) | (depth[~hit] < 1e3)).all()


def test_noalloc_entry_writes_the_same_channels():
    """gbv_render_noalloc with the aux channels in its scene record writes
    the channels gbv_render writes (it allocates nothing for them: the
    caller's buffers are written in place)."""
    import ctypes as C
    import torch
    from barney_gb300 import _native as N
    from barney_gb300.device import _ptr, _stream
    s = scenes.small_scene(dims=32, spp=3, width=40, height=32)
    s.volume_user_id = 6
    g = GpuScene(s)
    want = _aux_gpu(s.width, s.height)
    acc_w = g.render(spp=3, aux=want)
    got = _aux_gpu(s.width, s.height)
    acc = g.new_accum()
    rec = g.record()
    for f, k in (("d_depth", "depth"), ("d_prim_id", "prim_id"), ("d_inst_id", "inst_id"), ("d_obj_id", "obj_id")):
        setattr(rec, f, got[k].data_ptr())
    st = N.lib().gbv_render_noalloc(C.byref(rec), _ptr(acc), s.width, s.height, 0, 3, None, _stream())
    assert st == N.GBV_OK, N.lib().gbv_last_error()
    torch.cuda.synchronize()
    assert torch.equal(acc, acc_w)
    for k in want:
        assert torch.equal(got[k], want[k]), k
    assert (got["obj_id"] == 6).any()
