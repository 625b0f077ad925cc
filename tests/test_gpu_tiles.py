"""gbv_render_tiles: each rank's share of the frame equals the full render
on the tiles it owns, leaves every other pixel alone, and the shares put
together are the frame."""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes, tiles
from barney_gb300.device import GpuScene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("R,multi", [(1, False), (3, False), (4, True), (200, False)])
def test_rank_shares_make_the_frame(cuda, R, multi):
    import torch
    if multi:
        s = scenes.frame_scene(dims=40, width=100, height=70, spp=3)
        s.env = scenes.env_sky(64, 32)
    else:
        s = scenes.small_scene(dims=40, spp=3, width=100, height=70)
    g = GpuScene(s)
    full = g.render()
    full2 = g.render(spp=2, accum=full.clone(), accum_id_start=3)
    cf = torch.zeros(N.GBV_NUM_COUNTERS, dtype=torch.int64, device="cuda")
    g.render(counters=cf)
    assembled = torch.full_like(full, float("nan"))
    csum = torch.zeros_like(cf)
    for r in range(R):
        mine = torch.full_like(full, -3.0)
        c = torch.zeros_like(cf)
        g.render_tiles(r, R, accum=mine, counters=c)
        g.render_tiles(r, R, spp=2, accum=mine, accum_id_start=3)
        csum += c
        low = tiles.tile_partition(s.width, s.height, r, R)
        owned = torch.zeros(full.shape[:2], dtype=torch.bool, device="cuda")
        for x, y in low:
            owned[y:y + 32, x:x + 32] = True
        assert torch.equal(mine[owned], full2[owned])
        assert bool((mine[~owned] == -3.0).all())
        tiles.unpack_tiles(assembled, tiles.pack_tiles(mine, low), low)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(assembled.cpu().numpy().view(np.uint32), full2.cpu().numpy().view(np.uint32))
    assert csum[:5].tolist() == cf[:5].tolist()


def test_render_tiles_rejects_bad_rank(cuda):
    import ctypes as C
    from barney_gb300.device import _ptr, _stream
    s = scenes.small_scene(dims=16, spp=1, width=8, height=8)
    g = GpuScene(s)
    acc = g.new_accum()
    rec = g.record()
    assert N.lib().gbv_render_tiles(C.byref(rec), _ptr(acc), 8, 8, 0, 1, 1, 1, None, _stream()) == 1
    assert N.lib().gbv_render_tiles(C.byref(rec), _ptr(acc), 8, 8, 0, 1, 0, 0, None, _stream()) == 1


def _codec_restated(accum, accum_id, lowers, W, H):
    """The compressed tile format restated with numpy float32 arithmetic:
    per pixel rgb/max(rgb) and alpha as RGBA8, max(rgb) as a ties-away half;
    then unpacked back to float RGBA (DistFB.cu:39-108)."""
    import oracle
    out = np.zeros((H, W, 4), np.float32)
    s = np.float32(1.0) / np.float32(accum_id)
    inv255 = np.float32(1.0) / np.float32(255.0)

    def b8(f):
        with np.errstate(invalid="ignore", over="ignore"):
            v = np.where(np.isnan(f), 0.0, np.trunc(f.astype(np.float64) * 256.0))
        return np.clip(v, 0, 255).astype(np.int64)

    for x0, y0 in lowers:
        blk = accum[y0:y0 + 32, x0:x0 + 32].astype(np.float32) * s
        m = np.maximum(np.maximum(blk[..., 0], blk[..., 1]), blk[..., 2])
        with np.errstate(divide="ignore", invalid="ignore"):
            rs = np.float32(1.0) / m
            rgb = blk[..., :3] * rs[..., None]
        q = np.concatenate([b8(rgb), b8(blk[..., 3:4])], axis=-1)
        half = np.vectorize(lambda f: oracle.float_to_half(float(f)))(m)
        scale = np.vectorize(lambda h: np.float32(np.frombuffer(np.uint16(h).tobytes(), np.float16)[0]))(half)
        c = q.astype(np.float32) * inv255
        c[..., :3] *= scale.astype(np.float32)[..., None]
        out[y0:y0 + 32, x0:x0 + 32] = c
    return out


@pytest.mark.parametrize("R", [1, 3])
def test_compressed_tiles_match_restated_codec(cuda, R):
    import torch
    s = scenes.small_scene(dims=40, spp=3, width=100, height=70)
    g = GpuScene(s)
    acc = g.render()
    out = torch.full((70, 100, 4), -1.0, device="cuda")
    for r in range(R):
        tiles.unpack_tiles_into(out, tiles.compress_tiles(acc, 3, r, R), r, R)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    a = acc.cpu().numpy()
    lowers = np.concatenate([tiles.tile_partition(100, 70, r, R) for r in range(R)])
    ref = _codec_restated(a, 3, lowers, 100, 70)
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
    # against the uncompressed read: one 8-bit step of the pixel's largest channel
    exact = a / 3.0
    top = np.maximum(exact[..., :3].max(axis=-1, keepdims=True), 1e-30)
    assert np.all(np.abs(got[..., :3] - exact[..., :3]) <= top * (1.0 / 255 + 2e-3))


def test_compressed_gather_one_rank(cuda):
    import socket
    import torch
    import torch.distributed as dist
    sock = socket.socket()
    sock.bind(("127.0.0.1", 0))
    port = sock.getsockname()[1]
    sock.close()
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        s = scenes.small_scene(dims=32, spp=2, width=70, height=40)
        g = GpuScene(s)
        acc = g.render()
        got = tiles.gather_frame(acc, 0, 1, compress=True, accum_id=2)
        ref = torch.zeros_like(acc)
        tiles.unpack_tiles_into(ref, tiles.compress_tiles(acc, 2, 0, 1), 0, 1)
        torch.cuda.synchronize()
        assert torch.equal(got, ref)
        plain = tiles.gather_frame(acc, 0, 1)
        assert torch.equal(plain, acc)
    finally:
        dist.destroy_process_group()
