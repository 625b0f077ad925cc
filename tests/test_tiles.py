"""The frame partition across ranks (the reference's round-robin 32x32
tiles) and its gather, run as two gloo ranks on the CPU; the batch split."""
import os
import socket

import numpy as np
import pytest

from barney_gb300 import tiles


@pytest.mark.parametrize("W,H,R", [(1, 1, 1), (100, 70, 3), (1920, 1080, 8), (31, 33, 2), (64, 64, 5), (40, 30, 7)])
def test_partition_covers_each_tile_once_round_robin(W, H, R):
    tx, ty = -(-W // 32), -(-H // 32)
    seen = []
    for r in range(R):
        low = tiles.tile_partition(W, H, r, R)
        # TiledFB::resize: numActiveTilesThisGPU = ceil(max(0, total - rank) / size)
        assert len(low) == max(0, -(-(tx * ty - r) // R))
        ids = [int(y // 32) * tx + int(x // 32) for x, y in low]
        assert ids == list(range(r, tx * ty, R))  # setTileCoordsKernel: tid * size + rank
        seen += ids
    assert sorted(seen) == list(range(tx * ty))


def test_partition_rejects_bad_ranks():
    from barney_gb300 import _native as N
    with pytest.raises(RuntimeError):
        tiles.tile_partition(64, 64, 2, 2)
    with pytest.raises(RuntimeError):
        tiles.tile_partition(64, 64, 0, 0)
    assert "rank" in N.lib().gbv_last_error().decode() or "bad" in N.lib().gbv_last_error().decode()


def test_pack_unpack_round_trip():
    import torch
    f = torch.arange(45 * 70 * 4, dtype=torch.float32).reshape(45, 70, 4)
    out = torch.full_like(f, -1.0)
    for r in range(3):
        low = tiles.tile_partition(70, 45, r, 3)
        tiles.unpack_tiles(out, tiles.pack_tiles(f, low), low)
    assert torch.equal(out, f)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, result_path):
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # every rank "renders" only its tiles of a deterministic frame; the
        # rest of its frame buffer holds a value that must not survive
        H, W = 75, 101
        full = torch.from_numpy(np.random.default_rng(3).random((H, W, 4), dtype=np.float32))
        mine = torch.full_like(full, float("nan") if rank else -7.0)
        low = tiles.tile_partition(W, H, rank, world)
        tiles.unpack_tiles(mine, tiles.pack_tiles(full, low), low)
        got = tiles.gather_frame(mine, rank, world)
        if rank == 0:
            np.save(result_path, got.numpy())
            np.save(result_path + ".ref.npy", full.numpy())
        else:
            assert got is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_gather_frame_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "frame.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    ref = np.load(out + ".ref.npy")
    np.testing.assert_array_equal(got, ref)


def test_shard_items_covers_and_balances():
    from barney_gb300 import scenes
    items = scenes.batch_items(64)
    w = [s.width * s.height * s.spp for s in items]
    for R in (1, 2, 3, 8):
        parts = tiles.shard_items(w, R)
        assert sorted(i for p in parts for i in p) == list(range(64))
        loads = [sum(w[i] for i in p) for p in parts]
        # greedy heaviest-first: no rank exceeds the mean by more than one item
        assert max(loads) - sum(w) / R <= max(w)
