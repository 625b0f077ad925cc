"""The frame and the batch split across ranks (one GPU per rank).

Frames: the reference's tiled frame buffer cuts a frame into 32x32-pixel
tiles, row-major, and gives rank r of R the tiles r, r + R, r + 2R, ...
(barney/fb/TiledFB.cu:226-255).  Each rank renders its tiles with
gbv_render_tiles; gather_frame is the one exchange step, bringing every
rank's tiles to the root (the reference's LocalFB::gatherColorChannel,
barney/fb/LocalFB.cpp:60-70, and DistFB over MPI).

Batches: independent (volume, view) items are shared out whole by
shard_items; there is no exchange on the data path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

TILE = 32


def tile_partition(width: int, height: int, rank: int, world: int) -> np.ndarray:
    """(k, 2) int array: lower-left pixel (x, y) of each 32x32 tile `rank`
    owns, in the order the rank renders them (gbv_tile_partition)."""
    n = C.c_int()
    N.check(N.lib().gbv_tile_partition(width, height, rank, world, C.byref(n), None), "gbv_tile_partition")
    out = np.zeros((max(n.value, 1), 2), np.int32)
    N.check(N.lib().gbv_tile_partition(width, height, rank, world, C.byref(n),
                                       out.ctypes.data_as(C.POINTER(C.c_int))), "gbv_tile_partition")
    return out[: n.value]


def pack_tiles(frame, lowers):
    """The owned tiles of a (H, W, 4) frame as one (k, 32, 32, 4) tensor (the
    part of a tile past the frame's edge is zero)."""
    import torch
    H, W, ch = frame.shape
    out = torch.zeros((len(lowers), TILE, TILE, ch), dtype=frame.dtype, device=frame.device)
    for k, (x, y) in enumerate(lowers):
        h, w = min(TILE, H - y), min(TILE, W - x)
        out[k, :h, :w] = frame[y:y + h, x:x + w]
    return out


def unpack_tiles(frame, tiles, lowers) -> None:
    """Writes packed tiles back into their places in the (H, W, 4) frame."""
    H, W, _ = frame.shape
    for k, (x, y) in enumerate(lowers):
        h, w = min(TILE, H - y), min(TILE, W - x)
        frame[y:y + h, x:x + w] = tiles[k, :h, :w]


def compress_tiles(accum, accum_id: int, rank: int, world: int):
    """The tiles `rank` owns of a (H, W, 4) CUDA accumulation frame in the
    compressed tile format (gbv_compress_tiles): a (k, 6144) uint8 tensor."""
    import torch
    from .device import _ptr, _stream
    H, W, _ = accum.shape
    k = len(tile_partition(W, H, rank, world))
    nb = int(N.lib().gbv_compressed_tile_bytes())
    out = torch.empty((max(k, 1), nb), dtype=torch.uint8, device=accum.device)
    N.check(N.lib().gbv_compress_tiles(_ptr(accum.contiguous()), W, H, accum_id, rank, world, _ptr(out), _stream()),
            "gbv_compress_tiles")
    return out[:k]


def unpack_tiles_into(out, tiles, rank: int, world: int, fmt: int = N.GBV_FB_FLOAT4) -> None:
    """Writes `rank`'s compressed tiles into the (H, W, 4) float32 (FLOAT4) or
    (H, W) int32 (RGBA8) CUDA frame `out` (gbv_unpack_tiles)."""
    from .device import _ptr, _stream
    H, W = out.shape[0], out.shape[1]
    if len(tiles) == 0:
        return
    N.check(N.lib().gbv_unpack_tiles(_ptr(tiles.contiguous()), W, H, rank, world, fmt, _ptr(out), _stream()),
            "gbv_unpack_tiles")


def gather_frame(frame, rank: int, world: int, root: int = 0, group=None, compress: bool = False,
                 accum_id: int = 1):
    """Brings every rank's owned tiles of its (H, W, 4) frame to `root`,
    which returns the assembled frame; other ranks return None.  One gather
    of fixed-size buffers (each rank pads its tile list to the largest
    rank's), so it runs on any torch.distributed backend that has gather.
    compress=True (CUDA frames): ships the compressed tile format (6 bytes a
    pixel instead of 16) and returns the read colour, accumulation / accum_id,
    as DistFB's gather does."""
    import torch
    import torch.distributed as dist
    H, W, ch = frame.shape
    if compress:
        most = len(tile_partition(W, H, 0, world))
        mine = compress_tiles(frame, accum_id, rank, world)
        buf = torch.zeros((max(most, 1), int(N.lib().gbv_compressed_tile_bytes())), dtype=torch.uint8,
                          device=frame.device)
        buf[: len(mine)] = mine
        bufs = [torch.empty_like(buf) for _ in range(world)] if rank == root else None
        dist.gather(buf, bufs, dst=root, group=group)
        if rank != root:
            return None
        out = torch.zeros((H, W, 4), dtype=torch.float32, device=frame.device)
        for r in range(world):
            unpack_tiles_into(out, bufs[r][: len(tile_partition(W, H, r, world))], r, world)
        return out
    most = len(tile_partition(W, H, 0, world))  # rank 0 owns the most tiles
    mine = tile_partition(W, H, rank, world)
    buf = torch.zeros((most, TILE, TILE, ch), dtype=frame.dtype, device=frame.device)
    if len(mine):
        buf[: len(mine)] = pack_tiles(frame, mine)
    bufs = [torch.empty_like(buf) for _ in range(world)] if rank == root else None
    dist.gather(buf, bufs, dst=root, group=group)
    if rank != root:
        return None
    out = frame.clone()
    for r in range(world):
        lowers = tile_partition(W, H, r, world)
        unpack_tiles(out, bufs[r][: len(lowers)], lowers)
    return out


def shard_items(weights, world: int) -> list:
    """Splits items of the given costs (e.g. pixels x passes) across `world`
    ranks: heaviest first, each to the least-loaded rank (the lowest rank on
    ties).  Returns one sorted index list per rank."""
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    order = sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i))
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(weights[i])
    return [sorted(p) for p in parts]
