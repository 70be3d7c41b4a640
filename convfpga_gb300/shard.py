"""Replica sharding of a convolution batch across host ranks (one GPU per rank).

Convolutions are independent, so a batch shards by signal with no exchange on the data
path: rank r convolves a contiguous slice of the batch on its own GPU and the results
are gathered on the host of rank 0 afterwards. The reference runs one device only
(host/src/fpga_init.c:86 picks devices[0]); this is the multi-GPU form of
fpgaf_conv3D_svm_batch (host/src/convfpga_svm_batch.c:36) for a node with several GPUs.
"""
from __future__ import annotations

from typing import Callable

import numpy as np


def shard_range(how_many: int, rank: int, world: int) -> tuple[int, int]:
    """(first, count) of the slice of `how_many` signals that rank `rank` convolves.

    Slices are contiguous and differ in length by at most one; every signal belongs to
    exactly one rank, and ranks beyond `how_many` get an empty slice.
    """
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    if how_many < 0:
        raise ValueError("how_many must be >= 0")
    base, extra = divmod(how_many, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def sharded_batch(n: int, sig: np.ndarray, filt: np.ndarray, how_many: int, flags: int, group=None,
                  conv: Callable | None = None) -> np.ndarray | None:
    """Convolves this rank's slice of the batch and gathers every slice on rank 0.

    sig: (how_many, n, n, n) complex64 host array (each rank may hold the full batch or
    only its slice at the same offsets); filt: (n, n, n), or (how_many, n, n, n) with
    FILTER_PER_SIGNAL. `conv(n, sig_slice, filt_slice, out_slice, count, flags)` performs
    the local convolution; it defaults to the library's host-buffer entry point
    (convgpu_conv3d_host). Returns the full (how_many, n, n, n) result on rank 0, None
    elsewhere. The gather goes through torch.distributed on host tensors (gloo).
    """
    import torch
    import torch.distributed as dist

    from . import FILTER_PER_SIGNAL, conv3d_host, last_error

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    first, count = shard_range(how_many, rank, world)
    out = np.zeros((count, n, n, n), np.complex64)
    if count:
        s = np.ascontiguousarray(sig[first:first + count])
        f = np.ascontiguousarray(filt[first:first + count]) if flags & FILTER_PER_SIGNAL else np.ascontiguousarray(filt)
        if conv is None:
            t = conv3d_host(n, s, f, out, count, flags)
            if not t.valid:
                raise RuntimeError(f"convgpu_conv3d_host failed on rank {rank}: {last_error()}")
        else:
            conv(n, s, f, out, count, flags)
    # Variable-length slices: pad to the longest slice for the fixed-size gather.
    longest = shard_range(how_many, 0, world)[1]
    buf = torch.zeros((longest, n, n, n, 2), dtype=torch.float32)
    if count:
        buf[:count] = torch.from_numpy(out.view(np.float32).reshape(count, n, n, n, 2))
    gathered = [torch.zeros_like(buf) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, gathered, dst=0, group=group)
    if rank != 0:
        return None
    full = np.empty((how_many, n, n, n), np.complex64)
    for r in range(world):
        f0, c = shard_range(how_many, r, world)
        if c:
            full[f0:f0 + c] = gathered[r][:c].numpy().view(np.complex64).reshape(c, n, n, n)
    return full
