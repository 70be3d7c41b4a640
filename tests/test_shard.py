"""Replica sharding across ranks, on CPU with gloo (world size 2): slicing, per-rank
convolution and the host gather. The local convolution is the oracle here (the GPU
version of the same call runs in bench.py under torchrun)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from convfpga_gb300.shard import shard_range


@pytest.mark.parametrize("how_many,world", [(0, 2), (1, 2), (3, 2), (4, 2), (7, 3), (5, 8)])
def test_shard_range_partitions_the_batch(how_many, world):
    seen = []
    lens = []
    for r in range(world):
        first, count = shard_range(how_many, r, world)
        seen.extend(range(first, first + count))
        lens.append(count)
    assert seen == list(range(how_many))
    assert max(lens) - min(lens) <= 1


def test_shard_range_rejects_bad_ranks():
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)
    with pytest.raises(ValueError):
        shard_range(-1, 0, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, how_many, per_signal, q):
    import torch.distributed as dist

    from convfpga_gb300 import FILTER_PER_SIGNAL
    from convfpga_gb300.shard import sharded_batch
    from oracle import conv3d

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n = 16
        rng = np.random.default_rng(5)
        sig = (rng.uniform(-1, 1, (how_many, n, n, n)) + 1j * rng.uniform(-1, 1, (how_many, n, n, n))).astype(np.complex64)
        fshape = (how_many, n, n, n) if per_signal else (n, n, n)
        filt = (rng.uniform(-1, 1, fshape) + 1j * rng.uniform(-1, 1, fshape)).astype(np.complex64)
        calls = []

        def local(n_, s, f, out, count, flags):
            calls.append(count)
            out[...] = conv3d(s, f, "fp32", engine="pocketfft")

        flags = FILTER_PER_SIGNAL if per_signal else 0
        full = sharded_batch(n, sig, filt, how_many, flags, conv=local)
        if rank == 0:
            ref = conv3d(sig, filt, "fp32", engine="pocketfft")
            q.put(("ok", float(np.max(np.abs(full - ref))), calls))
        else:
            q.put(("rank1", None, calls))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("how_many,per_signal", [(3, False), (4, True), (1, False)])
def test_two_rank_gloo_batch(how_many, per_signal):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, how_many, per_signal, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    r0 = [r for r in results if r[0] == "ok"]
    assert len(r0) == 1 and r0[0][1] == 0.0
    counts = sorted(sum(r[2]) for r in results)
    assert sum(counts) == how_many
