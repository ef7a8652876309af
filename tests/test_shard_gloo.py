"""Multi-rank sharding (world size 2, gloo on CPU): each rank's jumped start
state and shard concatenate to the one sequential stream, and the timing
reduction takes the max over ranks."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n, q):
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    from mrg8_gb300 import shard
    from oracle import pyoracle as po
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first, count = shard.shard_range(n, rank)
    st = shard.shard_state(13579, first)
    out, _ = po.Oracle().generate(st, count, po.U32)
    gathered = [torch.zeros(count, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(gathered, torch.from_numpy(out.astype(np.int64)))
    mx = shard.max_over_ranks(float(rank + 1), dist)
    if rank == 0:
        q.put((np.concatenate([g.numpy() for g in gathered]).astype(np.uint32), mx))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_concatenate_to_one_stream(lib, oracle):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    n, world = 50_000, 2
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    got, mx = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want, _ = oracle.randint(oracle.seed(13579), n * world)
    assert np.array_equal(got, want)
    assert mx == 2.0


def test_shard_range_validation():
    from mrg8_gb300 import shard
    assert shard.shard_range(10, 3) == (30, 10)
    with pytest.raises(ValueError):
        shard.shard_range(-1, 0)
