"""State sharding across ranks, checked with two gloo ranks on CPU."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from create_rate_subs_gb300.shard import shard_range


@pytest.mark.parametrize("n", [0, 1, 7, 1000, 2 ** 20 + 3])
@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_slabs_cover_every_state_once(n, world):
    spans = [shard_range(n, r, world) for r in range(world)]
    assert spans[0][0] == 0 and spans[-1][1] == n
    for (a, b), (c, d) in zip(spans, spans[1:]):
        assert b == c
    sizes = [b - a for a, b in spans]
    assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    a, b = shard_range(n, rank, world)
    # each rank "evaluates" its slab: a per-state checksum
    idx = torch.arange(a, b, dtype=torch.float64)
    local = torch.tensor([float((idx * 3.0 + 1.0).sum()), float(b - a)], dtype=torch.float64)
    dist.all_reduce(local)
    if rank == 0:
        out.put((float(local[0]), float(local[1])))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_cover_the_batch():
    n, world = 12345, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    total, count = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert count == n
    assert total == float(np.sum(np.arange(n) * 3.0 + 1.0))
