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


def _wdot_worker(rank, world, port, out):
    """One rank: its slab of the golden 53-species states through the
    reference's per-state functions on the host (crs_state_* on a host-only
    handle), then a sum over ranks of the (species, states) array in which
    each rank filled only its own columns (x + 0 is exact)."""
    import ctypes
    from conftest import load_golden
    from create_rate_subs_gb300 import _lib
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mech, g = load_golden("gri53")
    N, R, NREV, NPM = (int(x) for x in g["dims"])
    lib = _lib.load()
    h = ctypes.c_void_p()
    _lib.check(lib.crs_mech_load_host(mech.blob, len(mech.blob), ctypes.byref(h)))
    dp = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    n = g["T"].shape[0]
    a, b = shard_range(n, rank, world)
    full = torch.zeros((N, n), dtype=torch.float64)
    conc, fwd = np.zeros(N), np.zeros(R)
    rev, pm = np.zeros(max(NREV, 1)), np.zeros(max(NPM, 1))
    sp, dyN = np.zeros(N - 1), ctypes.c_double()
    yN, mw, rho = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    for i in range(a, b):
        T, P = float(g["T"][i]), float(g["P"][i])
        y = np.ascontiguousarray(g["Y"][: N - 1, i])
        _lib.check(lib.crs_state_eval_conc(h, T, P, dp(y), ctypes.byref(yN), ctypes.byref(mw),
                                           ctypes.byref(rho), dp(conc)))
        _lib.check(lib.crs_state_eval_rxn_rates(h, T, P, dp(conc), dp(fwd), dp(rev)))
        _lib.check(lib.crs_state_get_rxn_pres_mod(h, T, P, dp(conc), dp(pm)))
        _lib.check(lib.crs_state_eval_spec_rates(h, dp(fwd), dp(rev), dp(pm), dp(sp),
                                                 ctypes.byref(dyN)))
        full[: N - 1, i] = torch.from_numpy(sp)
        full[N - 1, i] = dyN.value
    lib.crs_mech_free(h)
    dist.all_reduce(full)
    if rank == 0:
        out.put((b - a, bool(np.array_equal(full.numpy(), g["wdot"]))))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_evaluate_their_slabs():
    """Two gloo ranks each evaluate their slab of a batch with the host
    per-state functions; the combined species rates equal the reference's
    golden vectors bit for bit."""
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_wdot_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    slab0, exact = q.get(timeout=180)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert slab0 > 0
    assert exact
