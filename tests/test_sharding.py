"""CPU: sharding of independent systems and right-hand sides across ranks,
including a two-rank gloo process group (host-side scatter/gather only)."""
import os
import socket

import numpy as np
import pytest

from spme_gb300.sharding import partition, run_sharded, split_rhs, system_cost


def test_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    costs = list(rng.uniform(1, 100, 64))
    for world in (1, 2, 3, 8):
        parts = partition(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= sum(costs) / world + max(costs) + 1e-9
    assert partition(costs, 4) == partition(costs, 4)  # deterministic


def test_split_rhs():
    assert split_rhs(16, 4) == [(0, 4), (4, 8), (8, 12), (12, 16)]
    assert split_rhs(5, 2) == [(0, 3), (3, 5)]
    assert split_rhs(1, 3) == [(0, 1), (1, 1), (1, 1)]


def test_system_cost_orders_by_size():
    assert system_cost(50000, 100, 8, 4) > system_cost(500, 24, 4, 4)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _systems():
    rng = np.random.default_rng(7)
    out = []
    for k in range(6):
        n = int(rng.integers(20, 60))
        L = 8.0 + k
        out.append(dict(pos=rng.uniform(0, L, (n, 3)), f=rng.standard_normal((1, 3 * n)), L=L,
                        K=12 + 2 * (k % 3), p=4, xi=0.8))
    return out


def _apply(sysd):
    import oracle
    return oracle.recip(sysd["pos"], sysd["L"], sysd["xi"], sysd["K"], sysd["p"], sysd["f"],
                        nthreads=1)


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    systems = _systems()
    costs = [system_cost(s["pos"].shape[0], s["K"], s["p"], 1) for s in systems]
    res = run_sharded(systems, costs, _apply, dist)
    if rank == 0:
        np.savez(out_path, *res)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_gather(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "res.npz")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    serial = [_apply(s) for s in _systems()]
    assert len(got.files) == len(serial)
    for k, ref in enumerate(serial):
        assert np.array_equal(got[f"arr_{k}"], ref)
