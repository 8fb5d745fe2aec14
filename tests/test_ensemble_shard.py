"""Instance sharding of an ensemble across ranks (CPU, gloo, world size 2).

The partition must be deterministic, disjoint and complete, and balanced on
the ensemble workload's seeded instances; the gather must give rank 0 the
same per-instance results as a single-rank run; a rank that fails before
the gather must make rank 0's gather fail with an error instead of hanging.
The per-instance work here is a host function (the GPU batch runs in the
GPU tests): only the host logic of the multi-rank path is under test."""
import os
import socket

import numpy as np
import pytest

from schrodingersem_gb300 import ensemble as ens


def _workload_costs(count=1024, seed=2026):
    """the ensemble workload's instance sizes: n ~ U{4..32}, p in {4,6,8}"""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(4, 33))
        p = int(rng.choice([4, 6, 8]))
        rng.integers(1 << 30)
        out.append(ens.instance_cost(n * n, p))
    return out


def test_shard_disjoint_complete_balanced():
    costs = _workload_costs()
    for world in (1, 2, 3, 4, 8):
        parts = ens.shard(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        assert ens.shard(costs, world) == parts  # deterministic
        assert ens.imbalance(costs, parts) < 1.02, (world, ens.imbalance(costs, parts))


def test_shard_more_ranks_than_instances():
    parts = ens.shard([3.0, 1.0], 4)
    assert parts == [[0], [1], [], []]
    with pytest.raises(ValueError):
        ens.shard([1.0], 0)


def _fake_result(i):
    return {"converged": i % 7 != 3, "steps": 100, "iterations": 30 + i % 11, "norm": 1.0 + 1e-12 * i}


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, costs, fail_rank, q):
    import datetime

    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    try:
        def run_share(idx):
            if rank == fail_rank:
                raise RuntimeError("injected failure of this rank's share")
            return {i: _fake_result(i) for i in idx}
        out = ens.run_sharded(costs, rank, world, run_share, dist)
        q.put((rank, "ok", out))
    except Exception as e:  # reported to the test, never swallowed
        q.put((rank, "error", repr(e)))
    finally:
        if fail_rank < 0:
            dist.destroy_process_group()


def _run(world, fail_rank):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    costs = _workload_costs(96)
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, costs, fail_rank, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(world):
        r, status, out = q.get(timeout=120)
        res[r] = (status, out)
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    return costs, res


def test_gather_matches_single_rank_gloo():
    costs, res = _run(2, -1)
    assert res[0][0] == "ok" and res[1][0] == "ok"
    assert res[1][1] is None
    single = ens.run_sharded(costs, 0, 1, lambda idx: {i: _fake_result(i) for i in idx})
    assert res[0][1] == single


def test_failed_rank_makes_gather_fail_not_hang():
    _, res = _run(2, 1)
    assert res[1][0] == "error" and "injected failure" in res[1][1]
    assert res[0][0] == "error"  # rank 0's gather ended with an error (peer gone or timeout)
