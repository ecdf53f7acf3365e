"""Multi-GPU sweep on CPU: the members split over the ranks of a world of
two gloo processes with no exchange but the reductions of the timing and
the error maxima (max over ranks) and of the step counts (sum)."""
import os

import pytest


def test_shard_partitions_and_balances():
    from filament_gb import sweep
    params = sweep.draw(64, 0)
    for world in (1, 2, 4, 8):
        parts = [sweep.shard(params, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        loads = [sum(sweep.step_cost(params[i]) for i in p) for p in parts]
        biggest = max(sweep.step_cost(p) for p in params)
        assert max(loads) - min(loads) <= biggest
    with pytest.raises(ValueError):
        sweep.shard(params, 2, 2)


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "filament.jl_gb300"))
    from filament_gb import sweep
    params = sweep.draw(64, 0)
    mine = sweep.shard(params, rank, world)
    got = [None] * world
    dist.all_gather_object(got, mine)
    # the bench's reductions: wall time and error maxima by MAX, steps by SUM
    t = torch.tensor([1.0 + rank, 1e-6 * (rank + 1)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(len(mine))], dtype=torch.float64)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    out.put((rank, got, t.tolist(), float(n[0])))
    dist.destroy_process_group()


def test_shards_over_two_gloo_ranks():
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    (r0, g0, t0, n0), (r1, g1, t1, n1) = res
    assert g0 == g1 and sorted(g0[0] + g0[1]) == list(range(64))
    assert t0 == t1 == [2.0, 2e-6]
    assert n0 == n1 == 64.0


def _bench_rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "filament.jl_gb300"), root):
        sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from filament_gb import sweep

    class FailingSweep:
        # the failure is made on the host: creating the batch raises on
        # every rank, with or without a GPU
        def __init__(self, *a, **k):
            raise RuntimeError("injected batch creation failure")

    sweep.Sweep = FailingSweep
    r = bench.time_sweep(n=4, steps=2, warmup=1, rank=rank, world=world, dist=dist)
    out.put((rank, r))
    dist.destroy_process_group()


def test_sharded_sweep_makes_the_same_collectives_after_an_error():
    """Every rank fails to create its batch (a failure injected on the
    host); all ranks still reach the barrier and the reductions, and report
    the error instead of waiting on each other."""
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_bench_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=300) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r in res:
        assert r["ranks"] == 2 and "injected" in r["error"]
