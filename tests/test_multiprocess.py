"""Multi-process host logic on CPU with the gloo backend (world size 2):
the ensemble's scenario sharding (one rank per GPU, no exchange) and the
bench's reductions over ranks."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "anuga-cuda_gb300")]
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from anuga_cuda import scenarios
    from anuga_cuda.ensemble import shard
    import bench
    specs = scenarios.ensemble_harbour_specs(40, seed=4)
    work = [sp[2] ** 1.5 for sp in specs]
    mine = shard(work, rank, world)
    # every rank learns every shard: together they partition the scenarios
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    load = sum(work[i] for i in mine)
    (mx,) = bench.reduce_over_ranks([load], dist, "max")
    (tot,) = bench.reduce_over_ranks([load], dist, "sum")
    q.put((rank, gathered, mx, tot, sum(work)))
    dist.barrier()
    dist.destroy_process_group()


def test_sharding_and_reductions_gloo():
    pytest.importorskip("torch.distributed")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, mx, tot, total_work in res:
        a, b = gathered
        assert sorted(a + b) == list(range(40)) and not set(a) & set(b)
        assert abs(tot - total_work) <= 1e-9 * total_work
        # longest-processing-time first keeps the busiest rank near half
        assert mx <= 0.6 * total_work
    assert res[0][1] == res[1][1]


def test_shard_is_deterministic_and_complete():
    from anuga_cuda.ensemble import shard
    work = [5.0, 1.0, 3.0, 3.0, 2.0, 8.0, 1.0]
    parts = [shard(work, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == list(range(7))
    assert parts == [shard(work, r, 3) for r in range(3)]
