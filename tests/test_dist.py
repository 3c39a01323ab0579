"""Multi-process (gloo, world size 2) tests of the replica/shard host logic
used by bench.py for N > 1: every instance is simplified by exactly one rank
and the per-rank results reduce to the single-process totals."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402

from parafrost_gb300.dist import allreduce_max, allreduce_sum, shard, shard_range  # noqa: E402


def test_shard_range_partitions():
    for n in range(0, 23):
        for w in range(1, 6):
            got = [i for r in range(w) for i in shard_range(n, r, w)]
            assert got == list(range(n))
            sizes = [len(shard_range(n, r, w)) for r in range(w)]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, jobs, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import parafrost_gb300 as pg
    from oracle import pyoracle as po
    processed, mx = 0, 0.0
    for (v, c, seed) in shard(jobs, rank, world):
        r = po.simplify(pg.random_ksat(v, c, 3, seed), pg.options_from())
        processed += sum(s["clauses_before"] for s in r.round_stats)
        mx = max(mx, float(seed))
    tot = allreduce_sum(processed)
    m = allreduce_max(mx)
    if rank == 0:
        out.put((tot, m))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_reduce_to_single_process_totals():
    import parafrost_gb300 as pg
    from oracle import pyoracle as po
    jobs = [(300 + 20 * i, (300 + 20 * i) * 4, i + 1) for i in range(7)]
    single = 0
    for (v, c, seed) in jobs:
        r = po.simplify(pg.random_ksat(v, c, 3, seed), pg.options_from())
        single += sum(s["clauses_before"] for s in r.round_stats)
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, jobs, q)) for r in range(2)]
    for p in procs:
        p.start()
    tot, m = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert tot == single
    assert m == float(len(jobs))
