"""CPU, world_size 2 over gloo: a block scan sharded by outer-index range equals the whole scan.

Each rank scans its own slice with the CPU oracle (the device path is the same slice through
es_launch); survivors and stage counts are gathered over gloo and merged on rank 0.  This covers
the host logic of bench.py --gpus N and of any multi-process driver without a GPU."""
import os
import sys

import pytest


def _worker(rank, world, port, k, t, n_outer, out):
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for p in (os.path.join(root, "erdos-selfridge_gb300"), os.path.join(root, "oracle")):
        sys.path.insert(0, p)
    import es_oracle as O
    import es_plan
    import es_shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    plan = es_plan.Plan(k)
    a, b = es_shard.shard_range(0, n_outer, rank, world)
    s, c, _ = O.scan_c(plan, t, o_range=(a, b), threads=1)
    got = [None] * world
    dist.all_gather_object(got, (s, c))
    if rank == 0:
        surv, counts = es_shard.merge(got)
        out.put((surv, counts, es_shard.least_good(plan, t, surv, es_plan.is_admissible)))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("k,t", [(120, 0), (70, 9)])
def test_two_rank_shard_equals_whole(k, t):
    import multiprocessing as mp
    import socket
    import es_oracle as O
    import es_plan
    plan = es_plan.Plan(k)
    n_outer = plan.R // plan.radix[0]
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, k, t, n_outer, q)) for r in range(2)]
    for p in procs:
        p.start()
    surv, counts, least = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ws, wc, _ = O.scan_c(plan, t, o_range=(0, n_outer))
    assert surv == ws and counts == wc


def test_shard_range_tiles():
    import es_shard
    for n, world in ((0, 3), (1, 4), (10, 3), (12345, 7)):
        parts = [es_shard.shard_range(5, 5 + n, r, world) for r in range(world)]
        assert parts[0][0] == 5 and parts[-1][1] == 5 + n
        assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
    with pytest.raises(ValueError):
        es_shard.shard_range(0, 10, 3, 3)
