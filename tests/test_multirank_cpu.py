"""Multi-rank host logic of the bench on CPU (gloo, world size 2): the seed
sharding of the disorder sweep, the max-over-ranks timing reduction, and the
reference arm's rank-0-only rule.  The GPU work itself is one independent
replica or shard per rank, with no collective on the data path."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group('gloo', rank=rank, world_size=world)
    mine = bench.shard_units(512, rank, world)
    slowest = bench.dist_reduce(1.0 + rank, world, 'max')
    total = bench.dist_reduce(len(mine), world, 'sum')

    class Args:
        workload = 'c5'
        gpus = world
        steps = 1
        warmup = 3
    # the reference arm: ranks other than 0 leave at once without work
    rc = bench.run_reference(Args()) if rank != 0 else None
    out.put((rank, mine, slowest, total, rc))
    dist.barrier()
    dist.destroy_process_group()


def test_sharding_and_reductions_two_ranks():
    ctx = mp.get_context('spawn')
    out = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        r, mine, slowest, total, rc = out.get(timeout=120)
        res[r] = (mine, slowest, total, rc)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    a, b = set(res[0][0]), set(res[1][0])
    assert not (a & b) and a | b == set(range(512))
    assert res[0][1] == res[1][1] == 2.0
    assert res[0][2] == res[1][2] == 512
    assert res[1][3] == 0
