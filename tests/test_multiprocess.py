"""The multi-rank bench path on CPU: two gloo ranks on 127.0.0.1 run the
barrier and max-over-ranks timing helpers bench.py uses around its timed
region."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    w, r, loc, pg = bench.dist_setup()
    assert (w, r) == (world, rank)
    bench.barrier(pg)
    out[rank] = bench.max_over_ranks(pg, float(rank + 1) * 10.0)
    pg.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_take_the_max():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(100)
        assert p.exitcode == 0
    assert out[0] == out[1] == 20.0


def _shard_rank(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "mojo-petsc4py_gb300"))
    import torch.distributed as dist
    from mojopetsc4py.batch import shard_systems

    dist.init_process_group("gloo", rank=rank, world_size=world)
    costs = [((s * 7919) % 97 + 1) * 16 for s in range(64)]
    mine = shard_systems(costs, world)[rank]
    got = [None] * world
    dist.all_gather_object(got, mine)
    out[rank] = got
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_batched_systems_shard_across_two_gloo_ranks():
    """Each rank derives its shard of the batch on its own; the shards agree,
    cover every system once and balance nnz * nrhs within the largest cost."""
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(100)
        assert p.exitcode == 0
    assert out[0] == out[1]
    shards = out[0]
    allsys = sorted(s for sh in shards for s in sh)
    assert allsys == list(range(64))
    costs = [((s * 7919) % 97 + 1) * 16 for s in range(64)]
    loads = [sum(costs[s] for s in sh) for sh in shards]
    assert abs(loads[0] - loads[1]) <= max(costs)
