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


def _gather_rank(rank, world, port, out):
    """Each rank fakes the results of its shard (values that name the system,
    row and column they belong to), gathers them on rank 0 over gloo with the
    bench's helper, and rank 0 reassembles the batch."""
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import sys

    import numpy as np

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "mojo-petsc4py_gb300")]
    import bench
    from mojopetsc4py.batch import assemble_shards, shard_systems

    w, r, _, pg = bench.dist_setup()
    sizes = [3 + (s * 5) % 11 for s in range(40)]
    nrhs = 4
    shards = shard_systems([sz * 9 * nrhs for sz in sizes], w)
    mine = shards[r]
    X = np.concatenate([[[s * 1000 + i + c / 10 for c in range(nrhs)] for i in range(sizes[s])]
                        for s in mine])
    part = {"X": X, "its": np.array([[s * 10 + c for c in range(nrhs)] for s in mine]),
            "reason": np.full((len(mine), nrhs), 2, dtype=np.int32),
            "relres": np.array([[s * 1e-10] * nrhs for s in mine])}
    parts = bench.gather_to_root(pg, part)
    if r == 0:
        Xa, info = assemble_shards(shards, parts, sizes, nrhs)
        out["X"] = Xa.tolist()
        out["its"] = info["its"].tolist()
        out["relres"] = info["relres"].tolist()
    else:
        out[f"none{r}"] = parts is None
    bench.barrier(pg)
    pg.destroy_process_group()


@pytest.mark.timeout(120)
def test_sharded_batch_results_gather_in_system_order():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_gather_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(100)
        assert p.exitcode == 0
    import numpy as np

    sizes = [3 + (s * 5) % 11 for s in range(40)]
    want = np.concatenate([[[s * 1000 + i + c / 10 for c in range(4)] for i in range(sizes[s])]
                           for s in range(40)])
    np.testing.assert_array_equal(np.array(out["X"]), want)
    np.testing.assert_array_equal(np.array(out["its"]),
                                  [[s * 10 + c for c in range(4)] for s in range(40)])
    assert out["none1"] is True


def test_assemble_shards_rejects_a_system_in_two_shards():
    import sys

    import numpy as np

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "mojo-petsc4py_gb300"))
    from mojopetsc4py.batch import assemble_shards

    sizes = [2, 3]
    part = lambda sh: {"X": np.zeros((sum(sizes[s] for s in sh), 1)),  # noqa: E731
                       "its": np.zeros((len(sh), 1)), "reason": np.zeros((len(sh), 1)),
                       "relres": np.zeros((len(sh), 1))}
    with pytest.raises(ValueError):
        assemble_shards([[0, 1], [1]], [part([0, 1]), part([1])], sizes, 1)
    with pytest.raises(ValueError):
        assemble_shards([[0], []], [part([0]), part([])], sizes, 1)
    X, info = assemble_shards([[1], [0]], [part([1]), part([0])], sizes, 1)
    assert X.shape == (5, 1) and info["its"].shape == (2, 1)
