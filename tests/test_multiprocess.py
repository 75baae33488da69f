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
