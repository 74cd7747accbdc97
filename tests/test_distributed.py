"""Multi-rank logic of bench.py on CPU ranks (gloo, world size 2): the
max-over-ranks step time and the barrier that bracket the timed region.  The
fit itself shards by cube with no data-path collective, so this is the only
cross-rank code."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import sys
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "REPEAT_BENCH_BACKEND": "gloo"})
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    m = bench.max_over_ranks(1.5 + r, w, "cpu")
    q.put((r, w, m))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(g[0] for g in got) == [0, 1]
    assert all(g[1] == 2 and g[2] == 2.5 for g in got)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25
