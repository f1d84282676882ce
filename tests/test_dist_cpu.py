"""bench.py's multi-GPU plumbing on CPU: two gloo ranks (replicas, no data-path collective).

Under torchrun each rank serves its own maps; ranks meet only at the barriers around the timed region and
in the max-over-ranks time / sum-over-ranks counter reductions that make the whole-job number.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local, pg = bench.dist_setup()
    bench.barrier(pg)
    mx = bench.allreduce_max(pg, 10.0 * (rank + 1))
    sm = bench.allreduce_sum(pg, float(rank + 1))
    bench.barrier(pg)
    q.put((r, w, local, mx, sm))
    pg.destroy_process_group()


def test_two_gloo_ranks_reduce_like_the_bench():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    for r, w, local, mx, sm in got:
        assert w == 2 and local == r
        assert mx == 20.0 and sm == 3.0


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    r, w, local, pg = bench.dist_setup()
    assert (r, w, local, pg) == (0, 1, 0, None)
    assert bench.allreduce_max(pg, 3.5) == 3.5 and bench.allreduce_sum(pg, 2.0) == 2.0
