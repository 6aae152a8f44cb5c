"""Replica mode of bench.py across ranks (the path does not shard: every GPU
runs its own pings, and only the timing is reduced). Two gloo ranks on the
CPU: the rendezvous on 127.0.0.1 and the max-over-ranks reduction the bench
uses for its timed region."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    w, r, local = bench.dist_env()
    dist = bench.init_dist(w)
    t = bench.max_over_ranks(dist, 0.5 + r)          # each rank's own "timed region"
    dist.barrier()
    q.put((r, local, t))
    dist.destroy_process_group()


def test_two_ranks_reduce_to_the_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r for r, _, _ in res] == [0, 1]
    assert all(t == 1.5 for _, _, t in res)


def test_single_process_needs_no_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.init_dist(1) is None
    assert bench.max_over_ranks(None, 3.0) == 3.0
