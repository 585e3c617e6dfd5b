"""The bench's N > 1 path on the CPU: replicas as gloo ranks (world size 2), each rank's timings reduced to the
slowest rank's, as bench.py does around its timed region."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    r, n, local, dist = bench.dist_setup(world)
    # rank k's step took 1 + k seconds on the device and 10 - k end to end
    out = bench.max_over_ranks([1.0 + rank, 10.0 - rank], dist)
    dist.barrier()
    q.put((r, n, local, out))
    dist.destroy_process_group()


def test_replicas_report_the_slowest_rank():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[:3] for g in got] == [(0, 2, 0), (1, 2, 1)]
    assert all(g[3] == [2.0, 10.0] for g in got)


def test_one_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([3.0, 4.0], None) == [3.0, 4.0]
