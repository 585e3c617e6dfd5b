"""The bench's host logic on the CPU: the N > 1 path (replicas as gloo ranks, world size 2, each rank's timings
reduced to the slowest rank's, as bench.py does around its timed region) and the roofline arithmetic of the pair
kernels and the LU."""
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


def test_rooflines_of_the_pair_kernels():
    # the 25k wing's per-tier point counts and phase times of one step: the dominant kernel and its figures
    sys.path.insert(0, ROOT)
    import bench

    pts = {"self": 115813152, "edge": 59978016, "vertex": 46096344, "contact": 1747470186, "near": 1218703101,
           "far": 2319825171}
    per = {"far": 102.5, "near": 174.2, "near_pairs": 451.5, "lu": 133.5, "adj_far": 198.3, "adj_near": 481.7,
           "adj_pairs": 2135.2, "setup": 0.9, "wake": 0.0}
    kernels, roof = bench.rooflines(per, pts, pts, 12824, ({"sm_max_mhz": 2070.0}, "measured"))
    touch = 115813152 + 59978016 + 46096344 + 1747470186
    assert roof["kernel"] == "adj_pairs_kernel<AdjAccW>"
    assert abs(roof["achieved"] - touch * (bench.FLOP_ADJ_EVAL + 2 * bench.FLOP_ADJ_SUMS) / 2.1352 / 1e12) < 1e-9
    assert abs(roof["peak"] - 152 * 128 * 2 * 2070e6 / 1e12) < 1e-9
    assert abs(roof["frac"] - roof["achieved"] / roof["peak"]) < 1e-15
    assert abs(roof["traffic"] - bench.DRAM_PER_TOUCH_POINT["adj_pairs"] * touch) < 1.0
    assert abs(kernels["far"]["achieved"] - pts["far"] * bench.FLOP_FWD_POINT / 0.1025 / 1e12) < 1e-9
    assert abs(kernels["lu"]["achieved"] - 2 / 3 * 12824 ** 3 / 0.1335 / 1e12) < 1e-9
    assert "wake" not in kernels and set(kernels) == {"far", "near", "near_pairs", "lu", "adj_far", "adj_near",
                                                      "adj_pairs"}
