"""The N > 1 path of bench.py (replicas on every rank, barrier, slowest-rank time,
whole-job rate) on two CPU ranks over gloo."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as td
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    td.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        r, w, loc = bench.dist()
        bench.barrier(w)
        ms = bench.max_over_ranks(100.0 + 50.0 * r, w)  # rank 1 is the slower one
        rate = bench.whole_job_rate(16, 3, w, ms)
        out.put((r, w, loc, ms, rate))
        bench.barrier(w)
    finally:
        td.destroy_process_group()


def test_two_gloo_ranks_time_by_the_slowest_and_sum_the_replicas():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, loc, ms, rate) in enumerate(res):
        assert (rank, world, loc) == (r, 2, r)
        assert ms == 150.0
        assert rate == pytest.approx(16 * 3 * 2 / 0.150)
