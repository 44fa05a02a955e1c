"""The multi-GPU form of this path is replicas only (independent grids, no
data-path collective).  Its host logic -- the max-over-ranks time and the
whole-job throughput of bench.py -- runs here as two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local = 0.010 + 0.002 * rank          # seconds of this replica
    slowest = bench.max_over_ranks(local, world, device="cpu")
    value = bench.job_mlups(1000, 50, world, slowest)
    dist.barrier()
    out.put((rank, slowest, value))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_whole_job():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, slowest, value in res:
        assert slowest == pytest.approx(0.012)
        assert value == pytest.approx(2 * 1000 * 50 / 0.012 / 1e6)


def test_single_process_needs_no_collective():
    import bench
    assert bench.max_over_ranks(0.5, 1) == 0.5
    assert bench.job_mlups(10, 2, 1, 1.0) == pytest.approx(2e-5)
