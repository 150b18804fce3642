"""bench.py's multi-process logic on CPU: world size 2 over gloo (127.0.0.1).

Replicas only: each rank times its own frames; the job's time is the slowest rank's,
taken with an all-reduce MAX, and the job's rate counts every rank's pixels. The
reference arm runs on rank 0 alone; other ranks exit without work."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(0.5 + rank, dist, "cpu")      # rank 1 is slower
    rate = bench.whole_job_rate(world, 2073600, 5, t) / 1e6
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, t, rate))


def test_max_over_ranks_and_job_rate_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [1.5, 1.5]
    assert res[0][2] == pytest.approx(2 * 2073600 * 5 / 1.5 / 1e6)


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.25, None, "cpu") == 0.25
    assert bench.whole_job_rate(1, 100, 4, 2.0) == 200.0


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, ROOT)
    import bench

    class A:
        workload, steps, warmup = "mandelbox_1080p", 1, 3
    assert bench.run_reference(A(), rank=1, world=2) == 0
