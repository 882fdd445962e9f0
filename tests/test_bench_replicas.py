"""The bench's N > 1 path on the CPU: two gloo ranks stand in for two GPUs.
Each rank times its own replica; the job's time is the max over ranks and
the whole-job throughput counts every rank's views (weak scaling)."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, ms_local, q):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.job_time_ms(ms_local[rank], world, torch.device("cpu"))
    q.put((rank, ms, bench.replica_value(ms, world, 16, 20)))
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_report_the_slowest_rank_and_the_whole_job():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ms_local = [10.0, 14.0]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, ms_local, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in out:
        assert ms == 14.0
        assert abs(value - 2 * 16 * 20 / 0.014) < 1e-6


def test_single_replica_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_time_ms(12.5, 1, None) == 12.5
    assert bench.replica_value(12.5, 1, 16, 20) == 16 * 20 / 0.0125
