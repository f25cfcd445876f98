"""The multi-GPU form of the bench is replicas: one process per GPU, each
filtering the same workload with no data-path collective; the whole job's time
is the maximum over ranks and its rate world x the per-rank work over that
time.  The host-side reduction runs here with two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.reduce_max(times[rank], dist, "cpu")
    dist.barrier()
    out.put((rank, t, bench.whole_job_rate(world, 1000, 3, t)))
    dist.destroy_process_group()


def test_replica_time_is_the_slowest_rank():
    ctx = torch.multiprocessing.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    times = [0.75, 0.80]
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in res] == [0, 1]
    for _, t, rate in res:
        assert t == max(times)
        assert rate == pytest.approx(2 * 1000 * 3 / max(times))


def test_single_rank_passes_through():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_max(0.5, None, "cpu") == 0.5
    assert bench.whole_job_rate(1, 65472, 3, 2.0) == pytest.approx(65472 * 3 / 2.0)
