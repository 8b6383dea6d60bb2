"""Host-side logic of the multi-replica benchmark, run as two gloo ranks on
the CPU: each rank renders its own frame, the job time is the slowest rank's
and the throughput counts every rank's micropolygons."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    assert (r, w, local) == (rank, world, rank)
    ms_max = bench.max_over_ranks(times[rank], dist, torch.device("cpu"))
    value = bench.replica_throughput(1000.0, w, ms_max)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
        f.write("%r %r\n" % (ms_max, value))


def test_two_replicas_take_the_slowest_rank(tmp_path):
    import torch.multiprocessing as mp
    times = [12.5, 20.0]
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, times, str(tmp_path)), nprocs=2, start_method="spawn")
    for rank in range(2):
        ms, value = map(float, (tmp_path / ("rank%d.txt" % rank)).read_text().split())
        assert ms == 20.0
        assert value == pytest.approx(2 * 1000.0 / 0.020)


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        cpu_scale = 0.4
        steps = 3
        warmup = 3

    assert bench.run_reference(A()) == 0


def test_single_process_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import torch
    import bench
    assert bench.max_over_ranks(3.25, None, torch.device("cpu")) == 3.25
    assert bench.replica_throughput(51_200_000, 1, 17.87) == pytest.approx(51_200_000 / 0.01787)
