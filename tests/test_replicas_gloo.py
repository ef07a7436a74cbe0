"""The multi-GPU path of bench.py is independent replicas (no data-path collective): each rank
runs its own frames and the job's throughput is all frames over the slowest rank's time.
Checked here with two gloo ranks on the CPU."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        value, job_ms = bench.replica_throughput(100.0 + 50.0 * rank, 4, dist, "cpu")
        dist.barrier()
        out[rank] = (value, job_ms)
    finally:
        dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    # every rank sees the slowest rank's time and counts all ranks' frames
    for r in range(world):
        value, job_ms = res[r]
        assert job_ms == pytest.approx(150.0)
        assert value == pytest.approx(4 * world / 0.150)


def test_replica_throughput_single_process():
    import bench

    value, job_ms = bench.replica_throughput(200.0, 5)
    assert job_ms == 200.0 and value == pytest.approx(25.0)
