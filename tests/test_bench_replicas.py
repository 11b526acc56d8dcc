"""bench.py's replica arithmetic with two gloo ranks on CPU: the job's time is the slowest rank's
and its rays are every rank's (`whole_job`), so the reported throughput is total rays over the
slowest rank's time. CPU only."""
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        rays = [1_000_000, 3_000_000][rank]
        ms = [250.0, 400.0][rank]
        value, t = bench.whole_job(rays, ms, world, "cpu")
        out[rank] = (value, t)
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_total_rays_over_the_slowest_rank():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as manager:
        out = manager.dict()
        mp.start_processes(_rank, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
        results = dict(out)
    for rank in (0, 1):
        value, t = results[rank]
        assert t == 400.0
        assert value == pytest.approx(4_000_000 / 0.4)


def test_one_rank_is_its_own_job():
    import bench
    value, t = bench.whole_job(2_000_000, 500.0, 1, "cpu")
    assert (value, t) == (4_000_000.0, 500.0)
