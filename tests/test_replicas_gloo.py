"""The multi-GPU form of the path is replicas: every rank registers its own
movies and the job rate is the world size over the slowest rank's time per
movie.  Checked here with two gloo ranks on the CPU (no GPU, no NCCL)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_local = 0.040 + 0.010 * rank          # seconds per movie on this rank
        t_job = bench.slowest_rank(t_local, dist, "cpu")
        out[rank] = (t_job, world / t_job)
    finally:
        dist.destroy_process_group()


def test_job_rate_is_world_over_slowest_rank():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    t_job, rate = out[0]
    assert t_job == pytest.approx(0.050)
    assert rate == pytest.approx(2 / 0.050)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.slowest_rank(0.04) == 0.04
