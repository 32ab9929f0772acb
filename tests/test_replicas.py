"""The multi-process path of bench.py on CPU: two gloo ranks. Replicas share nothing
on the data path; the only exchange is the max-over-ranks of the timed region, and the
job throughput counts every rank's rays against the slowest rank's time."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out_dir):
    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(times[rank], dist, "cpu")
        value = bench.job_rays_per_s(4096, 10, world, ms)
        # Replicas draw their own data: rank r seeds with r.
        g = torch.Generator().manual_seed(rank)
        sample = torch.rand(4, generator=g)
        gathered = [torch.zeros(4) for _ in range(world)]
        dist.all_gather(gathered, sample)
        torch.save({"ms": ms, "value": value, "distinct": not torch.equal(gathered[0], gathered[1])},
                   os.path.join(out_dir, f"rank{rank}.pt"))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_report_the_slowest_rank(tmp_path):
    times = [120.0, 150.0]
    mp.spawn(_rank_main, args=(2, _free_port(), times, str(tmp_path)), nprocs=2, join=True)
    res = [torch.load(tmp_path / f"rank{r}.pt") for r in range(2)]
    for r in res:
        assert r["ms"] == pytest.approx(150.0)
        assert r["value"] == pytest.approx(4096 * 10 * 2 / 0.150)
        assert r["distinct"]


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(7.5, None, "cpu") == 7.5
    assert bench.job_rays_per_s(4096, 200, 1, 1000.0) == pytest.approx(4096 * 200)
