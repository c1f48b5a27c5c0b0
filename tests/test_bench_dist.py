"""bench.py's multi-rank plumbing on CPU (gloo, world size 2): the barrier,
the max-over-ranks timing every rank agrees on, and the whole-job rate the
replicas report (units of all ranks over the slowest rank's time)."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank), "CUDA_VISIBLE_DEVICES": ""})
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist

    r, w = bench.dist_setup()
    assert (r, w) == (rank, world)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    local_ms = 100.0 + 50.0 * r  # rank 1 is the slow one
    ms_max = bench.max_over_ranks(local_ms, w)
    rate = bench.whole_job_rate(10, ms_max, w)
    bench.barrier(w)
    Path(out_dir, f"rank{r}.txt").write_text(f"{ms_max} {rate}")
    dist.destroy_process_group()


def test_two_rank_timing_and_rate(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    for r in range(world):
        ms_max, rate = map(float, (tmp_path / f"rank{r}.txt").read_text().split())
        assert ms_max == 150.0
        assert rate == pytest.approx(2 * 10 / 0.150)


def test_single_rank_rate_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.whole_job_rate(10, 500.0, 1) == pytest.approx(20.0)
