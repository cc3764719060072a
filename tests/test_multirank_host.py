"""Host logic of the multi-GPU bench path on CPU: two ``gloo`` ranks on 127.0.0.1.

The GB300 path does not shard (each rank runs an independent replica, no data exchange), so
what needs covering is the timing protocol around the replicas: every rank reads its rank
and world size from the launcher's environment, the job's time is the slowest rank's
(all-reduce MAX), and the whole-job rate counts every rank's cells.  Under a multi-rank
launch the reference arm runs on rank 0 alone; the other ranks return without work.
"""

import argparse
import os
import socket

import torch
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, ws: int, port: int, times: list) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench._dist() == (ws, rank, rank)
        ms = bench._max_over_ranks(times[rank], torch.device("cpu"))
        assert ms == max(times), (rank, ms)
        assert bench._job_rate(1000, 10, ws, ms) == 1000 * 10 * ws / (max(times) / 1e3)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_job_time():
    mp.spawn(_worker, args=(2, _free_port(), [12.5, 17.25]), nprocs=2, join=True)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.run_reference(argparse.Namespace(warmup=3, steps=5, ref_budget=1.0)) is None
