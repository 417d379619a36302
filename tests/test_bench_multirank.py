"""The multi-GPU bench path on CPU: world_size-2 gloo ranks.

bench.py under torchrun runs one process per GPU; windows are independent, so
each rank clusters its own shard (the config drawn with its shard seed) and the
only collectives are the max-over-ranks timings.  These tests run that host
logic with the gloo backend on two CPU processes (no GPU): rank/world parsing,
distinct per-rank shards, the max reduction and the whole-job rate.
"""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, results):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    r, w, local = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    try:
        packed, offsets, params = bench.rank_workload("c2", r, windows=3)
        step_ms = 10.0 + 5.0 * r  # rank 1 is the slow one
        ms = bench.reduce_max(step_ms, w, torch.device("cpu"))
        rate = bench.whole_job_rate(len(offsets) - 1, w, ms)
        results[r] = (r, w, local, float(packed[0, 0]), ms, rate)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_max_and_whole_job_rate():
    world = 2
    manager = mp.get_context("spawn").Manager()
    results = manager.dict()
    mp.start_processes(_worker, args=(world, _free_port(), results), nprocs=world, start_method="spawn", join=True)
    got = dict(results)
    assert sorted(got) == [0, 1]
    for r in (0, 1):
        rank, w, local, first, ms, rate = got[r]
        assert (rank, w, local) == (r, world, r)
        assert ms == 15.0                       # every rank sees the slowest rank's time
        assert rate == pytest.approx(3 * world / 0.015)
    assert got[0][3] != got[1][3]               # each rank clusters its own shard


def test_single_process_defaults():
    import bench

    assert bench.reduce_max(4.5, 1, None) == 4.5
    assert bench.whole_job_rate(256, 1, 2.0) == pytest.approx(128000.0)
    packed, offsets, params = bench.rank_workload("c1", 0)
    from hdbscan_gb300 import synthetic

    ref, ref_offsets, _ = synthetic.make("c1")
    np.testing.assert_array_equal(packed, ref)   # rank 0 is the config itself
