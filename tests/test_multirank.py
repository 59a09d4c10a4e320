"""The multi-GPU bench path (replicas, no data-path collective) on CPU ranks over gloo."""

from __future__ import annotations

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


def _worker(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import bench

    d, r, ws, local = bench._dist()
    try:
        assert (r, ws, local) == (rank, world, rank)
        bench._barrier(d)
        # each replica reports its own device time; the job is timed by the slowest
        t = bench._max_over_ranks(d, 10.0 + 5.0 * rank)
        out[rank] = (t, bench.replica_value(1000, 20, ws, t))
    finally:
        d.destroy_process_group()


def test_two_rank_replicas_take_the_slowest_rank_and_sum_the_work():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    assert res[0][1] == pytest.approx(2 * 1000 * 20 / 15e-3)


def test_single_process_needs_no_process_group():
    import bench

    d, r, ws, local = bench._dist()
    assert d is None and (r, ws, local) == (0, 1, 0)
    assert bench._max_over_ranks(None, 3.0) == 3.0
