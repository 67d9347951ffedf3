"""The replica path with world size 2 over gloo on the CPU: the timing reduction
takes the slowest rank and the units of all ranks, and replica seeds differ."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from quantit_gb300 import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = replicas.env()
        assert (r, w, lr) == (rank, world, rank)
        per_unit, t, n = replicas.whole_job_time_per_unit(seconds=1.0 + rank, units=3 + rank)
        mx = replicas.max_over_ranks([rank, 10 - rank])
        out[rank] = (per_unit, t, n, mx, replicas.replica_seed(7, rank))
    finally:
        dist.destroy_process_group()


def test_two_rank_timing_reduction_over_gloo():
    world, port = 2, _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for rank in range(world):
        per_unit, t, n, mx, seed = out[rank]
        assert t == 2.0 and n == 7.0          # slowest rank's time, all ranks' units
        assert per_unit == pytest.approx(2.0 / 7.0)
        assert mx == [1.0, 10.0]
    assert out[0][4] != out[1][4]


def test_single_process_is_identity():
    assert replicas.whole_job_time_per_unit(2.0, 4) == (0.5, 2.0, 4.0)
    assert replicas.max_over_ranks([3.0]) == [3.0]
