"""The multi-GPU contract of bench.py on CPU ranks (gloo, world size 2):
each rank renders its own replica (independent seeds), the job time is the
slowest rank's, and the job throughput counts every rank's samples.  The
path itself needs no collective (pixels and samples are independent)."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys

    import torch.distributed as dist

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    t_max = bench.max_over_ranks(ms, dist, "cpu")
    out[rank] = (t_max, bench.job_msamples(600 * 600 * 1024, world, t_max), bench.replica_seed(100, rank))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    assert res[0][1] == pytest.approx(600 * 600 * 1024 * 2 / 0.150 / 1e6)
    assert res[0][2] != res[1][2]


def test_single_rank_is_identity():
    import bench

    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.job_msamples(1_000_000, 1, 1000.0) == pytest.approx(1.0)
