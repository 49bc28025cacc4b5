"""The multi-GPU path on CPU ranks (gloo, world size 2): one frame split by
sample ranges (tpt/frame_split.py), the accumulators summed across ranks,
the job time the slowest rank's, the job throughput one frame's samples over
that time.  The ranks' "renders" are host tensors here: per (pixel, sample)
a value that depends only on the pair, as the GPU's per-sample streams do,
so the summed shares must equal the one-rank sum exactly."""
import os
import socket

import numpy as np
import pytest

W, H, SPP = 7, 5, 13  # an spp that does not divide evenly between the ranks


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _samples(b: int, e: int) -> np.ndarray:
    """Per-pixel sums (float4 layout) of samples [b, e): sample k of pixel p
    contributes sin(p + 0.1 k) and friends."""
    p = np.arange(W * H, dtype=np.float64)[:, None]
    k = np.arange(b, e, dtype=np.float64)[None, :]
    out = np.zeros((W * H, 4))
    out[:, 0] = np.sin(p + 0.1 * k).sum(1)
    out[:, 1] = np.cos(0.3 * p + k).sum(1)
    out[:, 2] = (k * 0 + p).sum(1)
    return out


def _rank_main(rank, world, port, out):
    import sys

    import torch
    import torch.distributed as dist

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, ".."))
    sys.path.insert(0, os.path.join(here, "..", "tiny-path-tracer_gb300"))
    import bench
    from tpt import frame_split

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b, e = frame_split.sample_range(rank, world, SPP)
    accum = torch.from_numpy(_samples(b, e))
    frame_split.reduce_shares(accum, dist)
    ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    t_max = bench.max_over_ranks(ms, dist, "cpu")
    out[rank] = ((b, e), accum.numpy().tolist(), t_max, bench.frame_msamples(W * H * SPP, t_max))
    dist.destroy_process_group()


def test_two_gloo_ranks_split_one_frame():
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    (b0, e0), (b1, e1) = res[0][0], res[1][0]
    assert (b0, e1) == (0, SPP) and e0 == b1 and abs((e0 - b0) - (e1 - b1)) <= 1
    full = _samples(0, SPP)
    for r in (0, 1):
        np.testing.assert_allclose(np.array(res[r][1]), full, rtol=1e-12, atol=1e-9)
    assert res[0][2] == res[1][2] == 150.0
    assert res[0][3] == pytest.approx(W * H * SPP / 0.150 / 1e6)


def test_sample_ranges_partition():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "tiny-path-tracer_gb300"))
    from tpt import frame_split

    for world in (1, 2, 3, 8):
        for spp in (0, 1, 7, 1024):
            r = [frame_split.sample_range(k, world, spp) for k in range(world)]
            assert r[0][0] == 0 and r[-1][1] == spp
            assert all(r[k][1] == r[k + 1][0] for k in range(world - 1))
            sizes = [e - b for b, e in r]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        frame_split.sample_range(2, 2, 16)
    # one rank: the reduction is the identity
    acc = np.ones(4)
    frame_split.reduce_shares(acc, None)
    assert (acc == 1).all()


def test_single_rank_is_identity():
    import bench

    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.frame_msamples(1_000_000, 1000.0) == pytest.approx(1.0)
