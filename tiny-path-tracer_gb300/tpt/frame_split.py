"""One frame split across GPUs, one process per GPU.

The reference parallelises one frame over image rows on the host cores
(main.cpp:157-159).  Here every rank renders the whole image but only its
share of the samples: rank r of N takes samples [r*spp/N, (r+1)*spp/N) of
every pixel (tpt_render_range).  Each sample draws from its own (pixel,
sample index) stream, so the shares add up to the one-GPU frame; the one
exchange step is a sum-reduce of the float4 accumulators (width*height*16
bytes), after which tpt_resolve_sums gives the mean image.  The scene is
replicated: every rank compiles and uploads it.
"""
from __future__ import annotations


def sample_range(rank: int, world: int, spp: int) -> tuple[int, int]:
    """The samples rank `rank` of `world` renders: a balanced, contiguous,
    disjoint partition of [0, spp) (shares differ by at most one sample)."""
    if world < 1 or not 0 <= rank < world or spp < 0:
        raise ValueError(f"bad partition: rank {rank} of {world}, spp {spp}")
    return rank * spp // world, (rank + 1) * spp // world


def reduce_shares(accum, dist=None) -> None:
    """Sums every rank's accumulators in place (all-reduce); a no-op on one
    rank.  accum: a torch tensor (CUDA under NCCL, host under gloo)."""
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(accum, op=dist.ReduceOp.SUM)


def render_split_frame(ctx, slot: int, width: int, height: int, spp: int, accum, rank: int = 0, world: int = 1,
                       dist=None, out=None, **kw):
    """This rank's share of the frame, the sum over ranks and the mean image
    (host array, or written to the device pointer `out`).  accum: a CUDA
    float32 tensor of width*height*4 elements.  Returns (image or None,
    this rank's render stats)."""
    b, e = sample_range(rank, world, spp)
    st = ctx.render_range(slot, width, height, b, e, accum.data_ptr(), **kw)
    reduce_shares(accum, dist)
    return ctx.resolve_sums(accum.data_ptr(), width, height, spp, out=out), st
