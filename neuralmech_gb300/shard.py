"""Shot sharding across ranks (one process per GPU).

The FWI gradient is a sum over shots, so the shots of one survey split into
contiguous blocks, one per rank. Each rank computes the misfit and gradient of
its block on its own GPU, and one all-reduce (sum) of the gradient and of the
FP64 misfit per gradient evaluation combines them. That is the only
collective of the path; there is no data-path exchange during the time loop.

``compute`` defaults to the GPU ``misfit_gradient``; any callable with the
same signature and return values may stand in (the CPU tests pass the FP64
oracle so that the rank logic runs under the gloo backend without a GPU).
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def shard_range(nshot: int, rank: int, world: int) -> slice:
    """Contiguous block of shots of `rank` (sizes differ by at most one)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(nshot, world)
    lo = rank * base + min(rank, extra)
    return slice(lo, lo + base + (1 if rank < extra else 0))


def distributed_misfit_gradient(vel, wavelet, src, rec, observed, grid, *, group=None, compute=None):
    """(misfit, grad) of all shots, each rank working on its own block.

    wavelet, src, rec and observed carry the leading shot axis of the whole
    survey; every rank passes the same full arrays and slices its block."""
    if compute is None:
        from .wavefd import misfit_gradient as compute
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    sl = shard_range(observed.shape[0], rank, world)
    if sl.stop > sl.start:
        J, g = compute(vel, wavelet[sl], src[sl], rec[sl], observed[sl], grid)
    else:  # more ranks than shots
        J = torch.zeros((), dtype=torch.float64, device=vel.device)
        g = torch.zeros_like(vel)
    J = torch.as_tensor(J, dtype=torch.float64, device=g.device).reshape(())
    dist.all_reduce(g, group=group)
    dist.all_reduce(J, group=group)
    return J, g
