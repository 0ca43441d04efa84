"""Shot sharding across processes (one GPU per process).

Shots are independent, so N ranks split a survey's shots with no exchange
during the solves; a gradient needs one sum of the three kernels (3 * nx*nz
floats) and of the misfit across ranks afterwards. This module holds that
host-side logic: which shots a rank owns, and the sum over ranks through a
torch.distributed process group (gloo on CPU tensors or NCCL).
"""
from __future__ import annotations

import numpy as np


def shard_shots(nsrc: int, rank: int, world: int) -> list:
    """Round-robin assignment: rank r owns shots r, r + world, ..."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    return list(range(rank, nsrc, world))


def reduce_gradient(kernels: dict, misfit: float, group=None):
    """Sums per-rank kernels (name -> float array) and misfit over the group.
    Sums run in float64 so the result does not depend on the rank count at
    float32 precision."""
    import torch
    import torch.distributed as dist

    names = sorted(kernels)
    flat = np.concatenate([np.asarray(kernels[n], np.float64).ravel() for n in names] + [np.array([misfit])])
    t = torch.from_numpy(flat)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out, off = {}, 0
    for n in names:
        size = np.asarray(kernels[n]).size
        out[n] = t[off:off + size].numpy().astype(np.float64)
        off += size
    return out, float(t[-1].item())
