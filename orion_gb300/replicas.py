"""Replicas: one process per GPU, each rendering a disjoint range of sample passes.

Every (pixel, pass) path of PathTracing::render has its own Sobol index
k*W*H + j*W + i (src/integrator/path.cpp:22-36), so N processes that render
passes [first + r*spp, first + (r+1)*spp) for r = 0..N-1 together render the
image of N*spp passes, and their film sums and counts simply add. Nothing is
exchanged while rendering; the one collective is the final film reduction, for
a caller that wants a single image.
"""
from __future__ import annotations

import numpy as np


def pass_range(rank: int, world: int, spp_per_rank: int, first_pass: int = 0) -> tuple[int, int]:
    """(first pass, number of passes) that `rank` of `world` renders."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    if spp_per_rank < 1:
        raise ValueError("spp_per_rank must be positive")
    return first_pass + rank * spp_per_rank, spp_per_rank


def reduce_film(film_sum: np.ndarray, film_count: np.ndarray | None = None, dst: int = 0, group=None):
    """Sums the ranks' film sums (and counts) into rank `dst` with torch.distributed.

    Works with any initialised backend (gloo on CPU tensors, NCCL after a copy
    to the device). Returns the reduced arrays on `dst` and the local ones
    elsewhere. FP32 sums are reduced in FP64 and rounded once.
    """
    import torch
    import torch.distributed as dist

    backend = dist.get_backend(group)
    device = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.from_numpy(np.ascontiguousarray(film_sum, dtype=np.float64)).to(device)
    dist.reduce(t, dst=dst, op=dist.ReduceOp.SUM, group=group)
    out_sum = t.cpu().numpy().astype(film_sum.dtype)
    out_count = None
    if film_count is not None:
        c = torch.from_numpy(np.ascontiguousarray(film_count, dtype=np.int64)).to(device)
        dist.reduce(c, dst=dst, op=dist.ReduceOp.SUM, group=group)
        out_count = c.cpu().numpy().astype(film_count.dtype)
    if dist.get_rank(group) != dst:
        return film_sum, film_count
    return out_sum, out_count
