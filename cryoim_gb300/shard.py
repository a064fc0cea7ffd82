"""Particle sharding across ranks and the reduction of partial reconstructions.

icosprocess scales by hand: each run takes a `first`..`last` particle range
(icosprocess/SRC/0main.f90:125-130), search and refinement are independent per
particle, and a reconstruction run writes a tnf partial that merge_icosprocess_subrec
sums (merge_reconstruct.f90:20-34).  Here one rank owns one GPU and a contiguous range;
the only exchange on the path is the sum of the (fa, fb, wg) partial accumulators, one
all_reduce (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

import numpy as np


def particle_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """1-based inclusive (first, last) of this rank's contiguous share of n particles;
    first > last when the rank gets none."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    first = rank * base + min(rank, extra) + 1
    count = base + (1 if rank < extra else 0)
    return first, first + count - 1


def allreduce_partials(fa: np.ndarray, fb: np.ndarray, wg: np.ndarray, wg_init: float = 0.0,
                       group=None) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Sum partial accumulators over all ranks.  Each rank's wg started at wg_init (0.01
    in reconstruct.f90:28, 0 in reconstruct_substep.f90:25); the sum keeps it once."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" \
        else torch.device("cpu")
    t = torch.from_numpy(np.stack([fa, fb, wg - wg_init]).astype(np.float64)).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out = t.cpu().numpy()
    del world
    return (out[0].astype(fa.dtype), out[1].astype(fb.dtype), (out[2] + wg_init).astype(wg.dtype))
