"""Replicas over several GPUs: photons are independent, so N processes (one
per GPU) run disjoint photon-id ranges of the same job and exchange once at
the end, an FP64 sum of their tallies.  No collective runs on the data path.
(The reference runs one process on one device, main.m:144-187; the split is
this engine's.)"""
from __future__ import annotations

import numpy as np


def photon_range(rank: int, world: int, total: int, first: int = 0) -> tuple[int, int]:
    """(first, n) of rank's share of photons [first, first + total): contiguous
    blocks, the first total % world ranks one photon longer."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("bad rank / world / total")
    base, extra = divmod(total, world)
    start = first + rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def reduce_tallies(tallies: dict, group=None) -> dict:
    """Sums every array of `tallies` over the process group in FP64 (one
    all-reduce per array); returns the sums as numpy arrays.  Without an
    initialised torch.distributed group the input is returned as FP64."""
    import torch
    import torch.distributed as dist

    out = {}
    for k, v in tallies.items():
        t = torch.as_tensor(np.asarray(v, dtype=np.float64))
        if dist.is_available() and dist.is_initialized():
            if dist.get_backend(group) == "nccl":
                t = t.cuda()
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out[k] = t.cpu().numpy()
    return out
