"""Sharding a volume reconstruction over ranks (one process per GPU).

Output planes of different y-tile rows are independent (octrecon/pipeline.py
process_row per row, :365-375), so rows are split into contiguous blocks, one
per rank, with no data-path collective.  The one exchange is the global clim
of the legacy quantisation (pipeline.py:388): a min / max all-reduce of two
numbers, after which every rank quantises its own planes.
"""
from __future__ import annotations

import math


def shard_rows(n_rows: int, rank: int, world: int) -> range:
    """Contiguous block of y-tile rows owned by `rank` (sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    base, extra = divmod(n_rows, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def global_clim(local_min: float, local_max: float, group=None):
    """[min, max] over all ranks of the finite dB values; a rank with no finite
    value passes NaN.  Returns (nan, nan) when no rank has any."""
    import torch
    import torch.distributed as dist
    lo = math.inf if math.isnan(local_min) else float(local_min)
    hi = -math.inf if math.isnan(local_max) else float(local_max)
    backend = dist.get_backend(group)
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.tensor([lo, -hi], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
    lo, hi = float(t[0]), -float(t[1])
    if lo > hi:
        return math.nan, math.nan
    return lo, hi
