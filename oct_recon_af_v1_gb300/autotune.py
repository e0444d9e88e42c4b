"""Launch-shape autotuners: the batched form's work queue (octgb_batch_process)
and the frame API's stitch tile shape (octgb_set_stitch_rows).

The persistent spectral kernel takes `grab` groups of 4 A-scans per atomic
operation on the work queue: small grabs balance load across SMs at the end
of the batch, large grabs cut queue traffic and keep each CTA on one tile
(fewer tile switches and depth-table reloads).  The order of the tile table
decides which tiles meet at the end of the queue.  `tune_batch` times every
candidate (grab, order) on the actual batch with CUDA events on the launching
stream, keeps the fastest, and caches it per batch signature (tile count and
total A-scans, bucketed) for the life of the process.
"""
from __future__ import annotations

import math

_CACHE: dict = {}
GRABS = (1, 2, 4, 8, 16, 32)
ORDERS = ("given", "largest_first")


def signature(tiles) -> tuple:
    total = sum(int(r.shape[0]) * (int(r.shape[1]) - int(apod)) for r, apod, _, _ in tiles)
    return len(tiles), int(round(math.log2(max(total, 1)) * 4))


def ordered(tiles, order: str):
    if order == "largest_first":
        return sorted(tiles, key=lambda t: -int(t[0].shape[0]) * (int(t[0].shape[1]) - int(t[1])))
    return list(tiles)


def cuda_timer(stream):
    """time(fn, reps) -> ms per call of fn, CUDA events on `stream` after a synchronize."""
    def time(fn, reps):
        import torch
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    return time


def tune_batch(ctx, tiles, threshold: float, stream, reps: int = 2, grabs=GRABS, orders=ORDERS, timer=None):
    """Return (grab, order, table of timings in ms) for this batch.  `timer`
    (default: CUDA events on `stream`) is time(fn, reps) -> ms per call."""
    time = timer or cuda_timer(stream)
    sig = signature(tiles)
    if sig in _CACHE:
        return _CACHE[sig]
    timings = {}
    for order in orders:
        work = ordered(tiles, order)
        for grab in grabs:
            ctx.batch_process(work, threshold, grab=grab)          # warm (tile table upload, caches)
            timings[(grab, order)] = time(lambda: ctx.batch_process(work, threshold, grab=grab), reps)
    best = min(timings, key=timings.get)
    _CACHE[sig] = (best[0], best[1], {f"{g}/{o}": round(t, 3) for (g, o), t in timings.items()})
    return _CACHE[sig]


STITCH_ROWS = (32, 64, 128)


def tune_stitch_rows(ctx, step, stream, key, reps: int = 3, rows=STITCH_ROWS, timer=None):
    """Output rows per stitch block of octgb_frames_process (its tile shape:
    32, 64 or 128 rows x 32 columns).  `step` runs one whole workload through
    the frame API (not under graph capture); each candidate is run once to
    build its slot tables, then timed over `reps` runs with CUDA events on the
    launching stream.  Every voxel sums its tiles in the same order for every
    shape, so the choice changes the time only.  Leaves the fastest set on the
    context and returns (rows, {rows: ms}); cached per `key`.  `timer`
    (default: CUDA events on `stream`) is time(fn, reps) -> ms per call."""
    time = timer or cuda_timer(stream)
    if key in _CACHE:
        best, table = _CACHE[key]
        ctx.set_stitch_rows(best)
        return best, table
    table = {}
    for r in rows:
        try:
            ctx.set_stitch_rows(r)
            step()
        except Exception:                                   # a shape whose patches exceed shared memory
            continue
        table[r] = round(time(step, reps), 3)
    if not table:
        raise RuntimeError("no stitch tile shape runs on this workload")
    best = min(table, key=table.get)
    ctx.set_stitch_rows(best)
    _CACHE[key] = (best, table)
    return best, table
