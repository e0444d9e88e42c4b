"""Row reconstruction on the GB300 kernels: the body of
octrecon/pipeline.py:223-302 (`Reconstructor.process_row`).

For each tile of the y-tile row (x-major, z-minor) and each batch of frames:
spectral stage -> stitch contribution -> num/den accumulation, all on the
device; then the row is finalised (weight threshold -> NaN, 20*log10(num/den))
into float32 dB planes, with each plane's clim.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Sequence

import numpy as np

from ._lib import Context
from .stitching import TileStitcher, min_weight_threshold


@dataclass
class RowTile:
    """One tile of the row: its stitcher and a reader of raw frames.

    read(frames) -> raw array (len(frames), interf, N) (numpy or CUDA tensor)."""
    stitcher: TileStitcher
    read: Callable[[np.ndarray], object]


class RowReconstructor:
    def __init__(self, ctx: Context, apod_size: int, n_out_z: int, n_out_x: int, batch_frames: int = 50,
                 threshold: float | None = None):
        self.ctx = ctx
        self.apod_size = int(apod_size)
        self.n_out_z = int(n_out_z)
        self.n_out_x = int(n_out_x)
        self.batch = int(batch_frames)
        self.threshold = min_weight_threshold(np.float32) if threshold is None else float(threshold)

    def process_row(self, tiles: Sequence[RowTile], frames, out=None, plane_clims: bool = False,
                    cancel=None, on_batch=None):
        frames = np.asarray(frames)
        nF = len(frames)
        self.ctx.row_begin(nF, self.n_out_z, self.n_out_x)
        jobs = [(t, s, frames[s:s + self.batch]) for t in tiles if not t.stitcher.empty
                for s in range(0, nF, self.batch)]
        for n, (t, s, fr) in enumerate(jobs):
            if cancel is not None and cancel.is_set():
                from ._lib import Cancelled
                raise Cancelled(4, "cancelled")
            raw = t.read(fr)
            self.ctx.row_add_batch(t.stitcher.plan, raw, self.apod_size, fr, s)
            if on_batch:
                on_batch(n + 1, len(jobs))
        return self.ctx.row_finalise(self.threshold, (nF, self.n_out_z, self.n_out_x), out, plane_clims)
