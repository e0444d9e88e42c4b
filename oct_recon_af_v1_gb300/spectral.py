"""SpectralProcessor on the GB300 kernels.

Same interface and results as octrecon/core/spectral.py:84-165
(`SpectralProcessor.magnitude(raw) -> (B, nX, N/2) float32`), plus the
stage-level operators the reference exposes: `fused_pre_fft` (the GPU operator
of octrecon/core/gpu_kernels.py:54-68) and `db` (magnitude + depth crop +
20*log10 with the plane clim, as the reference applies them downstream).

Arrays may be numpy (host; copied through the library's device buffers) or
torch CUDA tensors (used in place; results are written into CUDA tensors).
AScanBinning and the Wasatch frame-mean apodisation (`prepare_raw`,
spectral.py:20-71) run on the device first (octgb_prepare_raw) when the
processor is built with them.
"""
from __future__ import annotations

import numpy as np

from ._lib import Context
from .geometry import SpectralGeometry


class SpectralProcessor:
    def __init__(self, sg: SpectralGeometry, apod_size: int, ctx: Context | None = None, device: int = 0,
                 ascan_binning: int = 1, apod_mode: str = "lines", apod_group: int = 1):
        """apod_mode "lines" (the first apod_size lines are the apodisation) or
        "frame_mean" (no apodisation lines: the mean over a file's lines, then
        over its frame's apod_group files, spectral.py:59-63)."""
        if apod_mode not in ("lines", "frame_mean"):
            raise ValueError(f"apod_mode {apod_mode!r}: 'lines' or 'frame_mean'")
        self.ctx = ctx or Context(device)
        self.sg = sg
        self.apod_size = int(apod_size)
        self.binning = max(1, int(ascan_binning))
        self.apod_mode = 1 if apod_mode == "frame_mean" else 0
        self.apod_group = max(1, int(apod_group))
        self.n = sg.n
        self.nz = self.n // 2
        self.ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)

    def _out(self, raw, shape, dtype):
        if isinstance(raw, np.ndarray):
            return np.empty(shape, dtype)
        import torch
        tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.complex64): torch.complex64}[np.dtype(dtype)]
        return torch.empty(shape, dtype=tdt, device=raw.device)

    def prepare(self, raw):
        """(prepared raw, its apodisation line count): `raw` itself for the
        "lines" mode without binning, else prepare_raw on the device (float32,
        on the device for device input)."""
        if self.binning == 1 and self.apod_mode == 0:
            return raw, self.apod_size
        a = self.apod_size if self.apod_mode == 0 else 1
        args = (self.apod_size, self.binning, self.apod_mode, self.apod_group)
        if isinstance(raw, np.ndarray):
            return self.ctx.prepare_raw(raw, *args), a
        lines = self.ctx.prepared_lines(raw, *args)
        out = self._out(raw, (raw.shape[0], lines, self.n), np.float32)
        return self.ctx.prepare_raw(raw, *args, out=out), a

    def magnitude(self, raw):
        x, a = self.prepare(raw)
        B, interf, _ = x.shape
        out = self._out(x, (B, interf - a, self.nz), np.float32)
        return self.ctx.magnitude(x, a, out)

    def fused_pre_fft(self, raw):
        x, a = self.prepare(raw)
        B, interf, _ = x.shape
        out = self._out(x, (B, interf - a, self.n), np.complex64)
        return self.ctx.fused_pre_fft(x, a, out)

    def db(self, raw, z0: int = 0, nz: int | None = None):
        """20*log10|scan| for depth bins [z0, z0+nz) and the finite [min, max]."""
        nz = self.nz - z0 if nz is None else int(nz)
        x, a = self.prepare(raw)
        B, interf, _ = x.shape
        out = self._out(x, (B, interf - a, nz), np.float32)
        return self.ctx.db(x, a, z0, nz, out)
