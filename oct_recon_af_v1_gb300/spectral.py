"""SpectralProcessor on the GB300 kernels.

Same interface and results as octrecon/core/spectral.py:84-165
(`SpectralProcessor.magnitude(raw) -> (B, nX, N/2) float32`), plus the
stage-level operators the reference exposes: `fused_pre_fft` (the GPU operator
of octrecon/core/gpu_kernels.py:54-68) and `db` (magnitude + depth crop +
20*log10 with the plane clim, as the reference applies them downstream).

Arrays may be numpy (host; copied through the library's device buffers) or
torch CUDA tensors (used in place; results are written into CUDA tensors).
Only the "lines" apodisation mode without A-scan binning is handled by the
kernels (the identity branch of `prepare_raw`, spectral.py:49-71).
"""
from __future__ import annotations

import numpy as np

from ._lib import Context
from .geometry import SpectralGeometry


class SpectralProcessor:
    def __init__(self, sg: SpectralGeometry, apod_size: int, ctx: Context | None = None, device: int = 0,
                 ascan_binning: int = 1, apod_mode: str = "lines"):
        if apod_mode != "lines" or int(ascan_binning) != 1:
            raise NotImplementedError("GB300 kernels handle apod_mode='lines' without A-scan binning")
        self.ctx = ctx or Context(device)
        self.sg = sg
        self.apod_size = int(apod_size)
        self.n = sg.n
        self.nz = self.n // 2
        self.ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)

    def _out(self, raw, shape, dtype):
        if isinstance(raw, np.ndarray):
            return np.empty(shape, dtype)
        import torch
        tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.complex64): torch.complex64}[np.dtype(dtype)]
        return torch.empty(shape, dtype=tdt, device=raw.device)

    def magnitude(self, raw):
        B, interf, _ = raw.shape
        out = self._out(raw, (B, interf - self.apod_size, self.nz), np.float32)
        return self.ctx.magnitude(raw, self.apod_size, out)

    def fused_pre_fft(self, raw):
        B, interf, _ = raw.shape
        out = self._out(raw, (B, interf - self.apod_size, self.n), np.complex64)
        return self.ctx.fused_pre_fft(raw, self.apod_size, out)

    def db(self, raw, z0: int = 0, nz: int | None = None):
        """20*log10|scan| for depth bins [z0, z0+nz) and the finite [min, max]."""
        nz = self.nz - z0 if nz is None else int(nz)
        B, interf, _ = raw.shape
        out = self._out(raw, (B, interf - self.apod_size, nz), np.float32)
        return self.ctx.db(raw, self.apod_size, z0, nz, out)
