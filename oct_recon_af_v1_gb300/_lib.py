"""ctypes binding of liboctgb.so (the C ABI declared in include/octgb.h).

The library is loaded from the package's in-tree `_lib/` folder.  There is no
fallback: if the shared library is missing or fails to load, `load()` raises.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_float, c_int, c_int64, c_uint16, c_void_p
from pathlib import Path

import numpy as np

from ._build import LIB

OK, ERR_ARG, ERR_CUDA, ERR_STATE, ERR_CANCELLED, ERR_TIMEOUT, ERR_NOMEM = range(7)
U16, I16, F32 = 0, 1, 2
HOST, DEVICE = 0, 1

_DTYPE = {np.dtype(np.uint16): U16, np.dtype(np.int16): I16, np.dtype(np.float32): F32}

# name -> (restype, argtypes); every symbol include/octgb.h declares
SIGNATURES = {
    "octgb_create": (c_int, [c_int, POINTER(c_void_p)]),
    "octgb_destroy": (c_int, [c_void_p]),
    "octgb_last_error": (ctypes.c_char_p, [c_void_p]),
    "octgb_set_stream": (c_int, [c_void_p, c_void_p]),
    "octgb_synchronize": (c_int, [c_void_p]),
    "octgb_cancel": (c_int, [c_void_p]),
    "octgb_reset_cancel": (c_int, [c_void_p]),
    "octgb_launch_count": (c_int64, [c_void_p]),
    "octgb_set_geometry": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "octgb_fused_pre_fft": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_int]),
    "octgb_magnitude": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_int]),
    "octgb_db": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_int,
                         c_void_p]),
    "octgb_quantise": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_double, c_double, c_void_p, c_int]),
    "octgb_minmax": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p]),
    "octgb_stitch_plan": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p,
                                  c_void_p, c_void_p, c_void_p, c_int, POINTER(c_int)]),
    "octgb_row_begin": (c_int, [c_void_p, c_int, c_int, c_int]),
    "octgb_row_add_batch": (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_int]),
    "octgb_row_finalise": (c_int, [c_void_p, c_float, c_void_p, c_int, c_void_p]),
    "octgb_frames_process": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int,
                                     c_int, c_int, c_float, c_void_p, c_int, c_void_p]),
    "octgb_clim_reset": (c_int, [c_void_p]),
    "octgb_clim_get": (c_int, [c_void_p, c_void_p]),
    "octgb_quantise_running": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_int]),
    "octgb_graph_begin": (c_int, [c_void_p]),
    "octgb_graph_end": (c_int, [c_void_p, POINTER(c_int)]),
    "octgb_graph_launch": (c_int, [c_void_p, c_int]),
    "octgb_graphs_release": (c_int, [c_void_p]),
    "octgb_set_stitch_rows": (c_int, [c_void_p, c_int]),
    "octgb_selftest_wait_expiry": (c_int, [c_void_p, c_int, c_int]),
    "octgb_magnitude_noalloc": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p]),
    "octgb_batch_process": (c_int, [c_void_p, c_int, c_void_p, c_int, c_float, c_int]),
    "octgb_disp_load": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_void_p]),
    "octgb_disp_lines": (c_int, [c_void_p, c_void_p, c_int]),
    "octgb_disp_set_dk2": (c_int, [c_void_p, c_void_p]),
    "octgb_disp_eval": (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_int64, c_int, c_void_p,
                                c_void_p, c_int]),
    "octgb_xmedian": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p]),
    "octgb_xmean": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p]),
    "octgb_quantise_double": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_double, c_double, c_double, c_double,
                                      c_void_p, c_int]),
    "octgb_packbits": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_int64, c_void_p, c_void_p]),
    "octgb_prepare_raw": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_int,
                                  c_void_p, c_int, c_void_p]),
    "octgb_srr_decode": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_int,
                                 c_void_p, c_int]),
    "octgb_average_repeats": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_void_p,
                                      c_int]),
    "octgb_row_add_batch_ex": (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_int,
                                       c_int, c_int, c_void_p, c_int, c_int]),
    "octgb_linearise_precision": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_int]),
    "octgb_magnitude_precision": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_int]),
    "octgb_magnitude_exact": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_int]),
    "octgb_disp_images": (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_void_p, c_int]),
    "octgb_cnn_images": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_int]),
    "octgb_cnn_conv3x3": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                  c_int]),
    "octgb_cnn_conv3x3_tc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                  c_int]),
    "octgb_cnn_conv3x3_relu_pool_tc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                  c_int]),
    "octgb_cnn_conv3x3_bwd": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_int, c_int, c_int, c_int, c_int]),
    "octgb_cnn_conv3x3_bwd_tc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_int, c_int, c_int, c_int, c_int]),
    "octgb_cnn_relu_pool":(c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_int]),
    "octgb_cnn_relu_pool_bwd": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_int, c_int]),
    "octgb_cnn_dense": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int]),
    "octgb_cnn_dense_bwd": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_int, c_int, c_int]),
    "octgb_cnn_mse": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "octgb_cnn_adam": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_float, c_float, c_float,
                               c_float, c_int]),
}


class OctgbTile(ctypes.Structure):
    """struct octgb_tile (include/octgb.h)."""
    _fields_ = [("raw", c_void_p), ("B", c_int), ("interf", c_int), ("apod_size", c_int), ("plan_id", c_int),
                ("db", c_void_p)]

_lib = None


class OctgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"octgb error {code}: {msg}")
        self.code = code


class Cancelled(OctgbError):
    pass


def load(path: Path | None = None):
    """Load (once) and return the ctypes library handle; raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with oct_recon_af_v1_gb300.build() "
                           "(the GB300 path has no CPU fallback)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols(path: Path | None = None):
    """Names of SIGNATURES present in the library (symbol lookup only, no calls)."""
    lib = ctypes.CDLL(str(Path(path) if path else LIB))
    return [n for n in SIGNATURES if hasattr(lib, n)]


def _ptr(a):
    """(pointer, location) of a numpy array or a CUDA tensor-like object."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data, HOST
    if hasattr(a, "data_ptr") and getattr(a, "is_cuda", False):
        return a.data_ptr(), DEVICE
    if hasattr(a, "data_ptr"):  # torch CPU tensor
        return a.data_ptr(), HOST
    raise TypeError(f"unsupported array type {type(a)!r}")


def _raw_dtype(a) -> int:
    if isinstance(a, np.ndarray):
        dt = a.dtype
    else:
        import torch
        dt = {torch.int16: np.dtype(np.int16), torch.float32: np.dtype(np.float32)}.get(a.dtype)
        if dt is None and str(a.dtype) == "torch.uint16":
            dt = np.dtype(np.uint16)
    if dt not in _DTYPE:
        raise TypeError(f"raw spectra must be uint16, int16 or float32, got {dt}")
    return _DTYPE[dt]


class Context:
    """One octgb context (device, stream, geometry, work buffers)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = c_void_p()
        rc = self.lib.octgb_create(int(device), ctypes.byref(h))
        if rc != OK:
            raise OctgbError(rc, self.lib.octgb_last_error(None).decode())
        self.h = h
        self.device = int(device)
        self.n = None
        self.taps = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.octgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != OK:
            msg = self.lib.octgb_last_error(self.h).decode()
            raise (Cancelled if rc == ERR_CANCELLED else OctgbError)(rc, msg)

    # -------------------------------------------------------------- control
    def set_stream(self, stream_handle: int | None):
        self._check(self.lib.octgb_set_stream(self.h, c_void_p(stream_handle or None)))

    def follow_torch_stream(self):
        """Launch on torch's current CUDA stream; torch's default stream (handle
        0) maps to the legacy default stream (cudaStreamLegacy), so the
        context's work is ordered with torch's and with every other context
        that follows the same stream."""
        import torch
        h = torch.cuda.current_stream().cuda_stream
        self.set_stream(h if h else 1)                       # 1 == cudaStreamLegacy

    def synchronize(self):
        self._check(self.lib.octgb_synchronize(self.h))

    def cancel(self):
        self._check(self.lib.octgb_cancel(self.h))

    def reset_cancel(self):
        self._check(self.lib.octgb_reset_cancel(self.h))

    @property
    def launches(self) -> int:
        return int(self.lib.octgb_launch_count(self.h))

    # -------------------------------------------------------------- spectral
    def set_geometry(self, sinc_idx: np.ndarray, sinc_w: np.ndarray, window: np.ndarray):
        idx = np.ascontiguousarray(sinc_idx, dtype=np.int64)
        w = np.ascontiguousarray(sinc_w, dtype=np.float64)
        win = np.ascontiguousarray(np.stack([np.real(window), np.imag(window)], -1), dtype=np.float64)
        n, taps = idx.shape
        self._check(self.lib.octgb_set_geometry(self.h, n, taps, idx.ctypes.data, w.ctypes.data, win.ctypes.data))
        self.n, self.taps = n, taps

    def _raw_args(self, raw, apod_size, raw_dtype=None):
        if raw.ndim != 3:
            raise ValueError("raw must be (B, interf, N)")
        if isinstance(raw, np.ndarray):
            raw = np.ascontiguousarray(raw)
        elif not raw.is_contiguous():
            raw = raw.contiguous()
        B, interf, N = raw.shape
        if N != self.n:
            raise ValueError(f"raw has {N} spectral samples, geometry has {self.n}")
        p, loc = _ptr(raw)
        return raw, p, loc, (_raw_dtype(raw) if raw_dtype is None else int(raw_dtype)), B, interf

    def fused_pre_fft(self, raw, apod_size: int, out=None, raw_dtype=None):
        raw, p, loc, dt, B, interf = self._raw_args(raw, apod_size, raw_dtype)
        if out is None:
            out = np.empty((B, interf - apod_size, self.n), np.complex64)
        op, oloc = _ptr(out)
        self._check(self.lib.octgb_fused_pre_fft(self.h, p, dt, loc, B, interf, apod_size, op, oloc))
        return out

    def magnitude(self, raw, apod_size: int, out=None, raw_dtype=None):
        raw, p, loc, dt, B, interf = self._raw_args(raw, apod_size, raw_dtype)
        if out is None:
            out = np.empty((B, interf - apod_size, self.n // 2), np.float32)
        op, oloc = _ptr(out)
        self._check(self.lib.octgb_magnitude(self.h, p, dt, loc, B, interf, apod_size, op, oloc))
        return out

    def prepared_lines(self, raw, apod_size: int, binning: int = 1, apod_mode: int = 0, apod_group: int = 1,
                       raw_dtype=None) -> int:
        """Lines per B-scan of prepare_raw's result (apodisation + kept scan
        lines); a shape query, no device work."""
        raw, p, loc, dt, B, n_lines = self._raw_args(raw, apod_size, raw_dtype)
        n_out = ctypes.c_int(0)
        self._check(self.lib.octgb_prepare_raw(self.h, p, dt, loc, 0, n_lines, apod_size, binning, apod_mode,
                                               apod_group, ctypes.c_void_p(16), HOST, ctypes.byref(n_out)))
        return n_out.value

    def prepare_raw(self, raw, apod_size: int, binning: int = 1, apod_mode: int = 0, apod_group: int = 1,
                    out=None, raw_dtype=None):
        """prepare_raw on the device: (B, lines, N) -> float32 (B, a + kept, N)
        (numpy result for numpy input unless `out` is given)."""
        raw, p, loc, dt, B, n_lines = self._raw_args(raw, apod_size, raw_dtype)
        n_out = ctypes.c_int(0)
        if out is None:
            out = np.empty((B, self.prepared_lines(raw, apod_size, binning, apod_mode, apod_group, raw_dtype),
                            self.n), np.float32)
        op, oloc = _ptr(out)
        self._check(self.lib.octgb_prepare_raw(self.h, p, dt, loc, B, n_lines, apod_size, binning, apod_mode,
                                               apod_group, op, oloc, ctypes.byref(n_out)))
        return out

    def srr_decode(self, words, apod_range, scan_range, out=None):
        """Thorlabs SRR words (n_files, file_lines, n) uint16 (host or device)
        -> (n_files, apod + scan lines, n) int16, decoded on the device
        (io/srr.py:108-125).  A numpy result for numpy input unless `out` (a
        device or host array of that shape) is given."""
        if isinstance(words, np.ndarray):
            words = np.ascontiguousarray(words, dtype=np.uint16)
        elif not words.is_contiguous():
            words = words.contiguous()
        if words.ndim != 3:
            raise ValueError("words must be (n_files, file_lines, n)")
        n_files, file_lines, n = (int(v) for v in words.shape)
        a0, a1 = (int(v) for v in apod_range)
        s0, s1 = (int(v) for v in scan_range)
        if out is None:
            out = np.empty((n_files, (a1 - a0) + (s1 - s0), n), np.int16)
        p, loc = _ptr(words)
        op, oloc = _ptr(out)
        self._check(self.lib.octgb_srr_decode(self.h, p, loc, n_files, file_lines, n, a0, a1, s0, s1, op, oloc))
        return out

    def average_repeats(self, mag, n_frames: int, bscan_avg: int, ascan_avg: int, out=None):
        F, L, nz = mag.shape
        size_x = L // ascan_avg
        if out is None:
            out = np.empty((n_frames, size_x, nz), np.float32)
        if isinstance(mag, np.ndarray):
            mag = np.ascontiguousarray(mag, dtype=np.float32)
        p, loc = _ptr(mag)
        op, oloc = _ptr(out)
        self._check(self.lib.octgb_average_repeats(self.h, p, loc, n_frames, bscan_avg, size_x, ascan_avg, nz, op,
                                                   oloc))
        return out

    def linearise_precision(self, raw, apod_size: int, out=None, raw_dtype=None):
        """Precision form, stage (c): the linearised interferogram (B, nX, N)
        float32 from the tensor-core sinc (no window)."""
        raw, p, loc, dt, B, interf = self._raw_args(raw, apod_size, raw_dtype)
        if out is None:
            out = np.empty((B, interf - apod_size, self.n), np.float32)
        op, oloc = _ptr(out)
        self._check(self.lib.octgb_linearise_precision(self.h, p, dt, loc, B, interf, apod_size, op, oloc))
        return out

    def magnitude_precision(self, raw, apod_size: int, out=None, raw_dtype=None):
        """Precision form of magnitude(): tensor-core sinc, then window, FFT, |.|."""
        raw, p, loc, dt, B, interf = self._raw_args(raw, apod_size, raw_dtype)
        if out is None:
            out = np.empty((B, interf - apod_size, self.n // 2), np.float32)
        op, oloc = _ptr(out)
        self._check(self.lib.octgb_magnitude_precision(self.h, p, dt, loc, B, interf, apod_size, op, oloc))
        return out

    def magnitude_exact(self, raw, apod_size: int, out=None, raw_dtype=None):
        """Float64 form of magnitude(): exact background, float64 sinc, window
        and FFT, |X| rounded to float32 (integer raws only)."""
        raw, p, loc, dt, B, interf = self._raw_args(raw, apod_size, raw_dtype)
        if out is None:
            out = np.empty((B, interf - apod_size, self.n // 2), np.float32)
        op, oloc = _ptr(out)
        self._check(self.lib.octgb_magnitude_exact(self.h, p, dt, loc, B, interf, apod_size, op, oloc))
        return out

    def db(self, raw, apod_size: int, z0: int, nz: int, out=None, minmax: bool = True, raw_dtype=None):
        raw, p, loc, dt, B, interf = self._raw_args(raw, apod_size, raw_dtype)
        if out is None:
            out = np.empty((B, interf - apod_size, nz), np.float32)
        op, oloc = _ptr(out)
        mm = np.full(2, np.nan)
        self._check(self.lib.octgb_db(self.h, p, dt, loc, B, interf, apod_size, int(z0), int(nz), op, oloc,
                                      mm.ctypes.data if minmax else None))
        return out, (float(mm[0]), float(mm[1]))

    # -------------------------------------------------------------- estimation
    def disp_load(self, raw, apod_size: int, n_bscans: int, rep: int, hann: np.ndarray, raw_dtype=None):
        """Linearise + Hann/rms-window n_bscans x rep B-scans once (the geometry must
        carry a window of ones)."""
        raw, p, loc, dt, B, interf = self._raw_args(raw, apod_size, raw_dtype)
        if B != n_bscans * rep:
            raise ValueError("raw must hold n_bscans x rep B-scans")
        h = np.ascontiguousarray(hann, dtype=np.float64)
        self._check(self.lib.octgb_disp_load(self.h, p, dt, loc, int(n_bscans), int(rep), interf, int(apod_size),
                                             h.ctypes.data))
        self._disp_lines_shape = (B, interf - int(apod_size), self.n)

    def disp_lines(self, out=None):
        """The loaded, linearised and windowed lines (n_bscans * rep, nX, N) float32."""
        if out is None:
            out = np.empty((self._disp_lines_shape), np.float32)
        p, loc = _ptr(out)
        self._check(self.lib.octgb_disp_lines(self.h, p, loc))
        return out

    def disp_set_dk2(self, dk2: np.ndarray):
        d = np.ascontiguousarray(dk2, dtype=np.float64)
        self._check(self.lib.octgb_disp_set_dk2(self.h, d.ctypes.data))

    def disp_eval(self, betas, b0: int, nb: int, metric: int, top_k: int = 0, z_min: int = 20, mag=None):
        """Scores (n_beta, nb) float64 (None with metric 0); mag (optional) receives the
        magnitudes (n_beta, nb, nX, N/2) float32 (numpy array or CUDA tensor)."""
        b = np.ascontiguousarray(np.atleast_1d(np.asarray(betas, dtype=np.float64)))
        scores = np.empty((len(b), nb), np.float64) if metric else None
        mp, mloc = (None, HOST) if mag is None else _ptr(mag)
        self._check(self.lib.octgb_disp_eval(self.h, len(b), b.ctypes.data, int(b0), int(nb), int(metric),
                                             int(top_k), int(z_min),
                                             None if scores is None else scores.ctypes.data, mp, mloc))
        return scores

    def xmedian(self, mag, ignore_nan: bool = False) -> np.ndarray:
        """numpy.median / nanmedian over x of (frames, nX, nZ) float32 -> (frames, nZ) float64."""
        if isinstance(mag, np.ndarray):
            mag = np.ascontiguousarray(mag, dtype=np.float32)
        elif not mag.is_contiguous():
            mag = mag.contiguous()
        F, nx, nz = mag.shape
        p, loc = _ptr(mag)
        out = np.empty((F, nz), np.float64)
        self._check(self.lib.octgb_xmedian(self.h, p, loc, F, nx, nz, int(bool(ignore_nan)), out.ctypes.data))
        return out

    def xmean(self, mag) -> np.ndarray:
        """float64 mean over x (NaN ignored) of (frames, nX, nZ) float32 -> (frames, nZ)."""
        if isinstance(mag, np.ndarray):
            mag = np.ascontiguousarray(mag, dtype=np.float32)
        elif not mag.is_contiguous():
            mag = mag.contiguous()
        F, nx, nz = mag.shape
        p, loc = _ptr(mag)
        out = np.empty((F, nz), np.float64)
        self._check(self.lib.octgb_xmean(self.h, p, loc, F, nx, nz, out.ctypes.data))
        return out

    # -------------------------------------------------------------- quantisation
    def quantise(self, db, clim, out=None):
        p, loc = _ptr(db)
        n = int(np.prod(db.shape))
        if out is None:
            out = np.empty(db.shape, np.uint16)
        op, oloc = _ptr(out)
        c1, c2 = sorted(float(c) for c in clim)
        self._check(self.lib.octgb_quantise(self.h, p, n, loc, c1, c2, op, oloc))
        return out

    def quantise_double(self, db, plane_clim, clim, out=None):
        """Legacy double quantisation (tiff_writer.py:62-64) of one plane."""
        p, loc = _ptr(db)
        n = int(np.prod(db.shape))
        if out is None:
            out = np.empty(db.shape, np.uint16)
        op, oloc = _ptr(out)
        p1, p2 = (float(v) for v in plane_clim)
        c1, c2 = sorted(float(v) for v in clim)
        self._check(self.lib.octgb_quantise_double(self.h, p, n, loc, p1, p2, c1, c2, op, oloc))
        return out

    def packbits(self, img):
        """PackBits of every row of a (rows, cols) uint16 image -> (bytes, row sizes)."""
        rows, cols = img.shape
        if isinstance(img, np.ndarray):
            img = np.ascontiguousarray(img, dtype=np.uint16)
        p, loc = _ptr(img)
        cap = rows * (2 * cols + (2 * cols + 127) // 128 + 1)
        out = np.empty(max(cap, 1), np.uint8)
        sizes = np.empty(max(rows, 1), np.int32)
        total = ctypes.c_int64(0)
        self._check(self.lib.octgb_packbits(self.h, p, loc, rows, cols, out.ctypes.data, cap, sizes.ctypes.data,
                                            ctypes.byref(total)))
        return out[:total.value].tobytes(), sizes[:rows]

    def minmax(self, db):
        p, loc = _ptr(db)
        mm = np.full(2, np.nan)
        self._check(self.lib.octgb_minmax(self.h, p, int(np.prod(db.shape)), loc, mm.ctypes.data))
        return float(mm[0]), float(mm[1])

    # -------------------------------------------------------------- stitching
    def stitch_plan(self, n_rows, r0, r1, c0, c1, Wz, WxT, fz, shift=None, pdz=None) -> int:
        Wz = np.ascontiguousarray(Wz, dtype=np.float64)
        WxT = np.ascontiguousarray(WxT, dtype=np.float64)
        fz = np.ascontiguousarray(fz, dtype=np.float64)
        sh = None if shift is None else np.ascontiguousarray(shift, dtype=np.int64)
        pz = None if pdz is None else np.ascontiguousarray(pdz, dtype=np.float64)
        n_y = 0 if sh is None else sh.shape[0]
        pid = c_int(-1)
        self._check(self.lib.octgb_stitch_plan(
            self.h, int(n_rows), int(r0), int(r1), int(c0), int(c1), Wz.shape[0], WxT.shape[0],
            Wz.ctypes.data, WxT.ctypes.data, fz.ctypes.data,
            None if sh is None else sh.ctypes.data, None if pz is None else pz.ctypes.data, n_y, ctypes.byref(pid)))
        return pid.value

    def row_begin(self, n_frames: int, n_out_z: int, n_out_x: int):
        self._check(self.lib.octgb_row_begin(self.h, int(n_frames), int(n_out_z), int(n_out_x)))

    def row_add_batch(self, plan_id: int, raw, apod_size: int, frame_idx, frame_offset: int, raw_dtype=None):
        raw, p, loc, dt, B, interf = self._raw_args(raw, apod_size, raw_dtype)
        fi = np.ascontiguousarray(np.asarray(frame_idx).reshape(-1), dtype=np.int64)
        if len(fi) != B:
            raise ValueError("frame_idx must have one entry per B-scan")
        self._check(self.lib.octgb_row_add_batch(self.h, int(plan_id), p, dt, loc, B, interf, int(apod_size),
                                                 fi.ctypes.data, int(frame_offset)))

    def row_add_batch_ex(self, plan_id: int, raw, apod_size: int, frame_idx, frame_offset: int, binning: int = 1,
                         apod_mode: int = 0, bscan_avg: int = 1, ascan_avg: int = 1, raw_dtype=None):
        """One batch of a rare-format scan: len(frame_idx) frames x bscan_avg raw files."""
        raw, p, loc, dt, n_files, n_lines = self._raw_args(raw, apod_size if apod_mode == 0 else 1, raw_dtype)
        fi = np.ascontiguousarray(np.asarray(frame_idx).reshape(-1), dtype=np.int64)
        self._check(self.lib.octgb_row_add_batch_ex(self.h, int(plan_id), p, dt, loc, n_files, n_lines,
                                                    int(apod_size), int(binning), int(apod_mode), int(bscan_avg),
                                                    int(ascan_avg), fi.ctypes.data, len(fi), int(frame_offset)))

    def row_finalise(self, threshold: float, shape, out=None, plane_minmax: bool = False):
        if out is None:
            out = np.empty(shape, np.float32)
        op, oloc = _ptr(out)
        mm = np.full((shape[0], 2), np.nan) if plane_minmax else None
        self._check(self.lib.octgb_row_finalise(self.h, c_float(threshold), op, oloc,
                                                None if mm is None else mm.ctypes.data))
        return (out, mm) if plane_minmax else out

    # -------------------------------------------------------------- frame batches
    def frames_process(self, plan_ids, raws, apod_size: int, f0: int, n_out_z: int, n_out_x: int,
                       threshold: float, out=None, plane_minmax: bool = False, raw_dtype=None):
        """Spectral + stitch + finalise of one frame batch over several tiles
        (raws[t] of shape (B, interf, N), all on the host or all on the device)."""
        n = len(raws)
        if n != len(plan_ids) or n == 0:
            raise ValueError("one raw batch per plan id")
        ptrs, locs, keep = [], set(), []
        dt = None
        for r in raws:
            r2, p, loc, d, B, interf = self._raw_args(r, apod_size, raw_dtype)
            keep.append(r2)
            ptrs.append(p)
            locs.add(loc)
            dt = d if dt is None else dt
            if d != dt:
                raise ValueError("all raw batches must share one dtype")
        if len(locs) != 1:
            raise ValueError("raw batches must all be host or all device arrays")
        if out is None:
            out = np.empty((B, n_out_z, n_out_x), np.float32)
        op, oloc = _ptr(out)
        ids = (c_int * n)(*[int(i) for i in plan_ids])
        arr = (c_void_p * n)(*ptrs)
        mm = np.full((B, 2), np.nan) if plane_minmax else None
        self._check(self.lib.octgb_frames_process(
            self.h, n, ids, arr, dt, locs.pop(), B, interf, int(apod_size), int(f0), int(n_out_z), int(n_out_x),
            c_float(threshold), op, oloc, None if mm is None else mm.ctypes.data))
        return (out, mm) if plane_minmax else out

    def clim_reset(self):
        self._check(self.lib.octgb_clim_reset(self.h))

    def clim_get(self):
        c = np.full(2, np.nan)
        self._check(self.lib.octgb_clim_get(self.h, c.ctypes.data))
        return float(c[0]), float(c[1])

    def quantise_running(self, db, out):
        p, loc = _ptr(db)
        op, oloc = _ptr(out)
        self._check(self.lib.octgb_quantise_running(self.h, p, int(np.prod(db.shape)), loc, op, oloc))
        return out

    # -------------------------------------------------------------- graphs
    def graph_begin(self):
        self._check(self.lib.octgb_graph_begin(self.h))

    def graph_end(self) -> int:
        gid = c_int(-1)
        self._check(self.lib.octgb_graph_end(self.h, ctypes.byref(gid)))
        return gid.value

    def graph_launch(self, gid: int):
        self._check(self.lib.octgb_graph_launch(self.h, int(gid)))

    def graphs_release(self):
        """Destroy the context's captured graphs (a new geometry is refused while any exist)."""
        self._check(self.lib.octgb_graphs_release(self.h))

    def set_stitch_rows(self, rows: int):
        """Output rows per block of frames_process's stitch kernel (32, 64 or 128; results do not depend on it)."""
        self._check(self.lib.octgb_set_stitch_rows(self.h, int(rows)))

    # -------------------------------------------------------------- batched form
    def batch_process(self, tiles, threshold: float, grab: int = 4, raw_dtype: int = U16):
        """tiles: list of (raw_device_tensor (B, interf, N), apod_size, plan_id, db_device_tensor)."""
        arr = (OctgbTile * len(tiles))()
        for k, (raw, apod, plan, db) in enumerate(tiles):
            B, interf, N = raw.shape
            if N != self.n:
                raise ValueError("spectral length differs from the geometry")
            arr[k] = OctgbTile(raw.data_ptr(), B, interf, int(apod), int(plan), db.data_ptr())
        self._check(self.lib.octgb_batch_process(self.h, len(tiles), arr, int(raw_dtype), c_float(threshold),
                                                 int(grab)))
