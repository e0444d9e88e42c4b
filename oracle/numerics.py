"""ORACLE numerics — test infrastructure only (see oracle/__init__.py).

Each function restates one piece of the reference `octrecon` path on the CPU and
cites the reference file:line it follows.  Nothing here is used by the product.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIB = None

# ----------------------------------------------------------------------------- C kernel


def build(force: bool = False) -> Path:
    """Compile oracle/fused_pre_fft.c into oracle/_build/liboracle.so (Makefile)."""
    so = HERE / "_build" / "liboracle.so"
    src = HERE / "fused_pre_fft.c"
    if force or not so.exists() or so.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return so


def _lib():
    global _LIB
    if _LIB is None:
        lib = ctypes.CDLL(str(build()))
        lib.oracle_fused_pre_fft.restype = ctypes.c_int
        lib.oracle_fused_pre_fft.argtypes = [
            ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _LIB = lib
    return _LIB


_DT = {np.dtype(np.uint16): 0, np.dtype(np.int16): 1, np.dtype(np.float32): 2}


def fused_pre_fft_numba(raw: np.ndarray, apod_size: int, idx: np.ndarray, w: np.ndarray,
                        window: np.ndarray) -> np.ndarray:
    """core/cpu_kernels.py:12-41 restated in C (exact Numba types).

    raw (B, interf, N) uint16/int16/float32; idx (T, N) int; w (T, N) float32;
    window (N,) complex64 -> complex64 (B, nX, N)."""
    raw = np.ascontiguousarray(raw)
    if raw.dtype not in _DT:
        raw = raw.astype(np.float32)
    B, interf, N = raw.shape
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    w = np.ascontiguousarray(w, dtype=np.float32)
    T = idx.shape[0]
    win = np.ascontiguousarray(np.stack([window.real, window.imag], -1).astype(np.float32))
    out = np.empty((B, interf - apod_size, N), np.complex64)
    rc = _lib().oracle_fused_pre_fft(raw.ctypes.data, _DT[raw.dtype], B, interf, apod_size, N, T,
                                     idx.ctypes.data, w.ctypes.data, win.ctypes.data, out.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_fused_pre_fft failed ({rc})")
    return out


def ifft_rows(a: np.ndarray) -> np.ndarray:
    """core/spectral.py:160-164: pocketfft (scipy.fft.ifft, 1/N scaling), all cores."""
    import scipy.fft
    return scipy.fft.ifft(a, axis=-1, workers=os.cpu_count(), overwrite_x=True)


# ----------------------------------------------------------------------------- geometry
LAMBDA_RANGE_NM = {  # core/geometry.py:18-24
    "ganymede": (796.23, 1010.02), "ganymede_srr": (796.23, 1010.02), "gan632": (796.0, 1010.0),
    "telesto": (1208.69, 1372.50), "telesto_srr": (1208.69, 1372.50),
}


def matlab_linspace(a, b, n):
    """core/geometry.py:30-35."""
    y = a + (np.arange(n) * (b - a)) / (n - 1)
    y[0] = a
    y[-1] = b
    return y


def matlab_colon(a, d, b):
    """core/geometry.py:38-51 (MATLAB a:d:b, symmetric evaluation)."""
    tol = 2.0 * np.finfo(float).eps * max(abs(a), abs(b))
    n = int(np.floor((b - a) / d + tol / abs(d))) if d != 0 else -1
    if n < 0:
        return np.zeros(0)
    k = np.arange(n + 1, dtype=float)
    out = np.empty(n + 1)
    half = n // 2
    end = a + n * d
    out[: half + 1] = a + k[: half + 1] * d
    out[half + 1:] = end - (n - k[half + 1:]) * d
    return out


def chirp_to_lambda(chirp, oct_system):
    """core/geometry.py:57-60."""
    lmin, lmax = LAMBDA_RANGE_NM[oct_system.lower()]
    n = len(chirp)
    return 1.0 / (chirp * (1.0 / (n - 1) * (1.0 / lmax - 1.0 / lmin)) + 1.0 / lmin)


@dataclass
class Geometry:
    lambda_nm: np.ndarray
    k: np.ndarray
    k_lin: np.ndarray
    lambda_eq_nm: np.ndarray
    sinc_idx: np.ndarray    # (N, T)
    sinc_w: np.ndarray      # (N, T) float64
    window: np.ndarray      # (N,) complex128
    z_um: np.ndarray


def spectral_geometry(lambda_nm, dispersion, n_medium, interp_method="sinc5") -> Geometry:
    """core/geometry.py:84-128, dense (N, N) distance-matrix form as in the reference."""
    from scipy.interpolate import PchipInterpolator
    lam = np.asarray(lambda_nm, float).ravel()
    N = len(lam)
    k = 2 * np.pi / lam
    k_lin = matlab_linspace(k.max(), k.min(), N)
    taps = int(interp_method.lower()[4:])
    nq = (k_lin - k_lin.min()) / (k_lin.max() - k_lin.min()) * (N - 1)
    n = (k - k.min()) / (k.max() - k.min()) * (N - 1)
    dist = nq[:, None] - n[None, :]
    mask = np.abs(dist) < taps
    T = int(mask.sum(1).max())
    idx = np.zeros((N, T), np.int64)
    w = np.zeros((N, T), float)
    for i in range(N):
        jj = np.nonzero(mask[i])[0]
        idx[i, : len(jj)] = jj
        w[i, : len(jj)] = np.sinc(dist[i, jj])
    x, v = k, lam
    if x[0] > x[-1]:
        x, v = x[::-1], v[::-1]
    lambda_eq = PchipInterpolator(x, v, extrapolate=True)(k_lin)
    k_eq = 2 * np.pi / lambda_eq
    hann = 0.5 * (1 - np.cos(2 * np.pi * np.arange(N) / (N - 1)))
    hann = hann / np.sqrt(np.mean(hann ** 2))
    window = hann * np.exp(1j * (-dispersion * (k_eq - k_eq.mean()) ** 2))
    l_sorted = np.sort([lambda_eq[0], lambda_eq[-1]])
    lambda0_um = l_sorted.mean() / 1e3
    dlambda_um = np.diff(l_sorted)[0] / 1e3
    z_step = 0.5 * lambda0_um ** 2 / dlambda_um / n_medium
    z_um = matlab_linspace(0.0, z_step * N / 2, N // 2)
    return Geometry(lam, k, k_lin, lambda_eq, idx, w, window, z_um)


# ----------------------------------------------------------------------------- spectral stage


def magnitude_numba(raw, g: Geometry, apod_size: int) -> np.ndarray:
    """core/spectral.py:136-153 with use_numba=True at float32: Numba pre-FFT
    (restated in C), pocketfft complex64 ifft, |.| of the first N/2 bins."""
    N = len(g.lambda_nm)
    spec = fused_pre_fft_numba(raw, apod_size, g.sinc_idx.T, g.sinc_w.T.astype(np.float32),
                               g.window.astype(np.complex64))
    ft = ifft_rows(spec)
    return np.abs(ft[..., : N // 2]).astype(np.float32, copy=False)


def magnitude_numba_exact_fft(raw, g: Geometry, apod_size: int) -> np.ndarray:
    """The Numba path's complex64 spectrum (core/cpu_kernels.py:12-41) through
    an inverse FFT without float32 rounding (complex128), |.| rounded to
    float32.  Against magnitude_numba this measures pocketfft's own float32
    rounding (core/spectral.py:160-164): the deviation from the reference
    path that any float32 FFT of another operation order starts from."""
    N = len(g.lambda_nm)
    spec = fused_pre_fft_numba(raw, apod_size, g.sinc_idx.T, g.sinc_w.T.astype(np.float32),
                               g.window.astype(np.complex64))
    ft = ifft_rows(spec.astype(np.complex128))
    return np.abs(ft[..., : N // 2]).astype(np.float32)


def linearise_numpy(raw, g: Geometry, apod_size: int, dtype) -> np.ndarray:
    """core/spectral.py:123-134 (the unfused NumPy path) at `dtype`."""
    x = np.asarray(raw).astype(dtype, copy=False)
    apod = x[:, :apod_size, :].mean(axis=1, keepdims=True)
    interf = x[:, apod_size:, :] - apod
    mv = interf.mean(axis=-1, keepdims=True)
    d = interf - mv
    idx = g.sinc_idx.T
    w = g.sinc_w.T.astype(dtype)
    out = np.zeros_like(d)
    for t in range(idx.shape[0]):
        out += w[t] * np.take(d, idx[t], axis=-1)
    out += mv
    return out


def magnitude_numpy(raw, g: Geometry, apod_size: int, dtype=np.float64) -> np.ndarray:
    """core/spectral.py:136-153 with use_numba=False: NumPy path at `dtype`
    (float64 = the FP64 oracle; float32 = the reference's NumPy float32 path)."""
    N = len(g.lambda_nm)
    cdt = np.complex64 if np.dtype(dtype) == np.float32 else np.complex128
    spec = linearise_numpy(raw, g, apod_size, dtype) * g.window.astype(cdt)
    ft = ifft_rows(spec)
    return np.abs(ft[..., : N // 2]).astype(dtype, copy=False)


def pre_fft_numpy(raw, g: Geometry, apod_size: int, dtype=np.float64) -> np.ndarray:
    """Stage (b)-(d) output of the NumPy path: linearised spectrum x window."""
    cdt = np.complex64 if np.dtype(dtype) == np.float32 else np.complex128
    return linearise_numpy(raw, g, apod_size, dtype) * g.window.astype(cdt)


# ----------------------------------------------------------------------------- stitching
CUTOFF_SIGMA = 3.0
MIN_WEIGHT = float(np.exp(-CUTOFF_SIGMA ** 2 / 2))      # core/stitching.py:20-21


def min_weight_threshold(dtype) -> float:
    """core/stitching.py:24-28."""
    return MIN_WEIGHT * (1.0 - 8 * float(np.finfo(dtype).eps))


def factor_z(n_rows, focus_pix_1based, focus_sigma):
    """core/stitching.py:31-33 (note the (2 sigma)^2 denominator)."""
    zI = np.arange(1, n_rows + 1, dtype=float)
    return np.exp(-(zI - focus_pix_1based) ** 2 / (2 * focus_sigma) ** 2) + np.exp(-3.0 ** 2 / 2)


def linear_interp_matrix(src, dst):
    """core/stitching.py:36-51 (MATLAB linear interpolation, 0 outside, 1e-9 node snap)."""
    W = np.zeros((len(dst), len(src)))
    inside = (dst >= src[0]) & (dst <= src[-1])
    q = dst[inside]
    j = np.searchsorted(src, q, side="right") - 1
    j = np.clip(j, 0, len(src) - 2)
    t = (q - src[j]) / (src[j + 1] - src[j])
    t[np.abs(t) < 1e-9] = 0.0
    t[np.abs(1.0 - t) < 1e-9] = 1.0
    rows = np.nonzero(inside)[0]
    W[rows, j] += 1 - t
    W[rows, j + 1] += t
    return W


@dataclass
class ScanDesc:
    """The ScanInfo.json fields the tiled geometry reads (io/scaninfo.py:26-65)."""
    x_centers_mm: np.ndarray
    y_centers_mm: np.ndarray
    z_depths_mm: np.ndarray
    n_x_px: int
    n_y_px: int
    tile_range_x_mm: float
    tile_range_y_mm: float
    x_offset: float = 0.0
    y_offset: float = 0.0


@dataclass
class Tiled:
    tile_x_mm: np.ndarray
    tile_y_mm: np.ndarray
    tile_z_mm: np.ndarray
    out_x_mm: np.ndarray
    out_y_mm: np.ndarray
    out_z_mm: np.ndarray
    focus_pix: np.ndarray


def tiled_geometry(si: ScanDesc, z_um_tile, focus_pix, output_pixel_size_um, crop_z_range_mm=None) -> Tiled:
    """core/geometry.py:146-202 (galvo correction term assumed 0, as the synthetic
    scans set galvoPhaseDelayXOffsetCorrection_mm)."""
    nd = len(si.z_depths_mm)
    focus = np.asarray(focus_pix, float).ravel()
    if focus.size == 1:
        focus = np.full(nd, focus[0])
    tx = si.x_offset + si.tile_range_x_mm * matlab_linspace(-0.5, 0.5, si.n_x_px + 1)
    ty = si.y_offset + si.tile_range_y_mm * matlab_linspace(-0.5, 0.5, si.n_y_px + 1)
    tx, ty = tx[:-1], ty[:-1]
    tz = np.asarray(z_um_tile) / 1e3
    if not np.any(np.isnan(focus)):
        ref = focus[0] if np.all(focus == focus[0]) else focus[int(np.argmin(np.abs(si.z_depths_mm)))]
        tz = tz - tz[int(np.round(ref)) - 1]
    dx = tx[1] - tx[0]
    dy = ty[1] - ty[0] if len(ty) > 1 else 0.0
    dz = tz[1] - tz[0]
    xc, yc, zd = si.x_centers_mm, si.y_centers_mm, si.z_depths_mm
    x_all = matlab_colon(xc.min() + tx[0], dx, xc.max() + tx[-1] + dx / 2)
    y_all = matlab_colon(yc.min() + ty[0], dy, yc.max() + ty[-1] + dy / 2)
    z_all = matlab_colon(zd.min() + tz[0], dz, zd.max() + tz[-1] + dz / 2)
    zero = int(np.argmin(np.abs(z_all)))
    z_all = dz * (np.arange(1, len(z_all) + 1) - (zero + 1))
    if len(xc) == 1:
        x_all = tx.copy()
    if len(yc) == 1:
        y_all = ty.copy()
    if output_pixel_size_um is not None:
        z_all = matlab_colon(z_all[0], output_pixel_size_um * 1e-3, z_all.max())
    if crop_z_range_mm is not None and len(crop_z_range_mm):
        lo, hi = crop_z_range_mm
        z_all = z_all[~((z_all < lo) | (z_all > hi))]
    return Tiled(tx, ty, tz, x_all, y_all, z_all, focus)


class Stitcher:
    """core/stitching.py:84-139 (TileStitcher, without optical-path correction)."""

    def __init__(self, tg: Tiled, xi_center_mm, z_depth_mm, focus_pix, focus_sigma, dtype=np.float32):
        nz = len(tg.tile_z_mm)
        x = tg.tile_x_mm + xi_center_mm
        z = tg.tile_z_mm + z_depth_mm
        if not np.isnan(focus_pix):
            z = z - tg.tile_z_mm[int(np.round(focus_pix)) - 1]
        x = x.copy(); z = z.copy()
        x[0] -= 1e-10; x[-1] += 1e-10
        z[0] -= 1e-10; z[-1] += 1e-10
        Wz = linear_interp_matrix(z, tg.out_z_mm)
        Wx = linear_interp_matrix(x, tg.out_x_mm)
        rows = np.nonzero(Wz.any(axis=0))[0]
        cols = np.nonzero(Wx.any(axis=1))[0]
        self.empty = rows.size == 0 or cols.size == 0
        if self.empty:
            return
        self.r0, self.r1 = int(rows[0]), int(rows[-1] + 1)
        self.c0, self.c1 = int(cols[0]), int(cols[-1] + 1)
        self.Wz = Wz[:, self.r0:self.r1].astype(dtype)
        self.WxT = Wx[self.c0:self.c1, :].T.astype(dtype)
        fz = factor_z(nz, focus_pix, focus_sigma) if not np.isnan(focus_pix) else np.ones(nz)
        self.fz = fz[self.r0:self.r1].astype(dtype)
        self.dtype = dtype

    def contribute(self, mag):
        """core/stitching.py:122-139 with oc=None: (B, nX, nZ) -> (num, den) (B, nOutZ, C)."""
        a = mag[..., self.r0:self.r1]
        f = np.broadcast_to(self.fz, a.shape).astype(self.dtype)
        a = a * f
        num = np.matmul(np.matmul(a, self.Wz.T).transpose(0, 2, 1), self.WxT)
        den = np.matmul(np.matmul(f, self.Wz.T).transpose(0, 2, 1), self.WxT)
        return num, den


def finalise(num, den, dtype=np.float32):
    """pipeline.py:296-300: weight below threshold -> NaN, 20*log10(num/den)."""
    den = den.copy()
    den[den < min_weight_threshold(dtype)] = np.nan
    with np.errstate(divide="ignore", invalid="ignore"):
        return (20 * np.log10(num / den)).astype(np.float32, copy=False)


# ----------------------------------------------------------------------------- quantisation
MAXBIT = 2 ** 16 - 1


def matlab_uint16(v):
    """io/tiff_writer.py:26-30."""
    out = np.floor(np.abs(v) + 0.5) * np.sign(v)
    out = np.nan_to_num(out, nan=0.0)
    return np.clip(out, 0, MAXBIT).astype(np.uint16)


def db_to_bits(db, clim):
    """io/tiff_writer.py:33-38 (evaluated in float64, as write_legacy_tiff does :62)."""
    db = np.asarray(db, dtype=np.float64)
    c1, c2 = sorted(clim)
    bits = matlab_uint16((db - c1) / (c2 - c1) * (MAXBIT - 1)).astype(np.uint32) + 1
    bits = np.minimum(bits, MAXBIT).astype(np.uint16)
    bits[np.isnan(db)] = 0
    return bits


def bits_to_db(bits, clim):
    """io/tiff_writer.py:41-45."""
    c1, c2 = sorted(clim)
    out = (bits.astype(np.float64) - 1) * (c2 - c1) / (MAXBIT - 1) + c1
    out[bits == 0] = np.nan
    return out


def plane_clim(db):
    """io/tiff_writer.py:48-50."""
    fin = db[np.isfinite(db)]
    return (float(fin.min()), float(fin.max())) if fin.size else (np.nan, np.nan)


def lsb_report(a_db, b_db, clim, floor_db=None):
    """Quantise two dB arrays with ONE shared clim and compare the codes.

    Returns dict(max_lsb, exact_frac, n) over voxels finite in both (and above
    `floor_db` in b when given)."""
    qa = db_to_bits(a_db, clim).astype(np.int64)
    qb = db_to_bits(b_db, clim).astype(np.int64)
    sel = np.isfinite(a_db) & np.isfinite(b_db)
    if floor_db is not None:
        sel &= np.asarray(b_db) > floor_db
    d = np.abs(qa - qb)[sel]
    return {"max_lsb": int(d.max()) if d.size else 0, "exact_frac": float((d == 0).mean()) if d.size else 1.0,
            "n": int(d.size)}


# dB levels relative to the reference's median (deep noise floor to strong reflectors)
DB_LEVELS = ((-np.inf, -30.0), (-30.0, -20.0), (-20.0, -10.0), (-10.0, 0.0), (0.0, 10.0), (10.0, np.inf))


def lsb_levels(a_db, b_db, clim, levels=DB_LEVELS):
    """Codes of a and b with ONE shared clim, compared per dB level of b
    (relative to b's median over voxels finite in both).  Returns a list of
    dict(lo, hi, n, exact_frac, max_lsb, n_diff), the overall row last
    (lo = hi = None)."""
    a_db, b_db = np.asarray(a_db), np.asarray(b_db)
    qa = db_to_bits(a_db, clim).astype(np.int64)
    qb = db_to_bits(b_db, clim).astype(np.int64)
    sel = np.isfinite(a_db) & np.isfinite(b_db)
    d = np.abs(qa - qb)[sel]
    rel = np.asarray(b_db, np.float64)[sel]
    rel = rel - np.median(rel)
    rows = []
    for lo, hi in tuple(levels) + ((None, None),):
        m = np.ones(d.shape, bool) if lo is None else (rel >= lo) & (rel < hi)
        dm = d[m]
        rows.append({"lo": lo, "hi": hi, "n": int(dm.size), "n_diff": int((dm != 0).sum()),
                     "exact_frac": float((dm == 0).mean()) if dm.size else 1.0,
                     "max_lsb": int(dm.max()) if dm.size else 0})
    return rows


def format_levels(name, rows):
    """One printable line per level table."""
    out = [f"{name}:"]
    for r in rows:
        lvl = "all" if r["lo"] is None else f"[{r['lo']:g},{r['hi']:g}) dB"
        out.append(f"  {lvl:>14s} n={r['n']:9d} exact={100 * r['exact_frac']:8.4f}% max={r['max_lsb']} LSB")
    return "\n".join(out)


# ----------------------------------------------------------------------------- estimation
Z_MIN_PIX = 20                                           # estimation/dispersion.py:40
TOP_FRACTION = 0.01                                      # estimation/dispersion.py:41


def disp_metric(A, name):
    """estimation/dispersion.py:46-63: (B, nX, nZ) float32 magnitude -> (B,)
    sharpness, depth pixels >= 20 only; I = (A^2 in float32) as float64."""
    B = A.shape[0]
    if name == "legacy_peak":
        return np.log(A[:, :, Z_MIN_PIX:] + 1e-12).mean(axis=1).max(axis=1)
    I = (A[:, :, Z_MIN_PIX:] ** 2).reshape(B, -1).astype(np.float64)
    if name == "top_percentile":
        M = I.shape[1]
        k = max(1, int(M * TOP_FRACTION))
        return np.log(np.partition(I, M - k, axis=1)[:, M - k:].mean(axis=1))
    if name == "kurtosis":
        return (I ** 2).sum(axis=1) / I.sum(axis=1) ** 2
    if name == "entropy":
        p = I / I.sum(axis=1, keepdims=True)
        return (p * np.log(p + 1e-30)).sum(axis=1)
    raise ValueError(name)


class DispScorer:
    """estimation/dispersion.py:66-107 over raw arrays: X = linearise * Hann/rms
    once (complex64), then per beta ifft(X * exp(-i beta dk^2)) |.| of the
    first N/2 bins, mean over repeats, metric.  raw_list: (rep, interf, N)."""

    def __init__(self, lambda_nm, raw_list, metric, apod_size):
        g = spectral_geometry(lambda_nm, 0.0, 1.33)
        N = len(g.lambda_nm)
        self.nz = N // 2
        self.metric = metric
        hann = 0.5 * (1 - np.cos(2 * np.pi * np.arange(N) / (N - 1)))
        hann = hann / np.sqrt(np.mean(hann ** 2))
        k_eq = 2 * np.pi / g.lambda_eq_nm
        self.dk2 = (k_eq - k_eq.mean()) ** 2
        self.X = np.stack([(linearise_numpy(r, g, apod_size, np.float32) * hann).astype(np.complex64)
                           for r in raw_list])                      # (B, rep, nX, N)

    def magnitude(self, beta, idx=None):
        X = self.X if idx is None else self.X[idx:idx + 1]
        spec = X * np.exp(-1j * float(beta) * self.dk2).astype(np.complex64)
        return np.abs(ifft_rows(spec)[..., : self.nz]).mean(axis=1)

    def scores(self, beta, idx=None):
        return disp_metric(self.magnitude(beta, idx), self.metric)


# ----------------------------------------------------------------------------- rare raw formats
def bin_ascans(x, binning):
    """core/spectral.py:27-45 AScanBinning: filter2 'same' (zero padded) average
    of `binning` consecutive A-lines, decimated from max(1, B//2) - 1; the
    window of kept column c is lines c - ceil(B/2) + 1 .. c + floor(B/2); sum
    acc = x0*h, acc = acc + xt*h in the array's dtype, h = 1/B."""
    x = np.asarray(x)
    n = x.shape[-2]
    s0 = max(1, binning // 2) - 1
    cols = np.arange(s0, n, binning)
    left = (binning + 1) // 2 - 1
    h = x.dtype.type(1.0 / binning)
    out = None
    for t in range(binning):
        lines = cols + t - left
        ok = (lines >= 0) & (lines < n)
        sl = np.zeros(x.shape[:-2] + (len(cols), x.shape[-1]), x.dtype)
        sl[..., ok, :] = x[..., lines[ok], :]
        term = sl * h
        out = term if out is None else out + term
    return out


def prepare_raw(raw, apod_size, binning=1, apod_mode="lines", apod_group=1, dtype=np.float32):
    """core/spectral.py:48-68: float array whose first lines are the
    apodisation (apod_size lines, or the frame mean for apod_mode 'frame_mean':
    mean over a file's lines, then over its frame's apod_group files), then the
    (binned) scan lines; `raw` itself when nothing applies."""
    if apod_mode == "frame_mean":
        x = np.asarray(raw).astype(dtype)
        B, nL, N = x.shape
        g = max(1, int(apod_group))
        apod = x.reshape(B // g, g, nL, N).mean(axis=2).mean(axis=1)
        apod = np.repeat(apod, g, axis=0)[:, None, :]
        if binning > 1:
            x = bin_ascans(x, binning)
        return np.concatenate([apod, x], axis=1)
    if binning > 1:
        x = np.asarray(raw).astype(dtype)
        return np.concatenate([x[:, :apod_size, :], bin_ascans(x[:, apod_size:, :], binning)], axis=1)
    return raw


def srr_decode(words, apod_range, scan_range):
    """io/srr.py:108-125: SRR words (files, file_lines, n) uint16 -> int16
    (files, apod + scan lines, n): every word modulo 4096 (only the low 12 bits
    are data, :118), then each file's apodisation lines [apodstart, apodend)
    followed by its scan lines [scanstart, scanend) (read_bscans, :120-125)."""
    w = (np.asarray(words, dtype=np.uint16) % 4096).astype(np.int16)
    a0, a1 = apod_range
    s0, s1 = scan_range
    return np.concatenate([w[:, a0:a1], w[:, s0:s1]], axis=1)


def average_repeats(mag, n_frames, bscan_avg, size_x, ascan_avg):
    """core/spectral.py:168-177: mean over B-scan repeats, then A-scan repeats."""
    nb, na = max(1, bscan_avg), max(1, ascan_avg)
    if nb == 1 and na == 1:
        return mag
    m5 = np.asarray(mag).reshape(n_frames, nb, size_x, na, mag.shape[-1])
    m4 = m5.mean(1) if nb > 1 else m5[:, 0]
    return m4.mean(2) if na > 1 else m4[:, :, 0]


# ----------------------------------------------------------------------------- legacy TIFF encoding
def legacy_double_bits(plane, plane_clim_, clim):
    """io/tiff_writer.py:62-64: the legacy double quantisation of one plane."""
    p = np.asarray(plane, np.float64)
    return db_to_bits(bits_to_db(db_to_bits(p, plane_clim_), plane_clim_), clim)


def packbits_encode_row(row_bytes: bytes) -> bytes:
    """PackBits of one row (TIFF compression 32773, rows packed separately):
    runs of >= 3 equal bytes (up to 128) as repeat packets, the rest as
    literal packets of up to 128 bytes."""
    b, n, i, out = row_bytes, len(row_bytes), 0, bytearray()
    while i < n:
        run = 1
        while i + run < n and run < 128 and b[i + run] == b[i]:
            run += 1
        if run >= 3:
            out += bytes([(257 - run) & 0xff, b[i]])
            i += run
            continue
        j = i
        while j < n and j - i < 128:
            if j + 2 < n and b[j] == b[j + 1] == b[j + 2]:
                break
            j += 1
        out += bytes([j - i - 1]) + b[i:j]
        i = j
    return bytes(out)
