"""Host-side FP64 spectral geometry: k-map, sinc band, window and depth axis.

Built once per scan (or per dispersion value) and uploaded to the device.  The
results are the same numbers the reference builds in
octrecon/core/geometry.py:84-128 (`build_spectral_geometry`): the sinc taps of
output sample i are the source samples j with |nq_i - n_j| < taps in increasing
j, zero-padded to the widest row; the window is the RMS-normalised symmetric
Hann times exp(-i*beta*(k_eq - mean k_eq)^2); the depth axis follows
yOCTInterfToScanCpx_getZ.

Unlike the reference (which forms an N x N distance matrix), the band of each
output row is located by binary search on the monotonic source positions, so a
2048-sample geometry takes O(N log N) work and no O(N^2) temporaries.  The
band is also summarised per output row as (first source index, tap count),
which is the form the device kernels consume.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

LAMBDA_RANGE_NM = {  # per-system wavelength range (octrecon/core/geometry.py:18-24)
    "ganymede": (796.23, 1010.02),
    "ganymede_srr": (796.23, 1010.02),
    "gan632": (796.0, 1010.0),
    "telesto": (1208.69, 1372.50),
    "telesto_srr": (1208.69, 1372.50),
}


def linspace_matlab(a: float, b: float, n: int) -> np.ndarray:
    """MATLAB linspace with exact end points (octrecon/core/geometry.py:30-35)."""
    y = a + (np.arange(n) * (b - a)) / (n - 1)
    y[0], y[-1] = a, b
    return y


def colon_matlab(a: float, d: float, b: float) -> np.ndarray:
    """MATLAB a:d:b: count with MATLAB's 2*eps tolerance, first half stepped from a,
    second half stepped back from the end point (octrecon/core/geometry.py:38-51)."""
    if d == 0:
        return np.zeros(0)
    tol = 2.0 * np.finfo(float).eps * max(abs(a), abs(b))
    n = int(np.floor((b - a) / d + tol / abs(d)))
    if n < 0:
        return np.zeros(0)
    k = np.arange(n + 1, dtype=float)
    h = n // 2
    return np.concatenate([a + k[: h + 1] * d, (a + n * d) - (n - k[h + 1:]) * d])


def chirp_to_lambda(chirp: np.ndarray, oct_system: str) -> np.ndarray:
    """Per-pixel wavelength from a Thorlabs chirp (octrecon/core/geometry.py:57-60)."""
    lmin, lmax = LAMBDA_RANGE_NM[oct_system.lower()]
    n = len(chirp)
    return 1.0 / (np.asarray(chirp, float) * ((1.0 / lmax - 1.0 / lmin) / (n - 1)) + 1.0 / lmin)


def _pchip(x: np.ndarray, y: np.ndarray, xq: np.ndarray) -> np.ndarray:
    """MATLAB interp1(..., 'pchip') for strictly monotonic x (either direction),
    with extrapolation (the reference calls scipy's PchipInterpolator,
    octrecon/core/geometry.py:63-68)."""
    from scipy.interpolate import PchipInterpolator
    x = np.asarray(x, float)
    if x[0] > x[-1]:
        x, y = x[::-1], y[::-1]
    return PchipInterpolator(x, y, extrapolate=True)(xq)


@dataclass
class SpectralGeometry:
    lambda_nm: np.ndarray      # (N,) raw per-pixel wavelength
    k: np.ndarray              # (N,) 2*pi/lambda (1/nm)
    k_lin: np.ndarray          # (N,) equispaced target k, descending
    lambda_eq_nm: np.ndarray   # (N,) wavelength of the equispaced samples
    sinc_idx: np.ndarray       # (N, T) int64 source indices (padding: 0)
    sinc_w: np.ndarray         # (N, T) float64 weights (padding: 0)
    band_start: np.ndarray     # (N,) int32 first source index of each output row
    band_len: np.ndarray       # (N,) int32 taps used by each output row
    window: np.ndarray         # (N,) complex128 Hann/rms * exp(i*phase)
    z_um: np.ndarray           # (N/2,) depth in the medium
    interp_method: str

    @property
    def n(self) -> int:
        return len(self.lambda_nm)

    @property
    def taps(self) -> int:
        return self.sinc_idx.shape[1]


def sinc_band(k: np.ndarray, k_lin: np.ndarray, taps: int):
    """Banded sinc interpolation operator from samples at k onto k_lin.

    Normalised positions nq (targets) and n (sources) span [0, N-1]; output i
    takes every source j with |nq_i - n_j| < taps, weight sinc(nq_i - n_j)."""
    N = len(k)
    nq = (k_lin - k_lin.min()) / (k_lin.max() - k_lin.min()) * (N - 1)
    n = (k - k.min()) / (k.max() - k.min()) * (N - 1)
    if not (np.all(np.diff(n) > 0) or np.all(np.diff(n) < 0)):
        raise ValueError("source k positions must be strictly monotonic")
    desc = n[0] > n[-1]
    ns = n[::-1] if desc else n                     # ascending view
    # candidate window in the ascending view, widened by one on each side and
    # then filtered with the exact strict test on the reference's expression
    lo = np.searchsorted(ns, nq - taps, side="left") - 1
    hi = np.searchsorted(ns, nq + taps, side="right") + 1
    lo = np.clip(lo, 0, N)
    hi = np.clip(hi, 0, N)
    rows = []
    for i in range(N):
        js = np.arange(lo[i], hi[i])
        jj = (N - 1 - js) if desc else js           # original source indices
        dist = nq[i] - n[jj]
        keep = np.abs(dist) < taps
        jj, dist = jj[keep], dist[keep]
        order = np.argsort(jj)
        rows.append((jj[order], dist[order]))
    T = max(len(r[0]) for r in rows)
    idx = np.zeros((N, T), np.int64)
    w = np.zeros((N, T), float)
    start = np.zeros(N, np.int32)
    length = np.zeros(N, np.int32)
    for i, (jj, dist) in enumerate(rows):
        idx[i, : len(jj)] = jj
        w[i, : len(jj)] = np.sinc(dist)
        if len(jj):
            if np.any(np.diff(jj) != 1):
                raise ValueError("sinc band is not contiguous")
            start[i] = jj[0]
        length[i] = len(jj)
    return idx, w, start, length


def build_spectral_geometry(lambda_nm: np.ndarray, dispersion_quadratic_term: float, n_medium: float,
                            interp_method: str = "sinc5") -> SpectralGeometry:
    lam = np.asarray(lambda_nm, float).ravel()
    N = len(lam)
    k = 2 * np.pi / lam
    k_lin = linspace_matlab(k.max(), k.min(), N)
    m = interp_method.lower()
    if not m.startswith("sinc"):
        raise NotImplementedError(f"interp_method {interp_method!r}: only sincN is supported")
    idx, w, start, length = sinc_band(k, k_lin, int(m[4:]))

    lambda_eq = _pchip(k, lam, k_lin)
    k_eq = 2 * np.pi / lambda_eq
    hann = 0.5 * (1 - np.cos(2 * np.pi * np.arange(N) / (N - 1)))
    hann = hann / np.sqrt(np.mean(hann ** 2))
    window = hann * np.exp(1j * (-dispersion_quadratic_term * (k_eq - k_eq.mean()) ** 2))

    l0, l1 = np.sort([lambda_eq[0], lambda_eq[-1]])
    lambda0_um = 0.5 * (l0 + l1) / 1e3
    z_step = 0.5 * lambda0_um ** 2 / ((l1 - l0) / 1e3) / n_medium
    z_um = linspace_matlab(0.0, z_step * N / 2, N // 2)
    return SpectralGeometry(lam, k, k_lin, lambda_eq, idx, w, start, length, window, z_um, interp_method)


def dispersion_dk2(sg: SpectralGeometry) -> np.ndarray:
    """(k_eq - mean k_eq)^2 (float64), the per-sample factor of the dispersion phase."""
    k_eq = 2 * np.pi / sg.lambda_eq_nm
    return (k_eq - k_eq.mean()) ** 2


def hann_rms(n: int) -> np.ndarray:
    h = 0.5 * (1 - np.cos(2 * np.pi * np.arange(n) / (n - 1)))
    return h / np.sqrt(np.mean(h ** 2))
