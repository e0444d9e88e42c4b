"""Estimators on the GB300 kernels: dispersion scorer and search, focus helpers.

Dispersion (octrecon/estimation/dispersion.py): the scorer linearises and
Hann/rms-windows its B-scans once on the device (octgb_disp_load); every
candidate beta then costs one phase multiply, inverse FFT and |.| per A-scan
and a per-B-scan sharpness metric, all on the device (octgb_disp_eval), and a
whole list of betas (the coarse grid) runs in one launch.  `search_dispersion`
keeps the reference's search (dispersion.py:213-246: normalised coarse-grid
curves, refinement of their mean near the best grid point, per-B-scan optima
and their robust spread) but refines in rounds of candidates scored in one
launch each (`zoom_maximum`) where the reference calls scipy's sequential
bounded Brent.

Focus (octrecon/estimation/focus.py): the x-median depth profiles run on the
device (octgb_xmedian); the 1-D rules on a profile of ~1000 pixels
(imgaussfilt_1d, findpeaks_matlab, detect_peak_near, interface_pix) stay on the
host in float64, as MATLAB defines them.
"""
from __future__ import annotations

import numpy as np

from . import geometry as G
from ._lib import Context

Z_MIN_PIX = 20              # depth pixels ignored by the metrics (dispersion.py:40)
TOP_FRACTION = 0.01         # top_percentile (dispersion.py:41)
METRICS = ("top_percentile", "kurtosis", "entropy", "legacy_peak")
_METRIC_ID = {"top_percentile": 1, "kurtosis": 2, "entropy": 3, "legacy_peak": 4}


def hann_rms(n: int) -> np.ndarray:
    """MATLAB hann(n) (symmetric) scaled to unit rms (dispersion.py:76-77)."""
    h = 0.5 * (1 - np.cos(2 * np.pi * np.arange(n) / (n - 1)))
    return h / np.sqrt(np.mean(h ** 2))


class DispersionScorer:
    """GB300 form of DispersionScorer (octrecon/estimation/dispersion.py:66-107).

    raw_list: B-scans, each (rep, interf, N) raw counts (repeats of one y
    frame, as VolumeContext.read_raw returns them).  Same interface as the
    reference: window(beta), magnitude(beta, idx) -> (B or 1, nX, N/2) float32,
    scores(beta, idx) -> (B,) or (1,) float64, n_evals; plus scores_grid(betas)
    -> (len(betas), B), one launch for all betas.
    """

    def __init__(self, lambda_nm, raw_list, metric: str, apod_size: int, device: int = 0, rep: int | None = None,
                 raw_dtype=None):
        """raw_list: a list of host (rep, interf, N) arrays, or one array or CUDA
        tensor (B * rep, interf, N) with `rep` given (repeats consecutive)."""
        if metric not in METRICS:
            raise ValueError(f"unknown metric {metric!r}; choose from {METRICS}")
        self.metric = metric
        lam = np.asarray(lambda_nm, float)
        sg = G.build_spectral_geometry(lam, 0.0, 1.33)       # sinc band and k_eq do not depend on beta or n
        N = len(lam)
        self.n = N
        self.nz = N // 2
        if rep is None:
            raws = [np.asarray(r) for r in raw_list]
            if not raws:
                raise ValueError("no B-scans")
            rep = raws[0].shape[0]
            if any(r.shape != raws[0].shape or r.dtype != raws[0].dtype for r in raws):
                raise ValueError("all B-scans must have the same shape and dtype")
            raw = np.concatenate(raws, 0)
        else:
            raw = raw_list
            if raw.shape[0] % rep:
                raise ValueError("the B-scan count is not a multiple of rep")
        self.nrep = rep
        self.B = raw.shape[0] // rep
        interf = raw.shape[1]
        self.nx = interf - int(apod_size)
        k_eq = 2 * np.pi / sg.lambda_eq_nm
        self.dk2 = (k_eq - k_eq.mean()) ** 2                   # float64 (dispersion.py:78-79)
        self.ctx = Context(device)
        self.ctx.set_geometry(sg.sinc_idx, sg.sinc_w, np.ones(N, np.complex128))
        self.ctx.disp_load(raw, int(apod_size), self.B, rep, hann_rms(N), raw_dtype=raw_dtype)
        self.ctx.disp_set_dk2(self.dk2)
        self.top_k = max(1, int(self.nx * (self.nz - Z_MIN_PIX) * TOP_FRACTION))
        self.n_evals = 0

    @classmethod
    def from_context(cls, ctx, raw_list, metric: str, device: int = 0):
        """Build from the reference's VolumeContext (estimation/_common.py:38-118);
        rare formats are prepared on the device first (SpectralProcessor.prepare,
        core/spectral.py:112-116)."""
        h = ctx.hdr
        binning, frame_mean = max(1, int(h.spectra_avg)), h.apod_mode == "frame_mean"
        if binning == 1 and not frame_mean:
            return cls(ctx.lambda_nm, raw_list, metric, h.apod_size, device)
        prep = Context(device)
        try:
            raws = [prep.prepare_raw(np.asarray(r), h.apod_size, binning, 1 if frame_mean else 0,
                                     max(1, int(h.bscan_avg))) for r in raw_list]
        finally:
            prep.close()
        return cls(ctx.lambda_nm, raws, metric, 1 if frame_mean else h.apod_size, device)

    def close(self):
        self.ctx.close()

    def window(self, beta):
        return np.exp(-1j * float(beta) * self.dk2).astype(np.complex64)

    def _range(self, idx):
        return (0, self.B) if idx is None else (int(idx), 1)

    def magnitude(self, beta, idx=None) -> np.ndarray:
        b0, nb = self._range(idx)
        out = np.empty((1, nb, self.nx, self.nz), np.float32)
        self.ctx.disp_eval([beta], b0, nb, 0, mag=out)
        return out[0]

    def scores(self, beta, idx=None) -> np.ndarray:
        self.n_evals += 1
        b0, nb = self._range(idx)
        return self.ctx.disp_eval([beta], b0, nb, _METRIC_ID[self.metric], self.top_k, Z_MIN_PIX)[0]

    def scores_grid(self, betas, idx=None) -> np.ndarray:
        betas = np.asarray(betas, float)
        self.n_evals += len(betas)
        b0, nb = self._range(idx)
        return self.ctx.disp_eval(betas, b0, nb, _METRIC_ID[self.metric], self.top_k, Z_MIN_PIX)


def scores_batch(scorer, betas, idx=None) -> np.ndarray:
    """Scores of several betas, (len(betas), B) or (len(betas), 1): one
    launch on a scorer with `scores_grid`, one call per beta otherwise."""
    betas = np.asarray(betas, float)
    if hasattr(scorer, "scores_grid"):
        return np.asarray(scorer.scores_grid(betas, idx), float)
    return np.array([scorer.scores(b, idx) for b in betas], float)


def zoom_maximum(score, a: float, b: float, tol: float, points: int = 9):
    """Maximum of a score on [a, b]: every round scores `points` equispaced
    candidates at once (`score` takes an array of betas and returns their
    scores), and the next round's bracket is the best candidate's two
    neighbours, until candidates are at most `tol` apart.  The vertex of the
    parabola through the last best candidate and its neighbours is scored
    too and kept when it is better.  Returns (beta, score, rounds)."""
    lo0, hi0 = float(a), float(b)
    best_x, best_s, rounds = lo0, -np.inf, 0
    while True:
        xs = np.linspace(a, b, points)
        sc = np.asarray(score(xs), float)
        rounds += 1
        i = int(np.argmax(sc))
        if sc[i] > best_s:
            best_x, best_s = float(xs[i]), float(sc[i])
        h = (b - a) / (points - 1)
        if h <= tol or points < 3:
            break
        a, b = max(xs[i] - h, lo0), min(xs[i] + h, hi0)
    if 0 < i < points - 1:
        y0, y1, y2 = sc[i - 1], sc[i], sc[i + 1]
        curv = y0 - 2 * y1 + y2
        if curv < 0:
            v = float(xs[i] + 0.5 * h * (y0 - y2) / curv)
            sv = float(np.asarray(score(np.array([v])), float)[0])
            rounds += 1
            if sv > best_s:
                best_x, best_s = v, sv
    return best_x, best_s, rounds


def search_dispersion(scorer, lo: float, hi: float, initial: float, n_grid: int = 41, points: int = 9) -> dict:
    """The dispersion search of estimate_dispersion (dispersion.py:213-246:
    coarse grid, each B-scan's curve normalised to [0, 1] over the grid, the
    maximum of their mean near the best grid point, each B-scan's own
    optimum, the robust spread of those) with batched refinement: instead of
    a sequential bounded Brent, `zoom_maximum` scores `points` candidates per
    launch over the same bracket (the grid neighbours of the best point) and
    stops at the same tolerance, 2e-5 of the largest |bound|."""
    grid = np.linspace(lo, hi, int(n_grid))
    S = scores_batch(scorer, grid)                          # (n_grid, B)
    smin, span = S.min(axis=0), S.max(axis=0) - S.min(axis=0)
    span = np.where(span > 0, span, 1.0)
    curve = ((S - smin) / span).mean(axis=1)
    g = int(np.argmax(curve))
    tol = 2e-5 * max(abs(initial), abs(lo), abs(hi))

    def around(i):
        return grid[max(i - 1, 0)], grid[min(i + 1, len(grid) - 1)]

    def mean_score(xs):
        return ((scores_batch(scorer, xs) - smin) / span).mean(axis=1)

    x, sx, rounds = zoom_maximum(mean_score, *around(g), tol, points)
    value = x if sx >= curve[g] else float(grid[g])
    per = np.empty(S.shape[1])
    for j in range(S.shape[1]):
        i = int(np.argmax(S[:, j]))
        xj, sj, r = zoom_maximum(lambda xs, j=j: scores_batch(scorer, xs, j)[:, 0], *around(i), tol, points)
        per[j] = xj if sj >= S[i, j] else float(grid[i])
        rounds += r
    med = float(np.median(per))
    step = (hi - lo) / (n_grid - 1)
    return {"value": float(value), "candidates": grid, "score_curve": curve, "score_curves_per_bscan": ((S - smin) / span).T,
            "scores": S, "per_bscan_values": per, "median_per_bscan": med,
            "spread_mad": float(1.4826 * np.median(np.abs(per - med))),
            "at_bound": bool(value <= lo + step or value >= hi - step),
            "n_evaluations": int(getattr(scorer, "n_evals", 0)), "refine_rounds": rounds}


# --------------------------------------------------------------------------- focus helpers
def matlab_round(x):
    """MATLAB round(): halves away from zero."""
    x = np.asarray(x, float)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def imgaussfilt_1d(v, sigma: float = 4.0) -> np.ndarray:
    """MATLAB imgaussfilt on a vector (focus.py:44-52): Gaussian of
    2*ceil(2 sigma)+1 taps normalised to sum 1, replicate padding."""
    v = np.asarray(v, float).ravel()
    h = int(np.ceil(2 * sigma))
    taps = np.exp(-np.arange(-h, h + 1) ** 2 / (2 * sigma ** 2))
    taps = taps / taps.sum()
    padded = np.concatenate([np.repeat(v[:1], h), v, np.repeat(v[-1:], h)])
    return np.convolve(padded, taps, mode="valid")


def findpeaks_matlab(v) -> np.ndarray:
    """0-based indices of MATLAB findpeaks maxima (focus.py:55-72): larger than
    the left neighbour, a plateau reported at its first sample when the sample
    after it is smaller, end points never."""
    v = np.asarray(v, float)
    n = len(v)
    out = []
    i = 1
    while i < n - 1:
        if not v[i] > v[i - 1]:
            i += 1
            continue
        j = i
        while j + 1 < n - 1 and v[j + 1] == v[i]:
            j += 1
        if v[j + 1] < v[i]:                  # j <= n - 2 here
            out.append(i)
        i = j + 1
    return np.asarray(out, int)


def detect_peak_near(profile, guess_pix, search_px: int = 60, baseline_sigma: float = 30.0,
                     smooth_sigma: float = 4.0):
    """Confocal peak of a depth profile near a 1-based guess (focus.py:191-206):
    10 log10 with gaps interpolated, minus a sigma-30 baseline after sigma-4
    smoothing, the strongest MATLAB peak within +-search_px.  -> (pix or nan,
    prominence dB)."""
    prof = np.asarray(profile, float)
    lp = np.full(prof.shape, np.nan)
    ok = np.isfinite(prof) & (prof > 0)
    lp[ok] = 10 * np.log10(prof[ok])
    if ok.sum() < 10:
        return np.nan, 0.0
    lp = np.interp(np.arange(len(lp)), np.nonzero(ok)[0], lp[ok])
    detr = imgaussfilt_1d(lp, smooth_sigma) - imgaussfilt_1d(lp, baseline_sigma)
    p = findpeaks_matlab(detr) + 1
    p = p[np.abs(p - guess_pix) <= search_px]
    if p.size == 0:
        return np.nan, 0.0
    best = p[np.argmax(detr[p - 1])]
    return int(best), float(detr[best - 1])


def interface_pix_from_medians(medians):
    """Step-1 rule (focus.py:209-218) on per-frame x-median profiles
    (frames, nZ): the first maximum below the top third, 1-based, then the
    rounded median over frames."""
    med = np.array(medians, float, copy=True)
    nz = med.shape[-1]
    med[:, : int(matlab_round(nz / 3))] = np.nan
    vals = [int(np.nanargmax(m)) + 1 for m in med]
    return int(matlab_round(np.median(vals))), vals


def interface_pix(ctx: Context, mag_opc):
    """interface_pix (focus.py:209-218) with the x-medians on the device."""
    return interface_pix_from_medians(ctx.xmedian(mag_opc, ignore_nan=True))


def depth_profile(ctx: Context, mag, ignore_nan: bool = True) -> np.ndarray:
    """mean over frames of the x-median depth profiles (focus.py:156,255)."""
    med = ctx.xmedian(mag, ignore_nan=ignore_nan)
    with np.errstate(all="ignore"):
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", RuntimeWarning)
            return np.nanmean(med, axis=0) if ignore_nan else med.mean(axis=0)
