"""Generate the estimator fixtures of tests/golden/ by running the reference.

    python tests/golden/make_golden_estimation.py /path/to/reference

Runs where the reference octrecon source tree is importable (read-only), with
the same stand-ins as make_golden.py (empty `tifffile` module, NumPy path
instead of Numba).  Outputs (committed, small):

  scorer_case.npz       the reference DispersionScorer (estimation/dispersion.py:
                        66-107) on raw B-scans of the package's seeded spectrum
                        model with dispersion (beta_px = 1e-5; the raw B-scans
                        are regenerated from their seeds by the tests): scores of every
                        metric over a beta grid, for single B-scans (rep 1) and
                        for B-scans with two repeats, and the magnitudes of
                        one B-scan at one beta.
  estimation_volume.tar.xz
                        a small Ganymede scan written by the reference's own
                        generator (scripts/make_synthetic_volume.py: 1 x 1
                        tiles x depths 0, 50, 100 um, 32 A-scans, 5 frames).
  estimation_case.npz   estimate_dispersion (bounds -5e7..5e7, 4 B-scans) and
                        detect_focus (mode auto) of the reference on that
                        volume, device "cpu", as JSON text, plus the
                        inputs/outputs of its 1-D focus helpers on the
                        measured depth profiles.
"""
from __future__ import annotations

import json
import sys
import tarfile
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]


class _Hdr:
    def __init__(self, rep):
        self.bscan_avg = rep


class _ArrayContext:
    """The part of VolumeContext (estimation/_common.py:38-118) that
    DispersionScorer uses, over raw arrays instead of a volume."""

    def __init__(self, lambda_nm, apod, rep):
        from octrecon.core.geometry import build_spectral_geometry
        from octrecon.core.spectral import SpectralProcessor
        self.xp = np
        self.hdr = _Hdr(rep)
        self._sg = lambda b: build_spectral_geometry(lambda_nm, b, 1.33, "sinc5")
        self._sp = lambda b: SpectralProcessor(self._sg(b), apod, xp=np, dtype=np.float32, use_numba=False)

    def geometry(self, dispersion, n_medium=None):
        return self._sg(dispersion)

    def processor(self, dispersion, n_medium=None):
        return self._sp(dispersion)


def main(ref_root: str):
    ref_root = Path(ref_root)
    sys.modules.setdefault("tifffile", types.ModuleType("tifffile"))
    sys.path.insert(0, str(ref_root))
    sys.path.insert(0, str(ref_root / "scripts"))
    sys.path.insert(0, str(REPO))
    import octrecon.core.spectral as ref_spectral
    from make_synthetic_volume import make_volume
    from octrecon.estimation import dispersion as D
    from octrecon.estimation import focus as F
    from octrecon.estimation.dispersion import estimate_dispersion
    from octrecon.estimation.focus import detect_focus

    from oct_recon_af_v1_gb300 import synthetic

    lam = synthetic.lambda_nm()
    beta0 = synthetic.beta_ref_from_px(1e-5)
    betas = np.linspace(0.0, 2.0 * beta0, 9)
    out = {"lambda_nm": lam, "betas": betas, "apod_size": np.int64(25)}
    raw1 = synthetic.generate_numpy(3, 96, 25, seed=11)                 # 3 B-scans, rep 1
    raw2 = synthetic.generate_numpy(4, 64, 25, seed=12)                 # 2 B-scans x 2 repeats
    for tag, raw, rep in (("r1", raw1, 1), ("r2", raw2, 2)):
        ctx = _ArrayContext(lam, 25, rep)
        raws = [raw[i:i + rep] for i in range(0, raw.shape[0], rep)]
        out[f"rep_{tag}"] = np.int64(rep)
        for metric in D.METRICS:
            sc = D.DispersionScorer(ctx, raws, metric)
            out[f"scores_{tag}_{metric}"] = np.array([sc.scores(b) for b in betas])
            out[f"scores_{tag}_{metric}_idx1"] = np.array([sc.scores(b, 1) for b in betas[::4]])
        out[f"mag_{tag}"] = np.asarray(D.DispersionScorer(ctx, raws, "top_percentile").magnitude(beta0, 0))
    np.savez_compressed(HERE / "scorer_case.npz", **out)

    # ------------------------------------------------------------------ volume-level runs
    work = Path(tempfile.mkdtemp(prefix="octgb_est_"))
    vol = work / "estimation"
    make_volume(vol, nx=32, ny=5, tiles_x=1, tiles_y=1, depths=(0.0, 0.05, 0.1), n_lambda=2048, seed=5,
                system="gan632")
    orig_init = ref_spectral.SpectralProcessor.__init__

    def numpy_init(self, *a, **kw):
        kw["use_numba"] = False
        orig_init(self, *a, **kw)

    ref_spectral.SpectralProcessor.__init__ = numpy_init
    try:
        est = estimate_dispersion(str(vol), device="cpu", bounds=(-5e7, 5e7), n_bscans=4, log=None)
        foc = detect_focus(str(vol), device="cpu", log=None)
    finally:
        ref_spectral.SpectralProcessor.__init__ = orig_init
    # the reference's 1-D focus helpers on the measured profiles
    profiles = [np.asarray(m["profile"], float) for m in foc["drift"]["measurements"]]
    helper = {}
    for i, p in enumerate(profiles):
        helper[f"prof{i}"] = p
        helper[f"prof{i}_gauss4"] = F.imgaussfilt_1d(p, 4)
        helper[f"prof{i}_gauss30"] = F.imgaussfilt_1d(p, 30)
        lp = 10 * np.log10(np.where(p > 0, p, np.nan))
        helper[f"prof{i}_peaks"] = F.findpeaks_matlab(np.nan_to_num(lp, nan=-300.0))
        pix, prom = F.detect_peak_near(p, 300, 60)
        helper[f"prof{i}_near300"] = np.array([np.nan if not np.isfinite(pix) else pix, prom])
    rng = np.random.default_rng(3)
    mags = rng.gamma(2.0, 1.0, size=(3, 31, 200))
    mags[0, :5, 190:] = np.nan                                         # nanmedian columns
    helper["iface_mags"] = mags
    helper["iface_out"] = np.array(F.interface_pix(mags)[0])
    plateau = np.array([0, 1, 3, 3, 3, 2, 5, 5, 1, 4, 4, 4, 4, 0, 2, 2, 2, 2, 9, 9], float)
    helper["plateau"] = plateau
    helper["plateau_peaks"] = F.findpeaks_matlab(plateau)
    with tarfile.open(HERE / "estimation_volume.tar.xz", "w:xz") as tf:
        tf.add(vol, arcname="estimation")
    np.savez_compressed(HERE / "estimation_case.npz", estimate_json=np.array(json.dumps(est)),
                        focus_json=np.array(json.dumps(foc)), **helper)
    print("wrote", HERE / "scorer_case.npz", HERE / "estimation_case.npz", HERE / "estimation_volume.tar.xz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <path of the octrecon source tree>")
    main(sys.argv[1])
