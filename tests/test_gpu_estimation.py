"""Estimators on the GPU: the GB300 DispersionScorer against the reference's
scores (tests/golden/scorer_case.npz), its exact top-k selection (ties
included) against the oracle metric on the same magnitudes, the x-median and
x-mean kernels against numpy.median / nanmedian / nanmean, and octrecon's estimate_dispersion /
detect_focus on device "gb300" against the reference's own results on the
same volume (tests/golden/estimation_case.npz)."""
from __future__ import annotations

import json
import tarfile
from pathlib import Path

import numpy as np
import pytest

from oracle import numerics as O
from test_estimation_host import scorer_raws

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
METRICS = ("top_percentile", "kurtosis", "entropy", "legacy_peak")
# float32 spectra of two different FFTs: scores agree to ~1e-6 of their scale
ATOL = {"top_percentile": 2e-5, "legacy_peak": 2e-5, "entropy": 2e-5}
RTOL_KURT = 2e-5


@pytest.fixture(scope="module")
def built():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oct_recon_af_v1_gb300 as pkg
    pkg.build()
    return torch


@pytest.mark.parametrize("tag", ["r1", "r2"])
def test_scorer_matches_reference(built, tag):
    from oct_recon_af_v1_gb300.estimation import DispersionScorer
    case = dict(np.load(GOLDEN / "scorer_case.npz"))
    raws, rep = scorer_raws(tag)
    betas = case["betas"]
    for metric in METRICS:
        sc = DispersionScorer(case["lambda_nm"], raws, metric, 25)
        try:
            ref = case[f"scores_{tag}_{metric}"]
            got = np.array([sc.scores(b) for b in betas])
            grid = sc.scores_grid(betas)
            np.testing.assert_array_equal(grid, got)                  # one launch == one beta at a time
            got1 = np.array([sc.scores(b, 1) for b in betas[::4]])
            if metric == "kurtosis":
                np.testing.assert_allclose(got, ref, rtol=RTOL_KURT, atol=0)
                np.testing.assert_allclose(got1, case[f"scores_{tag}_{metric}_idx1"], rtol=RTOL_KURT, atol=0)
            else:
                np.testing.assert_allclose(got, ref, rtol=0, atol=ATOL[metric])
                np.testing.assert_allclose(got1, case[f"scores_{tag}_{metric}_idx1"], rtol=0, atol=ATOL[metric])
            # the curves peak at the same beta
            assert np.array_equal(np.argmax(got, 0), np.argmax(ref, 0))
            assert sc.n_evals == 2 * len(betas) + len(betas[::4])
        finally:
            sc.close()
    sc = DispersionScorer(case["lambda_nm"], raws, "top_percentile", 25)
    try:
        m = sc.magnitude(betas[len(betas) // 2], 0)
        ref = case[f"mag_{tag}"]
        assert m.shape == ref.shape
        assert np.abs(m - ref).max() / ref.max() < 1e-5
    finally:
        sc.close()


def test_scorer_metric_exact_on_its_magnitudes(built):
    """Radix select + float64 sums against the oracle metric on the very same
    magnitudes; the second case has every A-scan of a B-scan identical, so the
    top-k threshold value occurs 64 times (ties)."""
    from oct_recon_af_v1_gb300 import synthetic
    from oct_recon_af_v1_gb300.estimation import DispersionScorer
    lam = synthetic.lambda_nm()
    raw = synthetic.generate_numpy(2, 64, 25, seed=5)
    tie = raw.copy()
    tie[:, 25:, :] = tie[:, 25:26, :]                                   # identical A-scans
    for r in (raw, tie):
        for metric in METRICS:
            sc = DispersionScorer(lam, [r[0:1], r[1:2]], metric, 25)
            try:
                for beta in (0.0, 7.3e6, -2.1e7):
                    A = sc.magnitude(beta)
                    # float64 sums in another order; legacy_peak also float32 logf vs numpy's log
                    rtol = 1e-6 if metric == "legacy_peak" else 1e-11
                    np.testing.assert_allclose(sc.scores(beta), O.disp_metric(A, metric), rtol=rtol, atol=0)
            finally:
                sc.close()


def test_xmedian_matches_numpy(built):
    from oct_recon_af_v1_gb300._lib import Context
    rng = np.random.default_rng(9)
    ctx = Context(0)
    try:
        for F, nx, nz in ((5, 500, 1024), (3, 31, 200), (2, 1, 17), (1, 1000, 64)):
            m = rng.gamma(2.0, 1.0, size=(F, nx, nz)).astype(np.float32)
            m[0, : max(1, nx // 3), : nz // 4] = np.nan
            m[-1, :, nz - 1] = np.nan                                   # an all-NaN column
            import warnings
            with warnings.catch_warnings():
                warnings.simplefilter("ignore", RuntimeWarning)
                ref_nan = np.nanmedian(m.astype(float), axis=1)
            ref = np.median(m.astype(float), axis=1)
            np.testing.assert_array_equal(ctx.xmedian(m, ignore_nan=True), ref_nan)
            np.testing.assert_array_equal(ctx.xmedian(m, ignore_nan=False), ref)
            dev = built.from_numpy(m).cuda()
            np.testing.assert_array_equal(ctx.xmedian(dev, ignore_nan=True), ref_nan)
            with warnings.catch_warnings():
                warnings.simplefilter("ignore", RuntimeWarning)
                ref_mean = np.nanmean(m.astype(float), axis=1)
            np.testing.assert_allclose(ctx.xmean(dev), ref_mean, rtol=1e-13, atol=0)
    finally:
        ctx.close()


@pytest.fixture(scope="module")
def volume(tmp_path_factory):
    d = tmp_path_factory.mktemp("estvol")
    with tarfile.open(GOLDEN / "estimation_volume.tar.xz") as tf:
        tf.extractall(d, filter="data")
    case = np.load(GOLDEN / "estimation_case.npz")
    return d / "estimation", json.loads(str(case["estimate_json"])), json.loads(str(case["focus_json"]))


def test_plugin_estimate_dispersion_matches_reference(built, volume):
    from octrecon_ref import import_octrecon
    import_octrecon()
    from oct_recon_af_v1_gb300 import plugin
    plugin.register()
    from octrecon.estimation.dispersion import estimate_dispersion
    vol, ref, _ = volume
    est = estimate_dispersion(str(vol), device="gb300", bounds=ref["bounds"], n_bscans=4, log=None)
    assert est["device"] == "gb300"
    assert [(u["folder"], u["frame"]) for u in est["tiles_used"]] == \
        [(u["folder"], u["frame"]) for u in ref["tiles_used"]]
    np.testing.assert_allclose(est["score_curve"], ref["score_curve"], rtol=0, atol=1e-4)
    # The optima sit where the score curves are flat: near the top a curve is
    # S(b) ~ S* - c (b - b*)^2 with c ~ 1e-16 per unit^2 for these 32-A-scan
    # B-scans, so score differences of ~1e-6 (two float32 FFTs) move a bounded
    # Brent optimum by up to sqrt(1e-6 / c) ~ 1e5.  Bound: 1 % of the grid step.
    step = (ref["bounds"][1] - ref["bounds"][0]) / (len(ref["candidates"]) - 1)
    assert abs(est["value"] - ref["value"]) <= 0.01 * step
    np.testing.assert_allclose(est["per_bscan_values"], ref["per_bscan_values"], rtol=0, atol=0.01 * step)
    assert est["at_bound"] == ref["at_bound"]


def test_plugin_detect_focus_matches_reference(built, volume):
    from octrecon_ref import import_octrecon
    import_octrecon()
    from oct_recon_af_v1_gb300 import plugin
    plugin.register()
    from octrecon.estimation.focus import detect_focus
    vol, _, ref = volume
    foc = detect_focus(str(vol), device="gb300", log=None)
    assert foc["device"] == "gb300"
    assert foc["focus_positions"] == ref["focus_positions"]
    assert foc["step1"] == ref["step1"] and foc["step2"] == ref["step2"]
    assert foc["confocal_peak"]["value"] == ref["confocal_peak"]["value"]
    got = [m["detected_pix"] for m in foc["drift"]["measurements"]]
    assert got == [m["detected_pix"] for m in ref["drift"]["measurements"]]
    for m, r in zip(foc["drift"]["measurements"], ref["drift"]["measurements"]):
        p, q = np.asarray(m["profile"], float), np.asarray(r["profile"], float)
        assert np.nanmax(np.abs(p - q) / np.nanmax(np.abs(q))) < 1e-5


def test_windowed_lines_bit_exact(built):
    """The scorer's windowed lines equal float32(float64(linearised line) *
    hann) bit for bit (dispersion.py:84): the kernel's float32 form of the
    float64 product, with its float64 fallback near rounding boundaries, on
    lines whose samples span many binades (so both paths are exercised)."""
    from oct_recon_af_v1_gb300 import estimation as E
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import synthetic as S
    from oct_recon_af_v1_gb300._lib import Context
    lam = S.lambda_nm()
    sg = G.build_spectral_geometry(lam, 0.0, 1.33)
    ctx = Context(0)
    try:
        ctx.set_geometry(sg.sinc_idx, sg.sinc_w, np.ones(len(lam), np.complex128))
        rng = np.random.default_rng(17)
        raw = (rng.integers(0, 60000, size=(6, 25 + 40, 2048)) >> rng.integers(0, 14, size=(6, 65, 1))).astype(np.uint16)
        hann = E.hann_rms(len(lam))
        ctx.disp_load(raw, 25, 6, 1, hann, raw_dtype=0)
        got = ctx.disp_lines()
        lin = ctx.fused_pre_fft(raw, 25, raw_dtype=0)          # window of ones: the linearised line
        ref = (lin.real.astype(np.float64) * hann).astype(np.float32)
        assert got.dtype == np.float32 and got.shape == ref.shape
        np.testing.assert_array_equal(got.view(np.int32), ref.view(np.int32))
    finally:
        ctx.close()
