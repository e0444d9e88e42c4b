"""Rare raw formats on the GPU: the prepare and repeat-averaging kernels bit
for bit against the oracle (pinned to the reference in test_formats_host.py),
and the reference's own Reconstructor on device "gb300" on a binned,
B-/A-scan-repeated Thorlabs scan and a Wasatch frame-mean scan, against the
reference's planes (tests/golden/formats_case.npz)."""
from __future__ import annotations

import tarfile
from pathlib import Path

import numpy as np
import pytest

from oracle import numerics as O
from octrecon_ref import import_octrecon

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def fmt():
    return dict(np.load(GOLDEN / "formats_case.npz"))


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oct_recon_af_v1_gb300 as pkg
    pkg.build()
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import synthetic
    from oct_recon_af_v1_gb300._lib import Context
    c = Context(0)
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), 0.0, 1.33)
    c.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    yield c
    c.close()


def test_prepare_kernel_bit_exact(ctx, fmt):
    for name in ("combo", "wasatch"):
        apod, binning, nb, na, size_x, frame_mean = (int(v) for v in fmt[f"{name}_hdr"])
        raw = fmt[f"{name}_raw"]
        got = ctx.prepare_raw(raw, apod, binning, frame_mean, nb)
        np.testing.assert_array_equal(got, fmt[f"{name}_prepared"])
    rng = np.random.default_rng(12)
    raw = rng.integers(0, 4096, size=(6, 25 + 37, 2048)).astype(np.uint16)
    for binning in (2, 3, 4, 5):
        for mode, group in ((0, 1), (1, 3), (1, 1)):
            ref = O.prepare_raw(raw, 25, binning, "frame_mean" if mode else "lines", group)
            got = ctx.prepare_raw(raw, 25, binning, mode, group)
            np.testing.assert_array_equal(got, ref)


def test_repeat_kernel_bit_exact(ctx, fmt):
    np.testing.assert_array_equal(ctx.average_repeats(fmt["rep_mag"], 3, 2, 3), fmt["rep_out"])
    rng = np.random.default_rng(13)
    for nb, na in ((1, 2), (3, 1), (2, 2)):
        mag = rng.gamma(2.0, 1.0, size=(4 * nb, 7 * na, 1024)).astype(np.float32)
        np.testing.assert_array_equal(ctx.average_repeats(mag, 4, nb, na), O.average_repeats(mag, 4, nb, 7, na))


@pytest.mark.parametrize("name", ["combo", "wasatch"])
def test_reconstructor_rare_formats_match_reference(fmt, name, tmp_path):
    import_octrecon()
    from octrecon.pipeline import ReconConfig, Reconstructor

    from oct_recon_af_v1_gb300 import plugin
    plugin.register()
    with tarfile.open(GOLDEN / "formats_volumes.tar.xz") as tf:
        tf.extractall(tmp_path, filter="data")
    cfg = ReconConfig(volume_folder=str(tmp_path / name), device="gb300", precision="float32",
                      dispersion_quadratic_term=8.949e7, focus_positions=200.0, focus_sigma=10, crop_z_range_mm="none",
                      output_pixel_size_um=2, interp_method="sinc5", batch_frames=2, io_threads=1, write_tiff=False)
    R = Reconstructor(cfg, log=lambda *a: None)
    assert R._gb300.rare
    p = R.process_planes([1])[0].astype(float)
    ref32 = fmt[f"{name}_plane_float32"].astype(float)
    ref64 = fmt[f"{name}_plane_float64"].astype(float)
    assert np.array_equal(np.isfinite(p), np.isfinite(ref32))
    fin = np.isfinite(p) & np.isfinite(ref64)
    err, err_ref = np.abs(p - ref64)[fin].max(), np.abs(ref32 - ref64)[fin].max()
    assert err <= 1.5 * err_ref + 1e-4, (err, err_ref)
