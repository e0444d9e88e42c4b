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


@pytest.fixture(scope="module")
def srr():
    return dict(np.load(GOLDEN / "srr_case.npz"))


def test_srr_decode_kernel_bit_exact(ctx, srr):
    """The device decode of the reference's SRR files equals its reader's
    read_bscans, from host words and from device words; ragged widths (the
    scalar path) and other line ranges against the oracle."""
    import torch
    a0, a1, s0, s1 = (int(v) for v in srr["ranges"])
    words = srr["words"]
    np.testing.assert_array_equal(ctx.srr_decode(words, (a0, a1), (s0, s1)), srr["decoded"])
    wd = torch.from_numpy(words.view(np.int16)).cuda()
    out = torch.empty(srr["decoded"].shape, dtype=torch.int16, device="cuda")
    ctx.srr_decode(wd, (a0, a1), (s0, s1), out=out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), srr["decoded"])
    rng = np.random.default_rng(14)
    for n, lines, ar, sr in ((37, 11, (2, 5), (6, 11)), (2048, 40, (30, 40), (0, 25)), (8, 3, (0, 1), (0, 3))):
        w = rng.integers(0, 65536, size=(3, lines, n)).astype(np.uint16)
        ref = O.srr_decode(w, ar, sr)
        np.testing.assert_array_equal(ctx.srr_decode(w, ar, sr), ref)
        o = torch.empty(ref.shape, dtype=torch.int16, device="cuda")
        ctx.srr_decode(torch.from_numpy(w.view(np.int16)).cuda(), ar, sr, out=o)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(o.cpu().numpy(), ref)
    assert ctx.srr_decode(np.zeros((0, 5, 8), np.uint16), (0, 1), (1, 5)).shape == (0, 5, 8)
    from oct_recon_af_v1_gb300._lib import OctgbError
    with pytest.raises(OctgbError):
        ctx.srr_decode(words, (0, 0), (s0, s1))
    with pytest.raises(OctgbError):
        ctx.srr_decode(words, (a0, a1), (s0, words.shape[1] + 1))


def test_reconstructor_srr_decodes_on_device(srr, tmp_path):
    """The reference's Reconstructor on device "gb300" reading a Thorlabs SRR
    scan (B-scan repeats 2): the files' words go to the device undecoded, and
    the plane matches the reference's."""
    import_octrecon()
    from octrecon.pipeline import ReconConfig, Reconstructor

    from oct_recon_af_v1_gb300 import plugin
    plugin.register()
    with tarfile.open(GOLDEN / "srr_volume.tar.xz") as tf:
        tf.extractall(tmp_path, filter="data")
    cfg = ReconConfig(volume_folder=str(tmp_path / "srr"), device="gb300", precision="float32",
                      dispersion_quadratic_term=8.949e7, focus_positions=200.0, focus_sigma=10, crop_z_range_mm="none",
                      output_pixel_size_um=2, interp_method="sinc5", batch_frames=2, io_threads=1, write_tiff=False)
    R = Reconstructor(cfg, log=lambda *a: None)
    calls = []
    orig = R._gb300.ctx.srr_decode
    R._gb300.ctx.srr_decode = lambda *a, **k: calls.append(1) or orig(*a, **k)
    p = R.process_planes([1])[0].astype(float)
    assert calls, "the SRR words were not decoded on the device"
    ref32 = srr["plane_float32"].astype(float)
    ref64 = srr["plane_float64"].astype(float)
    assert np.array_equal(np.isfinite(p), np.isfinite(ref32))
    fin = np.isfinite(p) & np.isfinite(ref64)
    err, err_ref = np.abs(p - ref64)[fin].max(), np.abs(ref32 - ref64)[fin].max()
    assert err <= 1.5 * err_ref + 1e-4, (err, err_ref)


def test_spectral_processor_prepares_rare_formats(ctx):
    """The package's SpectralProcessor built with AScanBinning or the
    frame-mean apodisation: its magnitudes equal the magnitudes of the oracle's
    prepare_raw (the prepare kernel is bit-exact), for host and device input."""
    import torch

    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import synthetic
    from oct_recon_af_v1_gb300.spectral import SpectralProcessor
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), 0.0, 1.33)
    rng = np.random.default_rng(15)
    raw = rng.integers(0, 4096, size=(4, 25 + 30, 2048)).astype(np.uint16)
    for binning, mode, group in ((2, "lines", 1), (3, "frame_mean", 2), (1, "frame_mean", 1)):
        sp = SpectralProcessor(sg, 25, ctx=ctx, ascan_binning=binning, apod_mode=mode, apod_group=group)
        prep = O.prepare_raw(raw, 25, binning, mode, group)
        a = 1 if mode == "frame_mean" else 25
        ref = ctx.magnitude(prep, a)
        np.testing.assert_array_equal(sp.magnitude(raw), ref)
        dev = sp.magnitude(torch.from_numpy(raw.view(np.int16)).cuda())
        torch.cuda.synchronize()
        np.testing.assert_array_equal(dev.cpu().numpy(), ref)
