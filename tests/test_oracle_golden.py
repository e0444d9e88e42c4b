"""The oracle against the reference's golden vectors (CPU only).

Pins the CPU restatement before it is trusted as the checker:
  * its geometry equals the reference geometry stored in the fixtures;
  * its NumPy float32/float64 spectral paths equal the reference
    SpectralProcessor outputs (tests/golden/spectral_case.npz);
  * its Numba-kernel restatement (C) agrees with the reference float32 path;
  * its stitching + finalise reproduce the reference plane of the telesto
    format-test case and the unmodified-MATLAB golden plane within the
    reference's own tolerance (tests/test_formats.py:171-180).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import numerics as O


def test_geometry_matches_reference(spectral_case, telesto):
    for case in (spectral_case, telesto):
        g = O.spectral_geometry(case["lambda_nm"], float(case["dispersion"]), float(case["n_medium"]))
        np.testing.assert_array_equal(g.sinc_idx, case["sinc_idx"])
        np.testing.assert_array_equal(g.sinc_w, case["sinc_w"])
        np.testing.assert_allclose(g.window, case["window"], rtol=0, atol=1e-14)


def test_numpy_paths_match_reference(spectral_case):
    c = spectral_case
    g = O.spectral_geometry(c["lambda_nm"], float(c["dispersion"]), float(c["n_medium"]))
    m64 = O.magnitude_numpy(c["raw"], g, int(c["apod_size"]), np.float64)
    m32 = O.magnitude_numpy(c["raw"], g, int(c["apod_size"]), np.float32)
    np.testing.assert_allclose(m64, c["mag_fp64"], rtol=1e-12, atol=1e-12)
    # pocketfft float32 may vectorise differently across machines: a few ulps
    np.testing.assert_allclose(m32, c["mag_fp32"], rtol=1e-5, atol=1e-4)


def test_numba_restatement_close_to_reference_fp32(spectral_case):
    c = spectral_case
    g = O.spectral_geometry(c["lambda_nm"], float(c["dispersion"]), float(c["n_medium"]))
    mn = O.magnitude_numba(c["raw"], g, int(c["apod_size"]))
    ref = c["mag_fp32"].astype(np.float64)
    # both keep the float32 apodisation mean; they differ by float32 rounding only
    rel = np.abs(mn - ref) / (np.abs(ref).max())
    assert rel.max() < 1e-5
    db_n, db_r = 20 * np.log10(mn[..., 20:1000]), 20 * np.log10(ref[..., 20:1000])
    assert np.abs(db_n - db_r).max() < 0.05


def _scan(t):
    return O.ScanDesc(t["x_centers_mm"], t["y_centers_mm"], t["z_depths_mm"], int(t["n_x_px"]), int(t["n_y_px"]),
                      float(t["tile_range_x_mm"]), float(t["tile_range_y_mm"]), float(t["x_offset"]),
                      float(t["y_offset"]))


def _oracle_stitchers(t, g, dtype):
    tg = O.tiled_geometry(_scan(t), g.z_um, t["focus_pix"], float(t["output_pixel_size_um"]))
    st = {}
    for xi, zi in zip(t["tile_xi"], t["tile_zi"]):
        st[(int(xi), int(zi))] = O.Stitcher(tg, t["x_centers_mm"][xi], t["z_depths_mm"][zi], t["focus_pix"][zi],
                                            float(t["focus_sigma"]), dtype)
    return tg, st


def _oracle_plane(t, dtype):
    """Reference process_row restated: oracle magnitudes, oracle stitchers in
    `dtype`, optical-path gather, finalise."""
    g = O.spectral_geometry(t["lambda_nm"], float(t["dispersion"]), float(t["n_medium"]))
    tg, sts = _oracle_stitchers(t, g, dtype)
    apod = int(t["apod_size"])
    n_out_z, n_out_x = len(tg.out_z_mm), len(tg.out_x_mm)
    y = int(t["plane_y"])
    num = np.zeros((1, n_out_z, n_out_x), dtype)
    den = np.zeros((1, n_out_z, n_out_x), dtype)
    shift, pdz = t["opc_shift"], t["opc_pdz"]
    for k, (xi, zi) in enumerate(zip(t["tile_xi"], t["tile_zi"])):
        s = sts[(int(xi), int(zi))]
        raw = t["raw"][k][y:y + 1]
        mag = O.magnitude_numpy(raw, g, apod, np.float64) if dtype == np.float64 else O.magnitude_numba(raw, g, apod)
        rr = np.arange(s.r0, s.r1)
        src = np.clip(rr + shift[[y]][..., None], 0, mag.shape[-1] - 1)
        tt = rr + pdz[[y]][..., None]
        valid = (tt >= 0) & (tt <= mag.shape[-1] - 1)
        a = np.take_along_axis(mag, src, axis=-1)
        f = (valid * s.fz).astype(dtype)
        a = (a * f).astype(dtype)
        num[:, :, s.c0:s.c1] += np.matmul(np.matmul(a, s.Wz.T).transpose(0, 2, 1), s.WxT)
        den[:, :, s.c0:s.c1] += np.matmul(np.matmul(f, s.Wz.T).transpose(0, 2, 1), s.WxT)
    return O.finalise(num, den, dtype)[0]


def test_oracle_operators_match_reference(telesto):
    t = telesto
    g = O.spectral_geometry(t["lambda_nm"], float(t["dispersion"]), float(t["n_medium"]))
    tg, sts = _oracle_stitchers(t, g, np.float32)
    np.testing.assert_array_equal(tg.out_z_mm, t["out_z_mm"])
    np.testing.assert_array_equal(tg.out_x_mm, t["out_x_mm"])
    for (xi, zi), s in sts.items():
        key = f"st_{xi}_{zi}"
        assert [s.r0, s.r1, s.c0, s.c1] == list(t[key + "_rc"])
        np.testing.assert_array_equal(s.Wz, t[key + "_Wz"])
        np.testing.assert_array_equal(s.WxT, t[key + "_WxT"])
        np.testing.assert_array_equal(s.fz, t[key + "_fz"])


def test_oracle_pipeline_matches_reference_and_matlab(telesto):
    t = telesto
    p64 = _oracle_plane(t, np.float64).astype(float)
    ref64 = t["plane_fp64"].astype(float)
    fin = np.isfinite(p64) & np.isfinite(ref64)
    assert np.array_equal(np.isfinite(p64), np.isfinite(ref64))
    assert np.abs(p64 - ref64)[fin].max() < 1e-5
    m = t["matlab_plane"].astype(float)
    fin = np.isfinite(p64) & np.isfinite(m)
    assert np.abs(p64 - m)[fin].max() < 1e-4                 # tests/test_formats.py:173
    mism = np.isfinite(p64) != np.isfinite(m)
    assert not np.any(mism & ~t["matlab_tie"])

    p32 = _oracle_plane(t, np.float32).astype(float)
    ref32 = t["plane_fp32"].astype(float)
    assert np.array_equal(np.isfinite(p32), np.isfinite(ref32))
    fin = np.isfinite(p32) & np.isfinite(m)
    err_oracle = np.abs(p32 - m)[fin].max()
    err_ref = np.abs(ref32 - m)[fin].max()
    assert err_oracle <= 1.5 * err_ref + 1e-4, (err_oracle, err_ref)


def test_quantisation_semantics():
    db = np.array([np.nan, -10.0, 0.0, 5.0, 10.0, 10.0 + 1e-9, -10.0 - 1e-9, 2.5], np.float64)
    bits = O.db_to_bits(db, (10.0, -10.0))
    assert bits[0] == 0                       # NaN -> 0
    assert bits[1] == 1 and bits[6] == 1      # at / below c1 -> 1
    assert bits[4] == 65535 and bits[5] == 65535
    assert bits[2] == 32768                   # 32767 + 1
    # round half away from zero: (2.5 + 10)/20 * 65534 = 40958.75 -> 40959 + 1
    assert bits[7] == 40960
    back = O.bits_to_db(bits, (-10.0, 10.0))
    assert np.isnan(back[0]) and abs(back[4] - 10.0) < 1e-12
    assert O.plane_clim(np.array([np.nan, 1.0, -3.0, np.inf])) == (-3.0, 1.0)


def test_lsb_report_counts():
    a = np.array([0.0, 1.0, 2.0, np.nan])
    r = O.lsb_report(a, a, (0.0, 2.0))
    assert r == {"max_lsb": 0, "exact_frac": 1.0, "n": 3}
