"""Product host code against the reference's operators (CPU only).

The package builds its own FP64 geometry and stitching operators (own band
search instead of the reference's N x N distance matrix); they must equal the
reference's, which the fixtures store.
"""
from __future__ import annotations

import numpy as np

from oct_recon_af_v1_gb300 import geometry as G
from oct_recon_af_v1_gb300 import stitching as S
from oct_recon_af_v1_gb300 import synthetic


def test_spectral_geometry_equals_reference(spectral_case, telesto):
    for c in (spectral_case, telesto):
        sg = G.build_spectral_geometry(c["lambda_nm"], float(c["dispersion"]), float(c["n_medium"]))
        np.testing.assert_array_equal(sg.sinc_idx, c["sinc_idx"])
        np.testing.assert_array_equal(sg.sinc_w, c["sinc_w"])
        np.testing.assert_allclose(sg.window, c["window"], rtol=0, atol=1e-14)
        # compact band form agrees with the padded (N, T) form
        for i in range(0, sg.n, 97):
            L = sg.band_len[i]
            np.testing.assert_array_equal(sg.sinc_idx[i, :L], sg.band_start[i] + np.arange(L))
            assert np.all(sg.sinc_w[i, L:] == 0)
    np.testing.assert_array_equal(
        G.build_spectral_geometry(spectral_case["lambda_nm"], 0.0, 1.33).z_um, spectral_case["z_um"])


def test_matlab_grids():
    np.testing.assert_array_equal(G.linspace_matlab(0.0, 1.0, 5), [0, 0.25, 0.5, 0.75, 1.0])
    c = G.colon_matlab(-0.5, 0.1, 0.5)
    assert len(c) == 11 and c[0] == -0.5 and abs(c[-1] - 0.5) < 1e-15
    assert len(G.colon_matlab(1.0, 1.0, 0.0)) == 0
    lam = G.chirp_to_lambda(np.arange(2048.0), "telesto")
    assert abs(lam[0] - 1208.69) < 1e-9 and abs(lam[-1] - 1372.50) < 1e-9


def _layout(t):
    return S.ScanLayout(t["x_centers_mm"], t["y_centers_mm"], t["z_depths_mm"], int(t["n_x_px"]), int(t["n_y_px"]),
                        float(t["tile_range_x_mm"]), float(t["tile_range_y_mm"]), float(t["x_offset"]),
                        float(t["y_offset"]))


def test_stitch_operators_equal_reference(telesto):
    t = telesto
    sg = G.build_spectral_geometry(t["lambda_nm"], float(t["dispersion"]), float(t["n_medium"]))
    tg = S.tiled_geometry(_layout(t), sg.z_um, t["focus_pix"], float(t["output_pixel_size_um"]))
    np.testing.assert_array_equal(tg.out_z_mm, t["out_z_mm"])
    np.testing.assert_array_equal(tg.out_x_mm, t["out_x_mm"])
    np.testing.assert_array_equal(tg.tile_z_mm, t["tile_z_mm"])
    oc = S.OpticalPathCorrection.build(t["opc_poly"], tg.tile_x_mm, tg.tile_y_mm, tg.tile_z_mm)
    np.testing.assert_array_equal(oc.shift, t["opc_shift"])
    np.testing.assert_allclose(oc.pdz, t["opc_pdz"], rtol=0, atol=1e-12)
    for xi, zi in zip(t["tile_xi"], t["tile_zi"]):
        st = S.TileStitcher.build(tg, t["x_centers_mm"][xi], t["z_depths_mm"][zi], t["focus_pix"][zi],
                                  float(t["focus_sigma"]))
        key = f"st_{xi}_{zi}"
        assert [st.r0, st.r1, st.c0, st.c1] == list(t[key + "_rc"])
        np.testing.assert_array_equal(st.Wz, t[key + "_Wz"])
        np.testing.assert_array_equal(st.WxT, t[key + "_WxT"])
        np.testing.assert_array_equal(st.fz, t[key + "_fz"])
        # the device plan relies on <= 2 adjacent non-zeros per row / column
        for M in (st.Wz, st.WxT.T):
            for row in M:
                nz = np.flatnonzero(row)
                assert len(nz) <= 2 and (len(nz) < 2 or nz[1] == nz[0] + 1)


def test_threshold_and_factor_z():
    assert S.min_weight_threshold(np.float32) < S.MIN_WEIGHT
    f = S.factor_z(1024, 400.0, 80.0)
    assert abs(f[399] - (1 + S.MIN_WEIGHT)) < 1e-15
    assert abs(f.min() - S.MIN_WEIGHT) < 1e-6


def test_synthetic_generator_shapes_and_range():
    raw = synthetic.generate_numpy(2, 16, 25, seed=3)
    assert raw.shape == (2, 41, 2048) and raw.dtype == np.uint16
    again = synthetic.generate_numpy(2, 16, 25, seed=3)
    np.testing.assert_array_equal(raw, again)            # seeded
    env = synthetic.envelope(synthetic.SpectrumParams())
    assert abs(raw[:, :25, 1024].mean() - env[1024]) < 30    # background line ~ envelope
    lam = synthetic.lambda_nm()
    assert abs(lam[0] - 796.0) < 1e-9 and abs(lam[-1] - 1010.0) < 1e-9
