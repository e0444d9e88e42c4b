"""Parity at full workload sizes, in legacy codes with ONE shared clim, per dB
level (levels relative to the reference's median dB).

Three references, each computed on the CPU by the oracle from the same raws:
  * the Numba path (core/cpu_kernels.py:12-41 restated in C, pocketfft
    complex64 ifft, core/spectral.py:136-165), the reference CPU path;
  * its floor: the Numba spectrum through an inverse FFT without rounding
    (complex128).  Its deviation from the Numba path is pocketfft's own
    float32 rounding, which no float32 FFT of another operation order can
    reproduce; a GPU form is judged level by level against that deviation;
  * the float64 NumPy path (core/spectral.py:123-153 at float64).

Workloads: the 50 x (25 + 500) x 2048 volume of the single-tile case (z-crop
1000), the 6 tiles x 24 frames of one y-row of the 2 x 2 x 3 tiled volume
through the frame API (stitched, finalised), and 16 tiles of uneven size,
A-scan count and z-crop through the batched form.  The bounds below are the
measured values (GB300) with a small margin; the per-level tables print with
`pytest -s`.  Measured (overall exact codes / max LSB; the floor in brackets):
  single tile, float32 form vs Numba path   99.764 % / 7   (99.851 % / 5)
  single tile, precision form vs float64    99.736 % / 12  (float32 FFT of the
                                            exact spectrum: 99.844 % / 5)
  y-row slab, frame API vs oracle           99.840 % / 4   (99.900 % / 3)
  16 uneven tiles, batched form vs oracle   99.786 % / 2   (99.868 % / 1)
At every level the float32 forms mismatch ~1.6x as often as the floor: two
independent float32 FFT roundings (this one's and pocketfft's) instead of one.
Above median - 10 dB every form is within 1 LSB.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import numerics as O

pytestmark = pytest.mark.gpu


def _db(m, lo=0, hi=1000):
    with np.errstate(divide="ignore"):
        return 20 * np.log10(np.asarray(m, np.float64)[..., lo:hi])


def _clim(db):
    fin = np.asarray(db)[np.isfinite(db)]
    return float(fin.min()), float(fin.max())


def _row(rows, lo):
    """The row of a level table starting at `lo` (None: all voxels)."""
    return next(r for r in rows if r["lo"] == lo)


def _within_floor(got, floor, ratio, slack):
    """Per level: the GPU form's code mismatches at most `ratio` x the floor's
    plus `slack` of the level's voxels."""
    for g, f in zip(got, floor):
        assert g["n"] == f["n"]
        allowed = ratio * (1.0 - f["exact_frac"]) + slack
        assert 1.0 - g["exact_frac"] <= allowed, (g, f)


@pytest.fixture(scope="module")
def config0():
    """The single-tile workload at full size and its three references."""
    from oct_recon_af_v1_gb300 import synthetic as S
    lam = S.lambda_nm()
    beta = S.beta_ref_from_px(1e-5)
    raw = S.generate_numpy(50, 500, 25, seed=0)
    og = O.spectral_geometry(lam, beta, 1.33)
    return dict(raw=raw, lam=lam, beta=beta, og=og,
                numba=_db(O.magnitude_numba(raw, og, 25)),
                floor=_db(O.magnitude_numba_exact_fft(raw, og, 25)),
                fp64=_db(O.magnitude_numpy(raw, og, 25, np.float64)))


def test_config0_float32_form_vs_reference_cpu_path(gpu_ctx, config0):
    from oct_recon_af_v1_gb300 import geometry as G
    c = config0
    sg = G.build_spectral_geometry(c["lam"], c["beta"], 1.33)
    gpu_ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    db, _ = gpu_ctx.db(c["raw"], 25, 0, 1000)
    assert np.isfinite(db).all()
    clim = _clim(c["numba"])
    got = O.lsb_levels(db, c["numba"], clim)
    floor = O.lsb_levels(c["floor"], c["numba"], clim)
    print("\n" + O.format_levels("config 0, float32 form vs Numba path", got))
    print(O.format_levels("config 0, floor (Numba spectrum, exact FFT) vs Numba path", floor))
    _within_floor(got, floor, ratio=2.0, slack=1e-4)
    assert _row(got, None)["exact_frac"] >= 0.9972
    assert _row(got, None)["max_lsb"] <= 8
    for lo in (-20.0, -10.0, 0.0, 10.0):                 # above median - 20 dB: within 1 LSB
        assert _row(got, lo)["max_lsb"] <= 1, _row(got, lo)
    # no less accurate than the reference's float32 path against float64
    c64 = _clim(c["fp64"])
    vs64 = O.lsb_levels(db, c["fp64"], c64)
    ref64 = O.lsb_levels(c["numba"], c["fp64"], c64)
    print(O.format_levels("config 0, float32 form vs float64", vs64))
    print(O.format_levels("config 0, Numba path vs float64", ref64))
    # (equal to within float32-FFT rounding: measured 91.5591 % vs 91.5596 %,
    # both 395 LSB; the float32 form keeps the reference's float32
    # apodisation-mean store, which sets this figure)
    assert _row(vs64, None)["exact_frac"] >= _row(ref64, None)["exact_frac"] - 2e-4
    assert _row(vs64, None)["max_lsb"] <= _row(ref64, None)["max_lsb"] + 1


def test_config0_precision_form_vs_float64(gpu_ctx, config0):
    from oct_recon_af_v1_gb300 import geometry as G
    c = config0
    sg = G.build_spectral_geometry(c["lam"], c["beta"], 1.33)
    gpu_ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    mag = gpu_ctx.magnitude_precision(c["raw"], 25)
    db = _db(mag)
    clim = _clim(c["fp64"])
    got = O.lsb_levels(db, c["fp64"], clim)
    # the float32-FFT floor against float64: the exact spectrum rounded to
    # complex64 and transformed by pocketfft in float32
    s64 = O.pre_fft_numpy(c["raw"], c["og"], 25, np.float64)
    f32 = _db(np.abs(O.ifft_rows(s64.astype(np.complex64))[..., :1024]).astype(np.float32))
    floor = O.lsb_levels(f32, c["fp64"], clim)
    print("\n" + O.format_levels("config 0, precision form vs float64", got))
    print(O.format_levels("config 0, float32 FFT of the exact spectrum vs float64", floor))
    # the split-FP16 sinc adds a relative error (~3.5e-7) a float32 store does
    # not: at the strongest level the mismatch rate is 2.8x the floor's
    _within_floor(got, floor, ratio=3.0, slack=1e-4)
    assert _row(got, None)["exact_frac"] >= 0.9970
    assert _row(got, None)["max_lsb"] <= 13
    for lo in (-20.0, -10.0, 0.0, 10.0):
        assert _row(got, lo)["max_lsb"] <= 1, _row(got, lo)


def _yrow_case(torch, frames):
    """Tiles of y-row 0 of the tiled workload (6 tiles, `frames` B-scans each),
    generated on the device, with the package's plans and the oracle's stitchers."""
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300 import synthetic
    lay, focus = synthetic.config1_layout()
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    tg = S.tiled_geometry(lay, sg.z_um, focus, 1.0)
    order = [(xi, zi) for xi in range(2) for zi in range(3)]
    raws = [synthetic.u16_bits(synthetic.generate(frames, lay.n_x_px, 25, seed=500 + k, device="cuda", chunk=8))
            for k in range(len(order))]
    og = O.spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    sd = O.ScanDesc(lay.x_centers_mm, lay.y_centers_mm, lay.z_depths_mm, lay.n_x_px, lay.n_y_px,
                    lay.tile_range_x_mm, lay.tile_range_y_mm)
    otg = O.tiled_geometry(sd, og.z_um, focus, 1.0)
    return dict(lay=lay, focus=focus, sg=sg, tg=tg, order=order, raws=raws, og=og, otg=otg)


def _oracle_row(c, fft_exact=False):
    """Oracle reconstruction of the row slab: per tile the Numba path (or its
    exact-FFT floor), TileStitcher.contribute, row accumulation, finalise."""
    nF = c["raws"][0].shape[0]
    nz, nx = len(c["otg"].out_z_mm), len(c["otg"].out_x_mm)
    num = np.zeros((nF, nz, nx), np.float32)
    den = np.zeros((nF, nz, nx), np.float32)
    mag_fn = O.magnitude_numba_exact_fft if fft_exact else O.magnitude_numba
    for (xi, zi), raw in zip(c["order"], c["raws"]):
        st = O.Stitcher(c["otg"], c["lay"].x_centers_mm[xi], c["lay"].z_depths_mm[zi], c["focus"][zi], 80.0)
        if st.empty:
            continue
        n_, d_ = st.contribute(mag_fn(raw.cpu().numpy().view(np.uint16), c["og"], 25))
        num[:, :, st.c0:st.c1] += n_
        den[:, :, st.c0:st.c1] += d_
    return O.finalise(num, den)


def test_config1_yrow_slab_vs_reference_cpu_path(gpu_ctx):
    """One y-row of the tiled workload (6 tiles x 24 frames x 1000 A-scans):
    spectral stage, focus-weighted stitching and finalise through the frame
    API, against process_row's work in the oracle (pipeline.py:223-300)."""
    torch = pytest.importorskip("torch")
    from oct_recon_af_v1_gb300 import stitching as S
    c = _yrow_case(torch, 24)
    gpu_ctx.set_geometry(c["sg"].sinc_idx, c["sg"].sinc_w, c["sg"].window)
    ids = []
    for xi, zi in c["order"]:
        st = S.TileStitcher.build(c["tg"], c["lay"].x_centers_mm[xi], c["lay"].z_depths_mm[zi], c["focus"][zi], 80.0)
        ids.append(st.upload(gpu_ctx))
    nz, nx = len(c["tg"].out_z_mm), len(c["tg"].out_x_mm)
    thr = S.min_weight_threshold(np.float32)
    db = np.empty((24, nz, nx), np.float32)
    for f0 in range(0, 24, 8):                       # three frame batches of the row
        db[f0:f0 + 8] = gpu_ctx.frames_process(ids, [r[f0:f0 + 8] for r in c["raws"]], 25, f0, nz, nx, thr,
                                               raw_dtype=0)
    ref = _oracle_row(c)
    floor_db = _oracle_row(c, fft_exact=True)
    np.testing.assert_array_equal(np.isnan(db), np.isnan(ref))
    clim = _clim(ref)
    got = O.lsb_levels(db, ref, clim)
    floor = O.lsb_levels(floor_db, ref, clim)
    print("\n" + O.format_levels("y-row slab (6 tiles x 24 frames), GPU vs oracle", got))
    print(O.format_levels("y-row slab, floor (exact FFT) vs oracle", floor))
    _within_floor(got, floor, ratio=2.0, slack=1e-4)
    assert _row(got, None)["exact_frac"] >= 0.9980
    assert _row(got, None)["max_lsb"] <= 5
    for lo in (-30.0, -20.0, -10.0, 0.0, 10.0):
        assert _row(got, lo)["max_lsb"] <= 1, _row(got, lo)


def test_config3_sixteen_uneven_tiles_in_lsb(gpu_ctx):
    """16 tiles of uneven A-scan count, B-scan count and z-crop in one batched
    launch, each against the oracle's single-tile stitching and finalise, in
    codes with one clim over all tiles."""
    torch = pytest.importorskip("torch")
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300 import synthetic
    rng = np.random.default_rng(16)
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    gpu_ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    og = O.spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    tiles = []
    for k in range(16):
        B, nx, crop = int(rng.integers(2, 7)), int(rng.integers(300, 1201)), int(rng.integers(400, 1501))
        focus = float(rng.uniform(250, 650))
        lay = S.ScanLayout(np.array([0.0]), np.array([0.0]), np.array([0.0]), nx, B, nx * 1e-3, B * 1e-3)
        full = S.tiled_geometry(lay, sg.z_um, [focus], 1.0)
        crop = min(crop, len(full.out_z_mm))
        z0 = int(rng.integers(0, len(full.out_z_mm) - crop + 1))
        zr = (full.out_z_mm[z0] - 1e-9, full.out_z_mm[z0 + crop - 1] + 1e-9)
        tg = S.tiled_geometry(lay, sg.z_um, [focus], 1.0, zr)
        st = S.TileStitcher.build(tg, 0.0, 0.0, focus, 80.0)
        raw = synthetic.u16_bits(synthetic.generate(B, nx, 25, seed=1600 + k, device="cuda"))
        db = torch.full((B, nx, len(tg.out_z_mm)), -1.0, dtype=torch.float32, device="cuda")
        tiles.append(dict(raw=raw, plan=st.upload(gpu_ctx), db=db, st=st))
    thr = S.min_weight_threshold(np.float32)
    gpu_ctx.batch_process([(t["raw"], 25, t["plan"], t["db"]) for t in tiles], thr, grab=4)
    gpu_ctx.synchronize()
    gots, refs, floors = [], [], []
    for t in tiles:
        raw = t["raw"].cpu().numpy().view(np.uint16)
        st = t["st"]
        stn = O.Stitcher.__new__(O.Stitcher)
        stn.r0, stn.r1, stn.c0, stn.c1 = st.r0, st.r1, st.c0, st.c1
        stn.Wz, stn.WxT, stn.fz, stn.dtype = st.Wz, st.WxT, st.fz, np.float32
        for fn, acc in ((O.magnitude_numba, refs), (O.magnitude_numba_exact_fft, floors)):
            num, den = stn.contribute(fn(raw, og, 25))
            acc.append(O.finalise(num, den).ravel())
        gots.append(t["db"].cpu().numpy().transpose(0, 2, 1).ravel())
    got_db, ref_db, floor_db = (np.concatenate(v) for v in (gots, refs, floors))
    np.testing.assert_array_equal(np.isnan(got_db), np.isnan(ref_db))
    clim = _clim(ref_db)
    got = O.lsb_levels(got_db, ref_db, clim)
    floor = O.lsb_levels(floor_db, ref_db, clim)
    print("\n" + O.format_levels("16 uneven tiles (batched form) vs oracle", got))
    print(O.format_levels("16 uneven tiles, floor (exact FFT) vs oracle", floor))
    _within_floor(got, floor, ratio=2.0, slack=1e-4)
    assert _row(got, None)["exact_frac"] >= 0.9975
    assert _row(got, None)["max_lsb"] <= 3
    for lo in (-30.0, -20.0, -10.0, 0.0, 10.0):
        assert _row(got, lo)["max_lsb"] <= 1, _row(got, lo)
