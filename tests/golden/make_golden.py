"""Generate the golden fixtures of tests/golden/ by running the reference.

Needs the reference octrecon source tree (read-only) and its synthetic volume
generator; run in a container where it is importable:

    python tests/golden/make_golden.py /path/to/reference

`tifffile` is replaced by an empty stub module (only the TIFF writer uses it)
and the Numba kernel is switched off (numba is absent), so the reference runs
its NumPy path.  Outputs (committed, small):

  telesto_case.npz   the reference's own `telesto` format-test case
                     (tests/test_formats.py:47-58, make_volume seed 1): raw
                     int16 tiles, scan layout, resolved parameters, the
                     reference's stitch operators, its float64 and float32
                     planes for output y = 1, and the unmodified-MATLAB golden
                     plane + tie mask from tests/data/legacy_formats_ref.npz.
  telesto_volume.tar.gz  the same `telesto` scan as the reference's generator
                     writes it to disk (ScanInfo.json, Thorlabs Header.xml,
                     data/Spectral*.data, chirp): input of the end-to-end test
                     that drives the reference's own Reconstructor on device
                     "gb300".
  spectral_case.npz  one synthetic B-scan (config-0 spectrum model, uint16,
                     25 apodisation + 64 A-scans, seed 7) with the reference
                     geometry (sinc idx/w, window) and its SpectralProcessor
                     magnitudes at float32 and float64.
"""
from __future__ import annotations

import json
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]


def main(ref_root: str):
    ref_root = Path(ref_root)
    sys.modules.setdefault("tifffile", types.ModuleType("tifffile"))
    sys.path.insert(0, str(ref_root))
    sys.path.insert(0, str(ref_root / "scripts"))
    sys.path.insert(0, str(REPO))
    from make_synthetic_volume import make_volume
    from octrecon.core.geometry import build_spectral_geometry
    from octrecon.core.spectral import SpectralProcessor
    from octrecon.pipeline import ReconConfig, Reconstructor

    from oct_recon_af_v1_gb300 import synthetic

    # ------------------------------------------------------------ telesto pipeline case
    work = Path(tempfile.mkdtemp(prefix="octgb_golden_"))
    vol = work / "telesto"
    make_volume(vol, nx=8, ny=2, tiles_x=2, tiles_y=1, depths=(0.0, 0.01), n_lambda=2048, seed=1,
                system="telesto")
    info = json.loads((vol / "synthetic_info.json").read_text())
    out = {}
    for prec in ("float64", "float32"):
        cfg = ReconConfig(volume_folder=str(vol), device="cpu", precision=prec, dispersion_quadratic_term=8.949e7,
                          focus_positions=float(info["focus_pix"]), focus_sigma=10, crop_z_range_mm="none",
                          output_pixel_size_um=info.get("pixel_um", 2), interp_method="sinc5", batch_frames=4,
                          io_threads=2)
        R = Reconstructor(cfg, log=lambda *a: None)
        R.sp.use_numba = False
        out[prec] = R.process_planes([1])[0]
        if prec == "float32":
            R32 = R
    R = R32
    si, hdr = R.si, R.hdr
    tiles = si.tiles_in_row(0)
    raws = []
    for t in tiles:
        buf = np.empty((hdr.size_y, hdr.interf_size, hdr.n_lambda), np.dtype(hdr.raw_dtype))
        R.reader(t.folder).read_bscans(list(range(hdr.size_y)), buf)
        raws.append(buf)
    legacy = np.load(ref_root / "tests" / "data" / "legacy_formats_ref.npz")
    st = {}
    for (xi, zi), s in R.stitchers.items():
        key = f"st_{xi}_{zi}"
        st[key + "_rc"] = np.array([s.r0, s.r1, s.c0, s.c1])
        st[key + "_Wz"] = np.asarray(s.Wz)
        st[key + "_WxT"] = np.asarray(s.WxT)
        st[key + "_fz"] = np.asarray(s.fz)
    np.savez_compressed(
        HERE / "telesto_case.npz",
        raw=np.stack(raws),                                    # (tiles, frames, interf, N) int16
        tile_xi=np.array([t.xi for t in tiles]), tile_zi=np.array([t.zi for t in tiles]),
        lambda_nm=R.lambda_nm, dispersion=np.float64(8.949e7), n_medium=np.float64(R.resolved["n_medium"]),
        focus_pix=np.asarray(R.focus, float), focus_sigma=np.float64(10.0),
        output_pixel_size_um=np.float64(R.resolved["output_pixel_size_um"]),
        apod_size=np.int64(hdr.apod_size),
        x_centers_mm=si.x_centers_mm, y_centers_mm=si.y_centers_mm, z_depths_mm=si.z_depths_mm,
        n_x_px=np.int64(si.n_x_px), n_y_px=np.int64(si.n_y_px), tile_range_x_mm=np.float64(si.tile_range_x_mm),
        tile_range_y_mm=np.float64(si.tile_range_y_mm), x_offset=np.float64(si.x_offset),
        y_offset=np.float64(si.y_offset), opc_poly=si.optical_path_polynomial(),
        out_x_mm=R.tg.out_x_mm, out_z_mm=R.tg.out_z_mm, tile_z_mm=R.tg.tile_z_mm,
        opc_shift=R.oc.shift, opc_pdz=R.oc.pdz,
        sinc_idx=R.sg.sinc_idx, sinc_w=R.sg.sinc_w, window=R.sg.window,
        plane_fp64=out["float64"], plane_fp32=out["float32"], plane_y=np.int64(1),
        matlab_plane=legacy["telesto__planeDb"], matlab_tie=legacy["telesto__tie"],
        **st)

    import tarfile
    with tarfile.open(HERE / "telesto_volume.tar.gz", "w:gz") as tf:
        tf.add(vol, arcname="telesto")

    # ------------------------------------------------------------ spectral case (config-0 model)
    lam = synthetic.lambda_nm()
    beta = synthetic.beta_ref_from_px(1e-5)
    raw = synthetic.generate_numpy(1, 64, 25, seed=7)
    sg = build_spectral_geometry(lam, beta, 1.33, "sinc5")
    m32 = SpectralProcessor(sg, 25, dtype=np.float32, use_numba=False).magnitude(raw)
    m64 = SpectralProcessor(sg, 25, dtype=np.float64, use_numba=False).magnitude(raw)
    np.savez_compressed(HERE / "spectral_case.npz", raw=raw, lambda_nm=lam, dispersion=np.float64(beta),
                        n_medium=np.float64(1.33), apod_size=np.int64(25), sinc_idx=sg.sinc_idx,
                        sinc_w=sg.sinc_w, window=sg.window, z_um=sg.z_um, mag_fp32=m32.astype(np.float32),
                        mag_fp64=m64)
    print("wrote", HERE / "telesto_case.npz", HERE / "spectral_case.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <path of the octrecon source tree>")
    main(sys.argv[1])
