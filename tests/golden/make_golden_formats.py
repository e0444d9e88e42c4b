"""Generate the rare-format fixtures of tests/golden/ by running the reference.

    python tests/golden/make_golden_formats.py /path/to/reference

Same stand-ins as make_golden.py (empty `tifffile`, NumPy path).  Two scans
written by the reference's own generator (scripts/make_synthetic_volume.py),
2 x 1 tiles x depths 0 and 10 um, 8 A-scans, 2 frames, n = 2048:

  combo    Thorlabs, AScanBinning 2, B-scan repeats 2, A-scan repeats 2
  wasatch  Wasatch raw (no apodisation lines: frame-mean background),
           B-scan repeats 2

For each: the scan itself (formats_volumes.tar.xz), and the reference's
process_planes([1]) plane at float64 and float32 (formats_case.npz), plus the
reference's prepare_raw of the first tile's files and average_repeats of
seeded magnitudes, to pin the oracle's restatements.
"""
from __future__ import annotations

import sys
import tarfile
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CASES = {"combo": dict(fmt="thorlabs", spectra_avg=2, bscan_avg=2, ascan_avg=2),
         "wasatch": dict(fmt="wasatch", bscan_avg=2)}


def main(ref_root: str):
    ref_root = Path(ref_root)
    sys.modules.setdefault("tifffile", types.ModuleType("tifffile"))
    sys.path.insert(0, str(ref_root))
    sys.path.insert(0, str(ref_root / "scripts"))
    import octrecon.core.spectral as ref_spectral
    from make_synthetic_volume import make_volume
    from octrecon.pipeline import ReconConfig, Reconstructor

    orig_init = ref_spectral.SpectralProcessor.__init__

    def numpy_init(self, *a, **kw):
        kw["use_numba"] = False
        orig_init(self, *a, **kw)

    ref_spectral.SpectralProcessor.__init__ = numpy_init
    work = Path(tempfile.mkdtemp(prefix="octgb_fmt_"))
    out = {}
    try:
        for name, kw in CASES.items():
            vol = work / name
            make_volume(vol, nx=8, ny=2, tiles_x=2, tiles_y=1, depths=(0.0, 0.01), n_lambda=2048, seed=3, **kw)
            for prec in ("float64", "float32"):
                cfg = ReconConfig(volume_folder=str(vol), device="cpu", precision=prec,
                                  dispersion_quadratic_term=8.949e7, focus_positions=200.0, focus_sigma=10,
                                  crop_z_range_mm="none", output_pixel_size_um=2, interp_method="sinc5",
                                  batch_frames=2, io_threads=1, write_tiff=False)
                R = Reconstructor(cfg, log=lambda *a: None)
                out[f"{name}_plane_{prec}"] = R.process_planes([1])[0]
            hdr = R.hdr
            t = R.si.tiles_in_row(0)[0]
            files = list(range(hdr.size_y * max(1, hdr.bscan_avg)))
            raw = np.empty((len(files), hdr.interf_size, hdr.n_lambda), np.dtype(hdr.raw_dtype))
            R.reader(t.folder).read_bscans(files, raw)
            out[f"{name}_raw"] = raw
            out[f"{name}_hdr"] = np.array([hdr.apod_size, max(1, hdr.spectra_avg), max(1, hdr.bscan_avg),
                                           max(1, hdr.ascan_avg), hdr.size_x, 1 if hdr.apod_mode == "frame_mean"
                                           else 0])
            out[f"{name}_prepared"] = ref_spectral.prepare_raw(raw, hdr.apod_size, max(1, hdr.spectra_avg),
                                                               hdr.apod_mode, max(1, hdr.bscan_avg), np, np.float32)
        rng = np.random.default_rng(8)
        mag = rng.gamma(2.0, 1.0, size=(3 * 2, 5 * 3, 17)).astype(np.float32)
        hdr_like = types.SimpleNamespace(bscan_avg=2, ascan_avg=3, size_x=5)
        out["rep_mag"] = mag
        out["rep_out"] = ref_spectral.average_repeats(mag, 3, hdr_like)
        with tarfile.open(HERE / "formats_volumes.tar.xz", "w:xz") as tf:
            for name in CASES:
                tf.add(work / name, arcname=name)
    finally:
        ref_spectral.SpectralProcessor.__init__ = orig_init
    np.savez_compressed(HERE / "formats_case.npz", **out)
    print("wrote", HERE / "formats_case.npz", HERE / "formats_volumes.tar.xz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <path of the octrecon source tree>")
    main(sys.argv[1])
