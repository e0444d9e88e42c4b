"""Generate the Thorlabs SRR fixtures of tests/golden/ by running the reference.

    python tests/golden/make_golden_srr.py /path/to/reference

Same stand-ins as make_golden.py (empty `tifffile`, NumPy path).  One scan
written by the reference's own generator (scripts/make_synthetic_volume.py,
format "srr": one .srr file per B-scan repeat, upper 4 bits of every word set
at random, which the reader must mask off), 2 x 1 tiles x depths 0 and 10 um,
8 A-scans, 2 frames, B-scan repeats 2, n = 2048:

  srr_volume.tar.xz  the scan itself
  srr_case.npz       the reference's process_planes([1]) plane at float64 and
                     float32; the first tile's files as stored (words after the
                     header, (files, file_lines, n) uint16) with the header's
                     apodisation / scan line ranges, and the reference
                     reader's decoded read_bscans of them, to pin the oracle's
                     restatement of the 12-bit decode.
"""
from __future__ import annotations

import sys
import tarfile
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


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
    work = Path(tempfile.mkdtemp(prefix="octgb_srr_"))
    out = {}
    try:
        vol = work / "srr"
        make_volume(vol, nx=8, ny=2, tiles_x=2, tiles_y=1, depths=(0.0, 0.01), n_lambda=2048, seed=5, fmt="srr",
                    bscan_avg=2)
        for prec in ("float64", "float32"):
            cfg = ReconConfig(volume_folder=str(vol), device="cpu", precision=prec,
                              dispersion_quadratic_term=8.949e7, focus_positions=200.0, focus_sigma=10,
                              crop_z_range_mm="none", output_pixel_size_um=2, interp_method="sinc5",
                              batch_frames=2, io_threads=1, write_tiff=False)
            R = Reconstructor(cfg, log=lambda *a: None)
            out[f"plane_{prec}"] = R.process_planes([1])[0]
        hdr = R.hdr
        t = R.si.tiles_in_row(0)[0]
        rd = R.reader(t.folder)
        files = list(range(hdr.size_y * max(1, hdr.bscan_avg)))
        raw = np.empty((len(files), hdr.interf_size, hdr.n_lambda), np.dtype(hdr.raw_dtype))
        rd.read_bscans(files, raw)
        h = rd.srr
        words = []
        for fi in files:
            b = (Path(rd.dir) / rd.file_name(fi)).read_bytes()
            words.append(np.frombuffer(b, dtype="<u2", offset=h["headerTotalBytes"]).reshape(-1, hdr.n_lambda))
        out["words"] = np.stack(words)
        out["ranges"] = np.array([h["apodstart"], h["apodend"], h["scanstart"], h["scanend"]])
        out["decoded"] = raw
        with tarfile.open(HERE / "srr_volume.tar.xz", "w:xz") as tf:
            tf.add(vol, arcname="srr")
    finally:
        ref_spectral.SpectralProcessor.__init__ = orig_init
    np.savez_compressed(HERE / "srr_case.npz", **out)
    print("wrote", HERE / "srr_case.npz", HERE / "srr_volume.tar.xz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <path of the octrecon source tree>")
    main(sys.argv[1])
