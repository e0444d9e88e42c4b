"""Legacy TIFF output on the GPU: the double-quantisation table and the
PackBits kernel against the oracle (bit for bit, byte for byte), the written
BigTIFF read back against db_to_bits of the float volume, and
Reconstructor.run() on device gb300 writing the TIFF of the telesto scan."""
from __future__ import annotations

import json
import tarfile

import numpy as np
import pytest

from oracle import numerics as O
from octrecon_ref import import_octrecon

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oct_recon_af_v1_gb300 as pkg
    pkg.build()
    from oct_recon_af_v1_gb300._lib import Context
    c = Context(0)
    yield c
    c.close()


def planes(rng, nz=50, nx=37):
    p = (rng.standard_normal((3, nz, nx)) * 12 - 40).astype(np.float32)
    p[0, :3, :5] = np.nan
    p[1, 10:20] = -40.0                                             # long equal runs
    p[2] = np.nan                                                   # a plane with no finite value
    return p


def test_double_quantisation_bit_exact(ctx):
    rng = np.random.default_rng(1)
    vol = planes(rng)
    clim = (-85.0, 12.5)
    for p in vol:
        pc = O.plane_clim(p)
        ref = O.legacy_double_bits(p, pc, clim)
        np.testing.assert_array_equal(ctx.quantise_double(p, pc, clim), ref)
    p = vol[0]
    np.testing.assert_array_equal(ctx.quantise_double(p, (-50.0, -30.0), clim),
                                  O.legacy_double_bits(p, (-50.0, -30.0), clim))


def test_packbits_kernel_matches_oracle(ctx):
    rng = np.random.default_rng(2)
    imgs = [rng.integers(0, 65536, (40, 33), dtype=np.uint16), np.zeros((7, 300), np.uint16),
            rng.integers(0, 3, (64, 1900), dtype=np.uint16), np.full((3, 1), 513, np.uint16)]
    for img in imgs:
        data, sizes = ctx.packbits(img)
        off = 0
        for r in range(img.shape[0]):
            ref = O.packbits_encode_row(img[r].astype("<u2").tobytes())
            assert data[off:off + sizes[r]] == ref
            off += int(sizes[r])
        assert off == len(data)


def test_written_tiff_round_trip(ctx, tmp_path):
    from oct_recon_af_v1_gb300 import tiff
    rng = np.random.default_rng(3)
    vol = planes(rng, 61, 45)
    clim = O.plane_clim(vol[np.isfinite(vol)])
    meta = {"x": {"order": 1, "units": "mm"}, "note": "test"}
    path = tmp_path / "v.tiff"
    tiff.write_legacy_tiff(path, vol, clim, meta)
    codes, m = tiff.read_legacy_tiff(path)
    np.testing.assert_array_equal(codes, O.db_to_bits(vol.astype(np.float64), clim))
    assert m == {"metadata": meta, "clim": [float(clim[0]), float(clim[1])], "version": 3}
    assert json.loads((tmp_path / "v.tiff.json").read_text()) == m
    pcs = np.array([O.plane_clim(p) for p in vol])
    tiff.write_legacy_tiff(path, vol, clim, meta, True, pcs, rows_per_strip=7)
    codes, _ = tiff.read_legacy_tiff(path)
    for k, p in enumerate(vol):
        np.testing.assert_array_equal(codes[k], O.legacy_double_bits(p, pcs[k], clim))


def test_reconstructor_run_writes_tiff(ctx, tmp_path):
    import_octrecon()
    from octrecon.pipeline import ReconConfig, Reconstructor

    from oct_recon_af_v1_gb300 import plugin, tiff
    plugin.register()
    import conftest
    with tarfile.open(conftest.GOLDEN / "telesto_volume.tar.gz") as tf:
        tf.extractall(tmp_path, filter="data")
    vol = tmp_path / "telesto"
    info = json.loads((vol / "synthetic_info.json").read_text())
    cfg = ReconConfig(volume_folder=str(vol), device="gb300", precision="float32", dispersion_quadratic_term=8.949e7,
                      focus_positions=float(info["focus_pix"]), focus_sigma=10, crop_z_range_mm="none",
                      output_pixel_size_um=info.get("pixel_um", 2), interp_method="sinc5", batch_frames=4,
                      io_threads=2, write_tiff=True, keep_float_volume=True, output_root=str(tmp_path / "out"),
                      output_name="rec")
    R = Reconstructor(cfg, log=lambda *a: None)
    summary = R.run()
    codes, meta = tiff.read_legacy_tiff(summary["tiff"])
    db = np.load(summary["float_volume"])
    np.testing.assert_array_equal(codes, O.db_to_bits(db.astype(np.float64), summary["clim_dB"]))
    assert meta["clim"] == list(summary["clim_dB"]) and meta["version"] == 3
