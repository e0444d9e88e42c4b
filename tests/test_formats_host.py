"""Rare raw formats on the host (no GPU): the oracle's prepare_raw,
AScanBinning, average_repeats and SRR 12-bit decode restatements against the
reference's own outputs (tests/golden/formats_case.npz, make_golden_formats.py;
srr_case.npz, make_golden_srr.py), bit for bit."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from oracle import numerics as O

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def fmt():
    return dict(np.load(GOLDEN / "formats_case.npz"))


@pytest.mark.parametrize("name", ["combo", "wasatch"])
def test_prepare_raw_matches_reference(fmt, name):
    apod, binning, nb, na, size_x, frame_mean = (int(v) for v in fmt[f"{name}_hdr"])
    got = O.prepare_raw(fmt[f"{name}_raw"], apod, binning, "frame_mean" if frame_mean else "lines", nb)
    ref = fmt[f"{name}_prepared"]
    assert got.dtype == ref.dtype and got.shape == ref.shape
    np.testing.assert_array_equal(got, ref)


def test_average_repeats_matches_reference(fmt):
    np.testing.assert_array_equal(O.average_repeats(fmt["rep_mag"], 3, 2, 5, 3), fmt["rep_out"])


def test_binning_edges():
    x = np.arange(2 * 7 * 3, dtype=np.float32).reshape(2, 7, 3)
    assert O.bin_ascans(x, 1).shape == (2, 7, 3)
    b3 = O.bin_ascans(x, 3)                         # kept columns 0, 3, 6; zero padding at both ends
    assert b3.shape == (2, 3, 3)
    h = np.float32(1.0 / 3)
    np.testing.assert_array_equal(b3[:, 0], (x[:, 0] * h + x[:, 1] * h))
    np.testing.assert_array_equal(b3[:, 2], (x[:, 5] * h + x[:, 6] * h))


def test_srr_decode_matches_reference_reader():
    srr = np.load(GOLDEN / "srr_case.npz")
    a0, a1, s0, s1 = (int(v) for v in srr["ranges"])
    assert (srr["words"] >= 4096).any()                 # the upper bits are set in the files
    got = O.srr_decode(srr["words"], (a0, a1), (s0, s1))
    assert got.dtype == srr["decoded"].dtype
    np.testing.assert_array_equal(got, srr["decoded"])


def test_plugin_srr_words_match_reference_reader(tmp_path):
    """The plug-in's read-ahead of SRR files (words as stored) followed by the
    oracle's decode equals the reference reader's read_bscans."""
    import tarfile

    from octrecon_ref import import_octrecon
    import_octrecon()
    from octrecon.io.srr import SRRTileReader

    from oct_recon_af_v1_gb300.plugin import _is_srr, _srr_words
    with tarfile.open(GOLDEN / "srr_volume.tar.xz") as tf:
        tf.extractall(tmp_path, filter="data")
    tile = sorted(p for p in (tmp_path / "srr").rglob("*.srr"))[0].parent
    rd = SRRTileReader(tile)
    assert _is_srr(rd)
    files = [0, 3, 1]
    sw = _srr_words(rd, files, rd.header.n_lambda)
    ref = np.empty((len(files), rd.header.interf_size, rd.header.n_lambda), np.int16)
    rd.read_bscans(files, ref)
    np.testing.assert_array_equal(O.srr_decode(sw.words, sw.apod_range, sw.scan_range), ref)
