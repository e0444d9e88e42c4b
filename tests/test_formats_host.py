"""Rare raw formats on the host (no GPU): the oracle's prepare_raw,
AScanBinning and average_repeats restatements against the reference's own
outputs (tests/golden/formats_case.npz, make_golden_formats.py), bit for bit."""
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
