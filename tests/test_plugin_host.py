"""Host logic of the device plug-in's row pipeline (no GPU)."""
from __future__ import annotations

import numpy as np

from oct_recon_af_v1_gb300.plugin import _frame_chunks


def test_frame_chunks_split_runs_and_batches():
    f = np.array([0, 1, 2, 3, 4, 7, 8, 20])
    got = [(off, list(fr)) for off, fr in _frame_chunks(f, 3)]
    assert got == [(0, [0, 1, 2]), (3, [3, 4]), (5, [7, 8]), (7, [20])]
    # every frame once, in order, at its output offset
    assert [v for _, fr in _frame_chunks(f, 3) for v in fr] == list(f)
    assert _frame_chunks(np.arange(0), 4) == []
    whole = _frame_chunks(np.arange(270), 30)
    assert len(whole) == 9 and all(len(fr) == 30 and fr[0] == off for off, fr in whole)
