"""Legacy TIFF on the host (no GPU): the package's PackBits decoder inverts
the oracle's encoder, including runs, literals, 128-byte limits and ragged
ends."""
from __future__ import annotations

import numpy as np

from oracle import numerics as O


def test_packbits_round_trip():
    from oct_recon_af_v1_gb300.tiff import packbits_decode
    rng = np.random.default_rng(5)
    cases = [b"", b"\x01", b"\x01\x01", b"\x02\x02\x02", bytes(300), bytes(range(256)) * 2,
             bytes([7]) * 129 + b"\x01\x02" + bytes([9]) * 3]
    for _ in range(50):
        n = int(rng.integers(1, 2000))
        cases.append(bytes(rng.integers(0, 3, n, dtype=np.uint8)))      # many short runs
    for c in cases:
        enc = O.packbits_encode_row(c)
        assert packbits_decode(enc) == c
        assert len(enc) <= len(c) + (len(c) + 127) // 128
