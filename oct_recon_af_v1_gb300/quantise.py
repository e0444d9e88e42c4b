"""Legacy uint16 quantisation on the device (octrecon/io/tiff_writer.py:26-50).

bits = min(uint16(round_half_away((dB - c1) / (c2 - c1) * 65534)) + 1, 65535),
NaN -> 0, clim = [min, max] of all finite dB of the volume.
"""
from __future__ import annotations

from ._lib import Context


def db_to_bits(ctx: Context, db, clim, out=None):
    return ctx.quantise(db, clim, out)


def plane_clim(ctx: Context, db):
    return ctx.minmax(db)
