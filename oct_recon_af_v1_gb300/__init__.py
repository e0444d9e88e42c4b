"""GB300-native (sm_103a) per-plane OCT reconstruction for octrecon.

Hand-written CUDA kernels behind a C ABI (include/octgb.h, liboctgb.so),
called from Python through ctypes.  The host side mirrors the reference
octrecon operator interfaces:

  geometry.build_spectral_geometry   octrecon/core/geometry.py:84-128
  spectral.SpectralProcessor         octrecon/core/spectral.py:84-165
  stitching.TileStitcher             octrecon/core/stitching.py:81-139
  reconstruct.RowReconstructor       octrecon/pipeline.py:223-302 (process_row)
  quantise.db_to_bits                octrecon/io/tiff_writer.py:33-38
  plugin.register                    device "gb300" for octrecon/backend.py:61-83

There is no CPU fallback: every compute call goes to the CUDA library and fails
loudly when it is missing.
"""
from __future__ import annotations

from ._build import LIB, build as _build_lib

__all__ = ["build", "LIB", "Context"]


def build(force: bool = False, verbose: bool = False):
    """Compile liboctgb.so for sm_103a (incremental)."""
    return _build_lib(force=force, verbose=verbose)


def __getattr__(name):
    if name == "Context":
        from ._lib import Context
        return Context
    raise AttributeError(name)
