"""ORACLE — test infrastructure, not product code.

CPU restatement of the reference (`octrecon`, atesfet/oct_recon_AF_v1) per-plane
reconstruction path, used only as the checker by `tests/`, by
`__graft_entry__.smoke()` and by `bench.py`'s CPU-baseline / reference arm.
The product package (`oct_recon_af_v1_gb300`) never imports this package.

Parity is pinned: `tests/test_oracle_golden.py` checks this restatement against
the reference's own golden vectors (`tests/data/legacy_formats_ref.npz`
`telesto__planeDb`, unmodified-MATLAB output) and against fixtures produced by
running the reference itself (`tests/golden/make_golden.py`).

Modules:
  numerics   C/OpenMP restatement of core/cpu_kernels.py:12-41 (ctypes), the
             FP64 NumPy path (core/spectral.py:123-153 at float64), geometry
             (core/geometry.py:30-128, dense form), stitching
             (core/stitching.py:20-139), finalise (pipeline.py:296-300) and the
             legacy quantisation (io/tiff_writer.py:26-50).
"""
