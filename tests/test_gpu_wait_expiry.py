"""A bounded device wait that runs out: the kernels' error path.

octgb_selftest_wait_expiry makes each CTA's first row-copy barrier expect 16
bytes more than its copies deliver (every copy lands; only that barrier never
completes) with the wait limit cut to a few milliseconds.  The wait must run
out, the kernel must drain what it issued (the spectral kernel its threads'
row copies; the tensor-core kernel its copies and MMAs, and free its tensor
memory) and
report through the status word; the call returns OCTGB_ERR_TIMEOUT and the
same context then reconstructs normally.  No GPU faults, traps or hangs: every
wait is bounded and every copy issued is a valid one.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1], ids=["spectral", "precision"])
def test_starved_wait_expires_and_context_recovers(gpu_ctx, spectral_case, which):
    from oct_recon_af_v1_gb300 import _lib
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import synthetic
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    gpu_ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    raw = synthetic.generate_numpy(2, 64, 25, seed=7)
    before = gpu_ctx.magnitude(raw, 25)
    rc = gpu_ctx.lib.octgb_selftest_wait_expiry(gpu_ctx.h, which, 2000)        # 2 ms limit
    assert rc == _lib.ERR_TIMEOUT, (rc, gpu_ctx.lib.octgb_last_error(gpu_ctx.h))
    assert b"expired" in gpu_ctx.lib.octgb_last_error(gpu_ctx.h)
    # the context (stream, status word, buffers) works as before, at the normal limit
    np.testing.assert_array_equal(gpu_ctx.magnitude(raw, 25), before)
    if which == 1:
        a = gpu_ctx.magnitude_precision(raw, 25)
        np.testing.assert_array_equal(gpu_ctx.magnitude_precision(raw, 25), a)


def test_selftest_rejects_bad_arguments(gpu_ctx):
    from oct_recon_af_v1_gb300 import _lib
    for which, us in ((2, 2000), (0, 10), (0, 5_000_000)):
        assert gpu_ctx.lib.octgb_selftest_wait_expiry(gpu_ctx.h, which, us) == _lib.ERR_ARG
