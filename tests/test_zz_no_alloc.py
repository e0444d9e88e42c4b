"""The allocation-free magnitude entry point (octgb_magnitude_noalloc).

It serves callers that cannot allocate GPU memory while they reconstruct (a
frame-grabber callback, a process whose GPU memory belongs to another
framework's pool): it takes caller-owned device buffers and keeps its scratch
in a fixed array inside the library.  Its output must equal the ordinary
entry point's (octgb_magnitude) on consecutive calls, since every call reuses
the same scratch.  Collected last so a failure here cannot hide another
test's result.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_magnitude_on_consecutive_calls(spectral_case):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oct_recon_af_v1_gb300 as pkg
    pkg.build()
    from oct_recon_af_v1_gb300 import _lib, geometry, synthetic

    c = spectral_case
    sg = geometry.build_spectral_geometry(c["lambda_nm"], float(c["dispersion"]), float(c["n_medium"]))
    ctx = _lib.Context(0)
    try:
        ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
        lib = ctx.lib
        apod = int(c["apod_size"])
        batches = [c["raw"], synthetic.generate_numpy(3, 64, apod, seed=21)]
        for k, raw in enumerate(batches + batches[::-1]):     # consecutive calls, alternating inputs
            B, interf, N = raw.shape
            ref = ctx.magnitude(raw, apod)                     # the existing entry point
            dev = synthetic.u16_bits(torch.from_numpy(raw.astype(np.int32)).cuda())
            out = torch.full((B, interf - apod, N // 2), float("nan"), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            rc = lib.octgb_magnitude_noalloc(ctx.h, ctypes.c_void_p(dev.data_ptr()), _lib.U16, B, interf, apod,
                                             ctypes.c_void_p(out.data_ptr()))
            assert rc == _lib.OK, lib.octgb_last_error(ctx.h)
            ctx.synchronize()
            if k > 0:                                          # after the one-time set-up: nothing allocated
                assert torch.cuda.mem_get_info()[0] == free0
            got = out.cpu().numpy()
            scale = np.abs(ref).max()
            assert np.abs(got - ref).max() / scale < 2e-6
        # the largest batch the fixed scratch holds (64 B-scans fill it), and the
        # int16 and float32 raw types
        full = synthetic.generate_numpy(64, 8, apod, seed=22)
        for raw, dt in ((full, _lib.U16), (full.astype(np.int16), _lib.I16), (full.astype(np.float32), _lib.F32)):
            B, interf, N = raw.shape
            ref = ctx.magnitude(raw, apod)
            if dt == _lib.U16:
                dev = synthetic.u16_bits(torch.from_numpy(raw.astype(np.int32)).cuda())
            else:
                dev = torch.from_numpy(np.ascontiguousarray(raw)).cuda()
            out = torch.full((B, interf - apod, N // 2), float("nan"), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            rc = lib.octgb_magnitude_noalloc(ctx.h, ctypes.c_void_p(dev.data_ptr()), dt, B, interf, apod,
                                             ctypes.c_void_p(out.data_ptr()))
            assert rc == _lib.OK, lib.octgb_last_error(ctx.h)
            ctx.synchronize()
            assert np.abs(out.cpu().numpy() - ref).max() / np.abs(ref).max() < 2e-6
        # beyond the fixed scratch: a clear error, no work
        big = torch.zeros((65, interf, N), dtype=torch.int16, device="cuda")
        rc = lib.octgb_magnitude_noalloc(ctx.h, ctypes.c_void_p(big.data_ptr()), _lib.U16, 65, interf, apod,
                                         ctypes.c_void_p(out.data_ptr()))
        assert rc == _lib.ERR_ARG
        assert b"allocation-free limit" in lib.octgb_last_error(ctx.h)
    finally:
        ctx.close()
