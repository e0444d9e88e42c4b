"""Batched form: many tiles of uneven size in one persistent launch fed by a
device work queue (octgb_batch_process).

Each tile is a single-tile reconstruction (TileStitcher of one tile: depth
resampling to the output grid with its focus weight, identity lateral
operator, octrecon/core/stitching.py:84-139, then finalise).  The result must
equal the frame-batch path on the same tile bit for bit, for any queue grab,
also when replayed from a CUDA graph, and stay close to the oracle.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import numerics as O

pytestmark = pytest.mark.gpu


def _tiles(ctx, torch, specs, seed=0):
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300 import synthetic
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    out = []
    for k, (B, nx, crop, focus) in enumerate(specs):
        lay = S.ScanLayout(np.array([0.0]), np.array([0.0]), np.array([0.0]), nx, B, nx * 1e-3, B * 1e-3)
        tg = S.tiled_geometry(lay, sg.z_um, [focus], 1.0, crop)
        st = S.TileStitcher.build(tg, 0.0, 0.0, focus, 80.0)
        plan = st.upload(ctx)
        raw = synthetic.u16_bits(synthetic.generate(B, nx, 25, seed=seed + k, device="cuda"))
        db = torch.full((B, nx, len(tg.out_z_mm)), -1.0, dtype=torch.float32, device="cuda")
        out.append(dict(raw=raw, plan=plan, db=db, st=st, tg=tg, nx=nx, B=B))
    return sg, out


SPECS = [(3, 37, (-0.1, 0.3), 300.0), (1, 50, (0.0, 0.6), 500.0), (5, 13, (-0.3, 0.9), 200.0),
         (2, 64, None, 400.0), (4, 21, (0.2, 0.5), 600.0)]


def test_batch_equals_frame_path_and_oracle(gpu_ctx):
    torch = pytest.importorskip("torch")
    from oct_recon_af_v1_gb300 import stitching as S
    sg, tiles = _tiles(gpu_ctx, torch, SPECS)
    thr = S.min_weight_threshold(np.float32)
    work = [(t["raw"], 25, t["plan"], t["db"]) for t in tiles]
    gpu_ctx.clim_reset()
    gpu_ctx.batch_process(work, thr, grab=4)
    gpu_ctx.synchronize()
    got = [t["db"].cpu().numpy().copy() for t in tiles]
    clim = gpu_ctx.clim_get()
    fin = np.concatenate([g[np.isfinite(g)] for g in got])
    assert clim == (float(fin.min()), float(fin.max()))
    for t, g in zip(tiles, got):
        nz = g.shape[-1]
        # frame-batch path on the same tile: planes (B, nz, nx)
        ref = gpu_ctx.frames_process([t["plan"]], [t["raw"]], 25, 0, nz, t["nx"], thr)
        np.testing.assert_array_equal(g, ref.transpose(0, 2, 1))
    # different queue grabs and a graph replay give the same bits
    for grab in (1, 3, 64):
        for t in tiles:
            t["db"].fill_(-1.0)
        gpu_ctx.batch_process(work, thr, grab=grab)
        gpu_ctx.synchronize()
        for t, g in zip(tiles, got):
            np.testing.assert_array_equal(t["db"].cpu().numpy(), g)
    stream = torch.cuda.Stream()
    gpu_ctx.set_stream(stream.cuda_stream)
    try:
        gpu_ctx.batch_process(work, thr, grab=4)
        gpu_ctx.synchronize()
        for t in tiles:
            t["db"].fill_(-1.0)
        torch.cuda.synchronize()
        gpu_ctx.graph_begin()
        gpu_ctx.batch_process(work, thr, grab=4)
        gid = gpu_ctx.graph_end()
        gpu_ctx.graph_launch(gid)
        gpu_ctx.synchronize()
        for t, g in zip(tiles, got):
            np.testing.assert_array_equal(t["db"].cpu().numpy(), g)
    finally:
        gpu_ctx.set_stream(None)
        gpu_ctx.graphs_release()


def test_batch_close_to_oracle(gpu_ctx):
    torch = pytest.importorskip("torch")
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300 import synthetic
    sg, tiles = _tiles(gpu_ctx, torch, SPECS[:3], seed=50)
    thr = S.min_weight_threshold(np.float32)
    gpu_ctx.batch_process([(t["raw"], 25, t["plan"], t["db"]) for t in tiles], thr, grab=2)
    gpu_ctx.synchronize()
    og = O.spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    for t in tiles:
        raw = t["raw"].cpu().numpy().view(np.uint16)
        mag = O.magnitude_numba(raw, og, 25)
        st = t["st"]
        stn = O.Stitcher.__new__(O.Stitcher)
        stn.r0, stn.r1, stn.c0, stn.c1 = st.r0, st.r1, st.c0, st.c1
        stn.Wz, stn.WxT, stn.fz, stn.dtype = st.Wz, st.WxT, st.fz, np.float32
        num, den = stn.contribute(mag)
        ref = O.finalise(num, den)                     # (B, nz, nx)
        got = t["db"].cpu().numpy().transpose(0, 2, 1)
        assert np.array_equal(np.isfinite(got), np.isfinite(ref))
        fin = np.isfinite(ref)
        # float32 spectra of two FFTs: dB agree within a few 1e-3 except at deep nulls
        err = np.abs(got[fin] - ref[fin])
        assert np.quantile(err, 0.999) < 5e-3 and err.max() < 0.5


def test_graph_replay_survives_other_batches(gpu_ctx):
    """A graph captured over a batch keeps replaying that batch after other
    batches (single tiles, a larger raw batch) ran on the same context: its
    tile table and buffers are never overwritten or freed under it."""
    torch = pytest.importorskip("torch")
    from oct_recon_af_v1_gb300 import stitching as S
    sg, tiles = _tiles(gpu_ctx, torch, SPECS, seed=80)
    thr = S.min_weight_threshold(np.float32)
    work = [(t["raw"], 25, t["plan"], t["db"]) for t in tiles]
    stream = torch.cuda.Stream()
    gpu_ctx.set_stream(stream.cuda_stream)
    try:
        gpu_ctx.batch_process(work, thr, grab=4)
        gpu_ctx.synchronize()
        got = [t["db"].cpu().numpy().copy() for t in tiles]
        gpu_ctx.graph_begin()
        gpu_ctx.batch_process(work, thr, grab=4)
        gid = gpu_ctx.graph_end()
        # more distinct tables than the context keeps unpinned, and a batch
        # with more apodisation rows than the captured one (the apod buffer grows)
        for rep in range(3):
            for w in work:
                gpu_ctx.batch_process([w], thr, grab=1 + rep)
            gpu_ctx.batch_process(work[::-1], thr, grab=2)
            gpu_ctx.batch_process(work + work[:2], thr, grab=3)
        gpu_ctx.synchronize()
        for t in tiles:
            t["db"].fill_(-1.0)
        torch.cuda.synchronize()
        gpu_ctx.graph_launch(gid)
        gpu_ctx.synchronize()
        for t, g in zip(tiles, got):
            np.testing.assert_array_equal(t["db"].cpu().numpy(), g)
    finally:
        gpu_ctx.set_stream(None)
        gpu_ctx.graphs_release()
