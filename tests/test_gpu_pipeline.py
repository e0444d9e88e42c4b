"""GPU row reconstruction (spectral + optical-path correction + focus-weighted
stitching + finalise) on the reference's `telesto` format-test case, through
the package's own host path (geometry, tiled grids, stitch plans).

Criteria follow the reference's tests: NaN masks equal to the reference
float32 plane and, against the unmodified-MATLAB golden plane, mismatches only
at weight-threshold ties (tests/test_formats.py:174-180); accuracy no worse
than the reference float32 path (tests/test_torch_backend.py:63-71):
err <= 1.5 * err_ref32 + 1e-4 dB and < 1e-2 dB.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _build(t, ctx):
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300.reconstruct import RowReconstructor, RowTile
    sg = G.build_spectral_geometry(t["lambda_nm"], float(t["dispersion"]), float(t["n_medium"]))
    ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    lay = S.ScanLayout(t["x_centers_mm"], t["y_centers_mm"], t["z_depths_mm"], int(t["n_x_px"]), int(t["n_y_px"]),
                       float(t["tile_range_x_mm"]), float(t["tile_range_y_mm"]), float(t["x_offset"]),
                       float(t["y_offset"]))
    tg = S.tiled_geometry(lay, sg.z_um, t["focus_pix"], float(t["output_pixel_size_um"]))
    oc = S.OpticalPathCorrection.build(t["opc_poly"], tg.tile_x_mm, tg.tile_y_mm, tg.tile_z_mm)
    tiles = []
    for k, (xi, zi) in enumerate(zip(t["tile_xi"], t["tile_zi"])):
        st = S.TileStitcher.build(tg, t["x_centers_mm"][xi], t["z_depths_mm"][zi], t["focus_pix"][zi],
                                  float(t["focus_sigma"]))
        st.upload(ctx, oc)
        tiles.append(RowTile(st, lambda fr, k=k: t["raw"][k][np.asarray(fr)]))
    rr = RowReconstructor(ctx, int(t["apod_size"]), len(tg.out_z_mm), len(tg.out_x_mm), batch_frames=1)
    return rr, tiles


def test_telesto_plane_matches_reference(gpu_ctx, telesto):
    t = telesto
    rr, tiles = _build(t, gpu_ctx)
    planes, clims = rr.process_row(tiles, [0, 1], plane_clims=True)
    p = planes[int(t["plane_y"])].astype(float)
    ref32 = t["plane_fp32"].astype(float)
    ref64 = t["plane_fp64"].astype(float)
    m = t["matlab_plane"].astype(float)
    assert p.shape == ref32.shape
    assert np.array_equal(np.isfinite(p), np.isfinite(ref32))
    mism = np.isfinite(p) != np.isfinite(m)
    assert not np.any(mism & ~t["matlab_tie"])
    fin = np.isfinite(p) & np.isfinite(m) & np.isfinite(ref32)
    err = np.abs(p - m)[fin].max()
    err_ref = np.abs(ref32 - m)[fin].max()
    assert err <= 1.5 * err_ref + 1e-4, (err, err_ref)
    assert err < 1e-2
    assert np.abs(p - ref64)[fin].max() < 1e-2
    fp = p[np.isfinite(p)]
    assert clims[int(t["plane_y"])].tolist() == [float(fp.min()), float(fp.max())]


def test_batching_does_not_change_result(gpu_ctx, telesto):
    t = telesto
    rr, tiles = _build(t, gpu_ctx)
    a = rr.process_row(tiles, [0, 1])
    rr.batch = 2
    b = rr.process_row(tiles, [0, 1])
    np.testing.assert_array_equal(a, b)
    c = rr.process_row(tiles, [1])
    np.testing.assert_array_equal(c[0], a[1])


def test_frames_api_equals_row_api(gpu_ctx, telesto):
    """All tiles of a frame batch in one call (num/den on chip) give the same
    planes, NaN masks and clims as the per-tile accumulation."""
    t = telesto
    rr, tiles = _build(t, gpu_ctx)
    ref, ref_mm = rr.process_row(tiles, [0, 1], plane_clims=True)
    ids = [tile.stitcher.plan for tile in tiles]
    raws = [t["raw"][k][0:2] for k in range(len(tiles))]
    gpu_ctx.clim_reset()
    db, mm = gpu_ctx.frames_process(ids, raws, int(t["apod_size"]), 0, rr.n_out_z, rr.n_out_x, rr.threshold,
                                    plane_minmax=True)
    np.testing.assert_array_equal(db, ref)
    np.testing.assert_array_equal(mm, ref_mm)
    assert gpu_ctx.clim_get() == (float(np.nanmin(ref)), float(np.nanmax(ref)))
    # one frame at a time from frame 1 (optical-path rows follow f0)
    one = gpu_ctx.frames_process(ids, [t["raw"][k][1:2] for k in range(len(tiles))], int(t["apod_size"]), 1,
                                 rr.n_out_z, rr.n_out_x, rr.threshold)
    np.testing.assert_array_equal(one[0], ref[1])


def test_graph_capture_replays_frame_batch(gpu_ctx, telesto):
    torch = pytest.importorskip("torch")
    t = telesto
    rr, tiles = _build(t, gpu_ctx)
    ref = rr.process_row(tiles, [0, 1])
    ids = [tile.stitcher.plan for tile in tiles]
    raws = [torch.from_numpy(np.ascontiguousarray(t["raw"][k][0:2])).cuda() for k in range(len(tiles))]
    db = torch.empty((2, rr.n_out_z, rr.n_out_x), dtype=torch.float32, device="cuda")
    bits = torch.empty(db.shape, dtype=torch.int16, device="cuda")
    stream = torch.cuda.Stream()
    gpu_ctx.set_stream(stream.cuda_stream)
    try:
        def seq():
            gpu_ctx.clim_reset()
            gpu_ctx.frames_process(ids, raws, int(t["apod_size"]), 0, rr.n_out_z, rr.n_out_x, rr.threshold, out=db)
            gpu_ctx.quantise_running(db, bits)
        seq()                                   # sizes every buffer
        gpu_ctx.synchronize()
        db.fill_(0)
        torch.cuda.synchronize()
        gpu_ctx.graph_begin()
        seq()
        gid = gpu_ctx.graph_end()
        n0 = gpu_ctx.launches
        gpu_ctx.graph_launch(gid)
        gpu_ctx.synchronize()
        assert gpu_ctx.launches - n0 == 6       # clim init, apod, spectral, stitch, quant table, quantise
        np.testing.assert_array_equal(db.cpu().numpy(), ref)
        from oracle import numerics as O
        clim = (float(np.nanmin(ref)), float(np.nanmax(ref)))
        np.testing.assert_array_equal(bits.cpu().numpy().view(np.uint16), O.db_to_bits(ref, clim))
        # a new geometry would reallocate buffers the graph replays: refused
        # until the context's graphs are released
        from oct_recon_af_v1_gb300 import _lib
        from oct_recon_af_v1_gb300 import geometry as G
        sg = G.build_spectral_geometry(t["lambda_nm"], float(t["dispersion"]), float(t["n_medium"]))
        with pytest.raises(_lib.OctgbError) as e:
            gpu_ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
        assert e.value.code == _lib.ERR_STATE
        gpu_ctx.graphs_release()
        gpu_ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
        with pytest.raises(_lib.OctgbError):
            gpu_ctx.graph_launch(gid)
    finally:
        gpu_ctx.set_stream(None)
        gpu_ctx.graphs_release()


def test_frames_host_input_ring_matches_device_input(gpu_ctx):
    """Page-locked host raws go through the copy stream and the staging ring;
    consecutive batches (more than the ring holds) must equal the device path."""
    torch = pytest.importorskip("torch")
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300 import synthetic
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    gpu_ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    lay = S.ScanLayout(np.array([-0.0225, 0.0225]), np.array([0.0]), np.array([0.0, 0.05]), 50, 8, 0.05, 0.008)
    tg = S.tiled_geometry(lay, sg.z_um, [300.0, 320.0], 1.0)
    order = [(xi, zi) for xi in range(2) for zi in range(2)]
    ids = []
    for xi, zi in order:
        st = S.TileStitcher.build(tg, lay.x_centers_mm[xi], lay.z_depths_mm[zi], [300.0, 320.0][zi], 80.0)
        ids.append(st.upload(gpu_ctx))
    tiles = [synthetic.u16_bits(synthetic.generate(8, 50, 25, seed=40 + k)) for k in range(len(order))]
    host = [t.pin_memory() for t in tiles]
    dev = [t.cuda() for t in tiles]
    nz, nx = len(tg.out_z_mm), len(tg.out_x_mm)
    thr = S.min_weight_threshold(np.float32)
    out_h = torch.empty((8, nz, nx), dtype=torch.float32, device="cuda")
    out_d = torch.empty_like(out_h)
    for s0 in range(0, 8, 2):                          # 4 batches through a 3-slot ring
        gpu_ctx.frames_process(ids, [h[s0:s0 + 2] for h in host], 25, s0, nz, nx, thr, out=out_h[s0:s0 + 2],
                               raw_dtype=0)
    gpu_ctx.synchronize()
    for s0 in range(0, 8, 2):
        gpu_ctx.frames_process(ids, [d[s0:s0 + 2] for d in dev], 25, s0, nz, nx, thr, out=out_d[s0:s0 + 2],
                               raw_dtype=0)
    gpu_ctx.synchronize()
    a, b = out_h.cpu().numpy(), out_d.cpu().numpy()
    assert np.isfinite(a).any()
    np.testing.assert_array_equal(a, b)


def test_frames_stitch_rows_do_not_change_result(gpu_ctx):
    """The stitch kernel's tile shape (32, 64 or 128 output rows per block, the
    autotuner's choice) changes no voxel and no clim: every voxel sums the same
    tiles in the same order."""
    torch = pytest.importorskip("torch")
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300 import synthetic
    from oct_recon_af_v1_gb300._lib import OctgbError
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    gpu_ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    lay = S.ScanLayout(np.array([-0.0225, 0.0225]), np.array([0.0]), np.array([0.0, 0.05]), 50, 4, 0.05, 0.004)
    tg = S.tiled_geometry(lay, sg.z_um, [300.0, 320.0], 1.0)
    order = [(xi, zi) for xi in range(2) for zi in range(2)]
    ids = []
    for xi, zi in order:
        st = S.TileStitcher.build(tg, lay.x_centers_mm[xi], lay.z_depths_mm[zi], [300.0, 320.0][zi], 80.0)
        ids.append(st.upload(gpu_ctx))
    dev = [synthetic.u16_bits(synthetic.generate(4, 50, 25, seed=60 + k)).cuda() for k in range(len(order))]
    nz, nx = len(tg.out_z_mm), len(tg.out_x_mm)
    thr = S.min_weight_threshold(np.float32)
    outs, clims = {}, {}
    try:
        for rows in (64, 32, 128):
            gpu_ctx.set_stitch_rows(rows)
            out = torch.empty((4, nz, nx), dtype=torch.float32, device="cuda")
            gpu_ctx.clim_reset()
            gpu_ctx.frames_process(ids, dev, 25, 0, nz, nx, thr, out=out, raw_dtype=0)
            gpu_ctx.synchronize()
            outs[rows], clims[rows] = out.cpu().numpy(), gpu_ctx.clim_get()
        assert np.isfinite(outs[64]).any()
        for rows in (32, 128):
            np.testing.assert_array_equal(outs[rows], outs[64])
            assert clims[rows] == clims[64]
        with pytest.raises(OctgbError):
            gpu_ctx.set_stitch_rows(48)
    finally:
        gpu_ctx.set_stitch_rows(64)
