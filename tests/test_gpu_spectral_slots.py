"""The spectral kernel's static schedule: each CTA steps its A-scan slots by
the grid stride (whole B-scans plus A-scans, carried into the next B-scan and
the next tile) without division.  A-scans are independent, so a batch whose
quads straddle B-scans and tiles, with several quads per CTA, must give the
same bits as launches of one B-scan (one quad per CTA, no stepping).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _geometry(ctx):
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import synthetic
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    return sg


def test_magnitude_odd_bscan_width_equals_single_bscan_launches(gpu_ctx):
    from oct_recon_af_v1_gb300 import synthetic
    _geometry(gpu_ctx)
    # 40 B-scans x 37 A-scans: 370 quads, most spanning two B-scans, several per CTA
    raw = synthetic.generate_numpy(40, 37, 25, seed=71)
    full = gpu_ctx.magnitude(raw, 25)
    assert np.isfinite(full).all()
    for b in range(raw.shape[0]):
        np.testing.assert_array_equal(gpu_ctx.magnitude(raw[b:b + 1], 25)[0], full[b])


def test_frames_many_quads_per_cta_equal_single_frame_calls(gpu_ctx):
    """One 8-frame call over 4 tiles (400 quads: the slot steps cross B-scans
    and tiles) against eight 1-frame calls, through stitching and finalise."""
    torch = pytest.importorskip("torch")
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300 import synthetic
    sg = _geometry(gpu_ctx)
    lay = S.ScanLayout(np.array([-0.0225, 0.0225]), np.array([0.0]), np.array([0.0, 0.05]), 50, 8, 0.05, 0.008)
    tg = S.tiled_geometry(lay, sg.z_um, [300.0, 320.0], 1.0)
    order = [(xi, zi) for xi in range(2) for zi in range(2)]
    ids = []
    for xi, zi in order:
        st = S.TileStitcher.build(tg, lay.x_centers_mm[xi], lay.z_depths_mm[zi], [300.0, 320.0][zi], 80.0)
        ids.append(st.upload(gpu_ctx))
    dev = [synthetic.u16_bits(synthetic.generate(8, 50, 25, seed=80 + k)).cuda() for k in range(len(order))]
    nz, nx = len(tg.out_z_mm), len(tg.out_x_mm)
    thr = S.min_weight_threshold(np.float32)
    out_all = torch.empty((8, nz, nx), dtype=torch.float32, device="cuda")
    out_one = torch.empty_like(out_all)
    gpu_ctx.frames_process(ids, dev, 25, 0, nz, nx, thr, out=out_all, raw_dtype=0)
    for f in range(8):
        gpu_ctx.frames_process(ids, [d[f:f + 1] for d in dev], 25, f, nz, nx, thr, out=out_one[f:f + 1],
                               raw_dtype=0)
    gpu_ctx.synchronize()
    a, b = out_all.cpu().numpy(), out_one.cpu().numpy()
    assert np.isfinite(a).any()
    np.testing.assert_array_equal(a, b)
