"""Learned estimator kernels on the GPU against the float64 oracle network:
convolution forward on ragged shapes, every parameter gradient of the whole
network, the Adam step, the probe images against a NumPy pooling of the
scorer's magnitudes, a short training run that lowers the loss, and what a
trained network gains over reconstructing without an estimate."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import cnn as C
from test_learned_host import small_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oct_recon_af_v1_gb300 as pkg
    pkg.build()
    from oct_recon_af_v1_gb300._lib import Context
    ctx = Context(0)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    yield torch, ctx
    ctx.close()


def test_conv_forward_ragged_shapes(torch_ctx):
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import _p
    rng = np.random.default_rng(1)
    for n, cin, cout, h, w in ((2, 3, 16, 32, 32), (1, 11, 21, 20, 37), (3, 1, 5, 7, 5), (2, 32, 32, 16, 16)):
        x = rng.standard_normal((n, cin, h, w))
        wt = rng.standard_normal((cout, cin, 3, 3))
        b = rng.standard_normal(cout)
        ref = C.conv3x3(x, wt, b)
        xd, wd, bd = (torch.tensor(a, dtype=torch.float32, device="cuda") for a in (x, wt, b))
        y = torch.empty((n, cout, h, w), dtype=torch.float32, device="cuda")
        ctx._check(ctx.lib.octgb_cnn_conv3x3(ctx.h, _p(xd), _p(wd), _p(bd), _p(y), n, cin, cout, h, w))
        torch.cuda.synchronize()
        np.testing.assert_allclose(y.cpu().numpy(), ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())


def _fp16(a):
    return np.asarray(a, np.float32).astype(np.float16).astype(np.float64)


def test_conv_tensor_cores_match_fp16_operands(torch_ctx):
    """The tcgen05 convolution equals the float64 convolution of the
    FP16-rounded operands (float32 accumulation: relative 1e-5), and the
    float32 kernel within the operands' rounding, on every shape the network
    uses and on ragged ones (edges, multi-row tiles, partial channel chunks)."""
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import BetaFocusNet, _p
    rng = np.random.default_rng(5)
    for n, cin, cout, h, w in ((2, 3, 32, 256, 256), (2, 32, 32, 128, 128), (3, 32, 32, 64, 64),
                               (3, 32, 32, 32, 32), (1, 11, 64, 16, 16), (2, 32, 96, 8, 384), (1, 1, 32, 128, 1)):
        assert BetaFocusNet.tc_supported(cin, cout, h, w)
        x = rng.standard_normal((n, cin, h, w)).astype(np.float32)
        wt = (rng.standard_normal((cout, cin, 3, 3)) * 0.3).astype(np.float32)
        b = rng.standard_normal(cout).astype(np.float32)
        ref16 = C.conv3x3(_fp16(x), _fp16(wt), b.astype(np.float64))
        xd, wd, bd = (torch.tensor(a, device="cuda") for a in (x, wt, b))
        y = torch.empty((n, cout, h, w), dtype=torch.float32, device="cuda")
        ctx._check(ctx.lib.octgb_cnn_conv3x3_tc(ctx.h, _p(xd), _p(wd), _p(bd), _p(y), n, cin, cout, h, w))
        y32 = torch.empty_like(y)
        ctx._check(ctx.lib.octgb_cnn_conv3x3(ctx.h, _p(xd), _p(wd), _p(bd), _p(y32), n, cin, cout, h, w))
        ctx.synchronize()
        got = y.cpu().numpy()
        scale = np.abs(ref16).max()
        np.testing.assert_allclose(got, ref16, rtol=0, atol=1e-5 * scale * np.sqrt(cin * 9))
        assert np.abs(got - y32.cpu().numpy()).max() < 2e-3 * scale, (cin, cout, h, w)
    from oct_recon_af_v1_gb300._lib import OctgbError
    with pytest.raises(OctgbError):
        ctx._check(ctx.lib.octgb_cnn_conv3x3_tc(ctx.h, _p(xd), _p(wd), _p(bd), _p(y), 1, 33, 32, 32, 32))


def test_conv_relu_pool_tensor_cores(torch_ctx):
    """The fused tensor-core convolution + ReLU + 2x2 mean equals the oracle's
    ReLU-pool of the float64 convolution of the FP16-rounded operands."""
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import _p
    rng = np.random.default_rng(6)
    for n, cin, cout, h, w in ((2, 3, 32, 256, 256), (2, 32, 32, 128, 128), (1, 5, 64, 6, 256)):
        x = rng.standard_normal((n, cin, h, w)).astype(np.float32)
        wt = (rng.standard_normal((cout, cin, 3, 3)) * 0.3).astype(np.float32)
        b = rng.standard_normal(cout).astype(np.float32)
        pre = C.conv3x3(_fp16(x), _fp16(wt), b.astype(np.float64))
        ref = np.maximum(pre, 0).reshape(n, cout, h // 2, 2, w // 2, 2).mean(axis=(3, 5))
        xd, wd, bd = (torch.tensor(a, device="cuda") for a in (x, wt, b))
        p = torch.empty((n, cout, h // 2, w // 2), dtype=torch.float32, device="cuda")
        ctx._check(ctx.lib.octgb_cnn_conv3x3_relu_pool_tc(ctx.h, _p(xd), _p(wd), _p(bd), _p(p), n, cin, cout, h, w))
        ctx.synchronize()
        np.testing.assert_allclose(p.cpu().numpy(), ref, rtol=0, atol=1e-5 * np.abs(pre).max() * np.sqrt(cin * 9))


def _bf16(a):
    """float32 -> BF16 (round to nearest even) -> float64."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _wgrad_ref(x, dy):
    """dw (K, C, 3, 3) and sum |dy| |x| per element, float64, as matrix products per tap."""
    n, C, H, W = x.shape
    K = dy.shape[1]
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    d2 = dy.transpose(1, 0, 2, 3).reshape(K, -1)
    dw, mag = np.zeros((K, C, 3, 3)), np.zeros((K, C, 3, 3))
    for i in range(3):
        for j in range(3):
            xs = xp[:, :, i:i + H, j:j + W].transpose(1, 0, 2, 3).reshape(C, -1)
            dw[:, :, i, j] = d2 @ xs.T
            mag[:, :, i, j] = np.abs(d2) @ np.abs(xs).T
    return dw, mag


def test_conv_grad_tensor_cores_match_bf16_operands(torch_ctx):
    """The tcgen05 weight gradient equals the float64 sum of the BF16-rounded
    operands' products within float32 accumulation (1e-4 of the sum of the
    products' magnitudes), on the network's shapes and ragged ones (widths not
    a multiple of 8, channel counts off the MMA sizes, one-row bands); the
    data gradient (BF16 tensor-core convolution with the flipped kernel) the
    float64 one of the rounded operands; db the float64 sum of dy."""
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import BetaFocusNet, _p
    rng = np.random.default_rng(8)
    for n, cin, cout, h, w in ((2, 3, 32, 256, 256), (2, 32, 32, 128, 128), (3, 32, 32, 64, 64),
                               (4, 32, 32, 32, 32), (1, 11, 21, 20, 37), (2, 5, 7, 9, 13), (1, 48, 128, 16, 16),
                               (2, 1, 1, 7, 5), (1, 16, 40, 3, 700), (2, 8, 16, 6, 30)):
        x = rng.standard_normal((n, cin, h, w)).astype(np.float32)
        wt = (rng.standard_normal((cout, cin, 3, 3)) * 0.3).astype(np.float32)
        dy = (rng.standard_normal((n, cout, h, w)) * 1e-6).astype(np.float32)   # gradients: small magnitudes
        ref_dw, mag = _wgrad_ref(_bf16(x), _bf16(dy))
        xd, wd, dyd = (torch.tensor(a, device="cuda") for a in (x, wt, dy))
        dw = torch.full((cout, cin, 3, 3), float("nan"), device="cuda")
        db = torch.empty(cout, device="cuda")
        dx = torch.empty((n, cin, h, w), device="cuda")
        scratch = torch.empty(cout * cin * 9, device="cuda")
        ctx._check(ctx.lib.octgb_cnn_conv3x3_bwd_tc(ctx.h, _p(xd), _p(wd), _p(dyd), _p(dx), _p(dw), _p(db),
                                                    _p(scratch), n, cin, cout, h, w))
        ctx.synchronize()
        got = dw.cpu().numpy().astype(np.float64)
        assert np.isfinite(got).all(), (cin, cout, h, w)
        err = np.abs(got - ref_dw)
        assert (err <= 1e-4 * mag + 1e-30).all(), (cin, cout, h, w, float((err / (mag + 1e-30)).max()))
        np.testing.assert_allclose(db.cpu().numpy(), dy.astype(np.float64).sum(axis=(0, 2, 3)), rtol=1e-4,
                                   atol=1e-4 * np.abs(dy).sum(axis=(0, 2, 3)).max())
        # dx: BF16 tensor cores where the convolution cout -> cin is a supported shape, else float32
        wf = np.flip(wt, (2, 3)).transpose(1, 0, 2, 3)              # (cin, cout, 3, 3)
        tc = BetaFocusNet.tc_supported(cout, cin, h, w)
        ref_dx = C.conv3x3(_bf16(dy) if tc else dy.astype(np.float64), _bf16(wf) if tc else wf.astype(np.float64),
                           np.zeros(cin))
        scale = np.abs(ref_dx).max()
        np.testing.assert_allclose(dx.cpu().numpy(), ref_dx, rtol=0, atol=1e-5 * scale * np.sqrt(cout * 9))
    from oct_recon_af_v1_gb300._lib import OctgbError
    with pytest.raises(OctgbError):
        ctx._check(ctx.lib.octgb_cnn_conv3x3_bwd_tc(ctx.h, _p(xd), _p(wd), _p(dyd), None, _p(dw), _p(db), None,
                                                    1, 49, 32, 8, 8))


def test_network_gradients_match_oracle(torch_ctx):
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import BetaFocusNet
    rng = np.random.default_rng(2)
    widths, img, hidden = (4, 5, 3, 4), 32, 6
    params = small_params(rng, widths=widths, img=img, hidden=hidden)
    net = BetaFocusNet(ctx, in_ch=3, widths=widths, img=img, hidden=hidden)
    for dst, src in zip(net.params, params):
        dst.copy_(torch.tensor(src, dtype=torch.float32))
    x = rng.standard_normal((3, 3, img, img))
    t = rng.standard_normal((3, 2)) * 0.5
    ref_pred, cache = C.forward(params, x)
    ref_loss, dout = C.mse(ref_pred, t)
    ref_grads = C.backward(params, cache, dout)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    td = torch.tensor(t, dtype=torch.float32, device="cuda")
    pred = net.forward(xd)
    loss, dout_d = net.loss_grad(pred, td)
    net.backward(dout_d)
    torch.cuda.synchronize()
    np.testing.assert_allclose(pred.cpu().numpy(), ref_pred, rtol=1e-4, atol=1e-5)
    assert float(loss.item()) == pytest.approx(ref_loss, rel=1e-4)
    for i, (g, r) in enumerate(zip(net.grads, ref_grads)):
        got = g.cpu().numpy().astype(float)
        err = np.abs(got - r).max() / max(np.abs(r).max(), 1e-12)
        assert err < 2e-4, (i, err)


def test_network_gradients_tensor_cores(torch_ctx):
    """Training on the tensor cores (FP16 forward, BF16 gradients) on a
    network whose layers take every path (tensor-core forward at widths 64 ..
    16, float32 forward at 8; tensor-core weight and data gradients): every
    parameter gradient within 3 % of the largest of the float64 oracle's."""
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import BetaFocusNet
    rng = np.random.default_rng(12)
    widths, img, hidden = (32, 32, 32, 32), 64, 16
    params = small_params(rng, widths=widths, img=img, hidden=hidden)
    net = BetaFocusNet(ctx, in_ch=3, widths=widths, img=img, hidden=hidden, train_tensor_cores=True)
    for dst, src in zip(net.params, params):
        dst.copy_(torch.tensor(src, dtype=torch.float32))
    x = rng.standard_normal((4, 3, img, img))
    t = rng.standard_normal((4, 2)) * 0.5
    ref_pred, cache = C.forward(params, x)
    _, dout = C.mse(ref_pred, t)
    ref_grads = C.backward(params, cache, dout)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    td = torch.tensor(t, dtype=torch.float32, device="cuda")
    pred = net.forward(xd, tensor_cores=True, fuse_pool=False)
    _, dout_d = net.loss_grad(pred, td)
    net.backward(dout_d)
    torch.cuda.synchronize()
    np.testing.assert_allclose(pred.cpu().numpy(), ref_pred, rtol=0, atol=1e-2 * np.abs(ref_pred).max())
    for i, (g, r) in enumerate(zip(net.grads, ref_grads)):
        got = g.cpu().numpy().astype(float)
        err = np.abs(got - r).max() / max(np.abs(r).max(), 1e-12)
        assert err < 3e-2, (i, err)


def test_adam_step_matches_formula(torch_ctx):
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import _p
    rng = np.random.default_rng(3)
    n = 1000
    p, g, m, v = (rng.standard_normal(n) for _ in range(4))
    v = np.abs(v)
    pd, gd, md, vd = (torch.tensor(a, dtype=torch.float32, device="cuda") for a in (p, g, m, v))
    lr, b1, b2, eps, step = 1e-3, 0.9, 0.999, 1e-8, 7
    ctx._check(ctx.lib.octgb_cnn_adam(ctx.h, _p(pd), _p(gd), _p(md), _p(vd), n, lr, b1, b2, eps, step))
    torch.cuda.synchronize()
    m2 = b1 * m + (1 - b1) * g
    v2 = b2 * v + (1 - b2) * g * g
    p2 = p - lr * (m2 / (1 - b1 ** step)) / (np.sqrt(v2 / (1 - b2 ** step)) + eps)
    np.testing.assert_allclose(md.cpu().numpy(), m2, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(vd.cpu().numpy(), v2, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(pd.cpu().numpy(), p2, rtol=1e-5, atol=1e-6)


def adaptive_pool_db(mag, z_keep, img=256):
    """NumPy adaptive average pooling (B, nX, nZ) -> (B, img(z), img(x)) dB."""
    B, nx, _ = mag.shape
    out = np.empty((B, img, img))
    for zi in range(img):
        z0, z1 = zi * z_keep // img, -(-(zi + 1) * z_keep // img)
        for xi in range(img):
            x0, x1 = xi * nx // img, -(-(xi + 1) * nx // img)
            out[:, zi, xi] = mag[:, x0:x1, z0:z1].astype(np.float64).mean(axis=(1, 2))
    return 20 * np.log10(out)


def test_probe_images_match_numpy(torch_ctx):
    torch, _ = torch_ctx
    from oct_recon_af_v1_gb300 import learned as L
    from oct_recon_af_v1_gb300 import synthetic as S
    from oct_recon_af_v1_gb300.estimation import DispersionScorer
    raw = S.generate(2, 300, 25, seed=4, device="cuda", beta_px=np.array([2e-5, -4e-5]),
                     focus_px=np.array([300.0, 700.0]))
    raw16 = S.u16_bits(raw)
    mk = L.ImageMaker(S.lambda_nm(), 25)
    try:
        imgs = mk.images(raw16, raw_dtype=0).cpu().numpy()
    finally:
        mk.close()
    sc = DispersionScorer(S.lambda_nm(), raw16, "top_percentile", 25, rep=1, raw_dtype=0)
    try:
        ref = np.stack([adaptive_pool_db(sc.magnitude(b), L.Z_KEEP) for b in L.probe_betas()], 1)   # (B, P, z, x)
    finally:
        sc.close()
    ref = (ref - ref.mean(axis=(1, 2, 3), keepdims=True)) / ref.std(axis=(1, 2, 3), keepdims=True)
    np.testing.assert_allclose(imgs, ref, rtol=0, atol=2e-4)


@pytest.mark.parametrize("tensor_cores", [False, True])
def test_training_lowers_loss(torch_ctx, tensor_cores):
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import BetaFocusNet
    widths = (32, 32, 32, 32) if tensor_cores else (8, 8, 8, 8)
    net = BetaFocusNet(ctx, in_ch=3, widths=widths, img=64, hidden=16, seed=1, train_tensor_cores=tensor_cores)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn((16, 3, 64, 64), device="cuda", generator=g)
    t = torch.stack([x[:, 0].mean((1, 2)) * 3, x[:, 1, :32].mean((1, 2)) * 3], -1).contiguous()
    first = float(net.train_step(x, t, 1e-3).item())
    for _ in range(200):
        loss = net.train_step(x, t, 1e-3)
    assert float(loss.item()) < 0.2 * first


def test_trained_network_gains_over_no_estimator(torch_ctx):
    """A network trained briefly on probe images of dispersion-free B-scans
    re-rendered at random dispersions (the scorer's phase trick) predicts,
    on held-out B-scans carrying the dispersion in their spectra, a beta whose
    sharpness is far closer to the searched optimum than reconstructing
    without an estimate (beta = 0), and a focus closer than a constant guess."""
    torch, _ = torch_ctx
    from oct_recon_af_v1_gb300 import learned as L
    from oct_recon_af_v1_gb300 import synthetic as S
    from oct_recon_af_v1_gb300._lib import U16, Context
    from oct_recon_af_v1_gb300.estimation import DispersionScorer
    rng = np.random.default_rng(21)
    lam = S.lambda_nm()
    mk = L.ImageMaker(lam, 25)
    net_ctx = Context(0)
    try:
        n_base, shifts, nx = 160, 8, 256
        X = torch.empty((n_base * shifts, 3, L.IMG, L.IMG), dtype=torch.float32, device="cuda")
        Y = np.empty((n_base * shifts, 2), np.float32)
        foc = rng.uniform(100, 900, n_base)
        k = 0
        for c0 in range(0, n_base, 40):
            raw = S.u16_bits(S.generate(40, nx, 25, seed=500 + c0, device="cuda", beta_px=0.0,
                                        focus_px=foc[c0:c0 + 40], chunk=40, precision="float32"))
            mk.load(raw, raw_dtype=U16)
            for _ in range(shifts):
                bc = -S.beta_ref_from_px(rng.uniform(-5e-5, 5e-5))
                mk.render(bc, out=X[k:k + 40])
                Y[k:k + 40] = L.targets(np.full(40, bc), foc[c0:c0 + 40])
                k += 40
        Yd = torch.tensor(Y, device="cuda")
        net = L.BetaFocusNet(net_ctx, seed=3)
        n, bs, steps = len(Y), 64, 600
        for it in range(steps):
            idx = torch.randint(0, n, (bs,), device="cuda")
            lr = 1e-5 + 0.5 * (2e-3 - 1e-5) * (1 + np.cos(np.pi * it / steps))
            net.train_step(X.index_select(0, idx), Yd.index_select(0, idx), float(lr))
        del X
        n_test = 24
        bpx = rng.uniform(-5e-5, 5e-5, n_test)
        ft = rng.uniform(100, 900, n_test)
        raw_t = S.u16_bits(S.generate(n_test, nx, 25, seed=999, device="cuda", beta_px=bpx, focus_px=ft,
                                      chunk=n_test, precision="float32"))
        imgs_t = mk.images(raw_t, raw_dtype=U16)
        pred32 = net.forward(imgs_t).cpu().numpy()
        pred_tc = net.predict(imgs_t).cpu().numpy()
        # the tensor-core forward (FP16 operands) stays close to the float32 one
        assert np.abs(pred_tc - pred32).max() < 0.02 * max(1.0, np.abs(pred32).max()), np.abs(pred_tc - pred32).max()
        beta_l, focus_l = L.decode(pred_tc)
        sc = DispersionScorer(lam, raw_t, "top_percentile", 25, rep=1, raw_dtype=U16)
        try:
            beta_s, grid, Sg = L.search_per_bscan(sc, -1.2 * L.beta_scale(), 1.2 * L.beta_scale(), 41)
            rng_j = Sg.max(0) - Sg.min(0)
            s = lambda b: np.array([sc.scores(b[j], j)[0] for j in range(n_test)])
            s_search, s_learn, s_none = s(beta_s), s(beta_l), s(np.zeros(n_test))
        finally:
            sc.close()
        gap_learn = (s_search - s_learn) / rng_j
        gap_none = (s_search - s_none) / rng_j
        print(f"sharpness gap to the search: learned {gap_learn.mean():.4f}, beta=0 {gap_none.mean():.4f}; "
              f"focus MAE learned {np.mean(np.abs(focus_l - ft)):.1f} px, constant {np.mean(np.abs(500 - ft)):.1f} px")
        assert gap_learn.mean() < 0.25 * gap_none.mean()
        assert np.mean(gap_learn) < 0.03
        assert np.mean(np.abs(focus_l - ft)) < 0.5 * np.mean(np.abs(500 - ft))
    finally:
        mk.close()
        net_ctx.close()


def test_fused_probe_images_match_magnitude_path(torch_ctx):
    """octgb_disp_images (depth pooling inside the dispersion kernel, then over
    A-scans) against the two-step path (octgb_disp_eval magnitudes, then
    octgb_cnn_images) with B-scan repeats averaged (rep 2) and a width that is
    not a multiple of 256: the same images up to float32 summation order."""
    torch, _ = torch_ctx
    from oct_recon_af_v1_gb300 import learned as L
    from oct_recon_af_v1_gb300 import synthetic as S
    from oct_recon_af_v1_gb300._lib import U16
    from oct_recon_af_v1_gb300.estimation import hann_rms
    from oct_recon_af_v1_gb300.learned import _p
    mk = L.ImageMaker(S.lambda_nm(), 25)
    try:
        nb, rep, nx = 3, 2, 300
        raw = S.u16_bits(S.generate(nb * rep, nx, 25, seed=33, device="cuda", beta_px=2e-5, focus_px=500.0,
                                    chunk=nb * rep, precision="float32"))
        ctx = mk.ctx
        ctx.disp_load(raw, 25, nb, rep, hann_rms(2048), raw_dtype=U16)
        betas = np.array([-3e6, 0.0, 4e6])
        fused = torch.empty((nb, 3, L.IMG, L.IMG), dtype=torch.float32, device="cuda")
        ctx._check(ctx.lib.octgb_disp_images(ctx.h, 3, betas.ctypes.data, 0, nb, L.Z_KEEP, _p(fused), 0))
        mag = torch.empty((3, nb, nx, 1024), dtype=torch.float32, device="cuda")
        ctx.disp_eval(betas, 0, nb, 0, mag=mag)
        ref = torch.empty_like(fused)
        ctx._check(ctx.lib.octgb_cnn_images(ctx.h, _p(mag), 3, nb, nx, L.Z_KEEP, _p(ref), 0))
        ctx.synchronize()
        np.testing.assert_allclose(fused.cpu().numpy(), ref.cpu().numpy(), rtol=0, atol=1e-4)
    finally:
        mk.close()


def test_dense_split_k_matches_float64(torch_ctx):
    """The dense layer over 8192 flattened features (split K across the SMs,
    slices summed in a fixed order) against float64, and bit-identical run to run."""
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import _p
    rng = np.random.default_rng(9)
    m, k, n = 300, 8192, 64
    x = rng.standard_normal((m, k)).astype(np.float32)
    w = (rng.standard_normal((n, k)) / np.sqrt(k)).astype(np.float32)
    b = rng.standard_normal(n).astype(np.float32)
    xd, wd, bd = (torch.tensor(a, device="cuda") for a in (x, w, b))
    pre = torch.empty((m, n), device="cuda")
    act = torch.empty((m, n), device="cuda")
    ctx._check(ctx.lib.octgb_cnn_dense(ctx.h, _p(xd), _p(wd), _p(bd), _p(pre), _p(act), m, k, n))
    first = pre.clone()
    ctx._check(ctx.lib.octgb_cnn_dense(ctx.h, _p(xd), _p(wd), _p(bd), _p(pre), _p(act), m, k, n))
    ctx.synchronize()
    ref = x.astype(np.float64) @ w.astype(np.float64).T + b
    np.testing.assert_allclose(pre.cpu().numpy(), ref, rtol=0, atol=2e-5 * np.abs(ref).max())
    np.testing.assert_array_equal(act.cpu().numpy(), np.maximum(pre.cpu().numpy(), 0))
    assert torch.equal(first, pre)
