"""Learned estimator kernels on the GPU against the float64 oracle network:
convolution forward on ragged shapes, every parameter gradient of the whole
network, the Adam step, the probe images against a NumPy pooling of the
scorer's magnitudes, and a short training run that lowers the loss."""
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


def test_training_lowers_loss(torch_ctx):
    torch, ctx = torch_ctx
    from oct_recon_af_v1_gb300.learned import BetaFocusNet
    net = BetaFocusNet(ctx, in_ch=3, widths=(8, 8, 8, 8), img=64, hidden=16, seed=1)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn((16, 3, 64, 64), device="cuda", generator=g)
    t = torch.stack([x[:, 0].mean((1, 2)) * 3, x[:, 1, :32].mean((1, 2)) * 3], -1).contiguous()
    first = float(net.train_step(x, t, 1e-3).item())
    for _ in range(200):
        loss = net.train_step(x, t, 1e-3)
    assert float(loss.item()) < 0.2 * first
