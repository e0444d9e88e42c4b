"""Learned estimator, host side (no GPU): the float64 oracle network's
gradients against finite differences, the target encoding, and the plain
per-B-scan search on a scorer with known optima."""
from __future__ import annotations

import numpy as np

from oracle import cnn as C


def small_params(rng, in_ch=3, widths=(4, 5, 3, 4), img=32, hidden=6):
    chans = [in_ch, *widths]
    p = []
    for cin, cout in zip(chans[:-1], chans[1:]):
        p += [rng.standard_normal((cout, cin, 3, 3)) * 0.4, rng.standard_normal(cout) * 0.1]
    flat = widths[-1] * (img // 16) ** 2
    p += [rng.standard_normal((hidden, flat)) * 0.3, rng.standard_normal(hidden) * 0.1,
          rng.standard_normal((2, hidden)) * 0.3, rng.standard_normal(2) * 0.1]
    return p


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    params = small_params(rng)
    x = rng.standard_normal((2, 3, 32, 32))
    t = rng.standard_normal((2, 2))
    pred, cache = C.forward(params, x)
    _, dout = C.mse(pred, t)
    grads = C.backward(params, cache, dout)
    eps = 1e-6
    for pi in range(len(params)):
        flat = params[pi].reshape(-1)
        for j in rng.choice(flat.size, size=min(6, flat.size), replace=False):
            old = flat[j]
            flat[j] = old + eps
            lp, _ = C.mse(C.forward(params, x)[0], t)
            flat[j] = old - eps
            lm, _ = C.mse(C.forward(params, x)[0], t)
            flat[j] = old
            fd = (lp - lm) / (2 * eps)
            g = grads[pi].reshape(-1)[j]
            assert abs(fd - g) <= 1e-6 + 1e-5 * abs(fd), (pi, j, fd, g)


def test_targets_round_trip():
    from oct_recon_af_v1_gb300 import learned as L
    beta = np.array([-7e7, 0.0, 3.1e7])
    foc = np.array([100.0, 500.0, 900.0])
    b, f = L.decode(L.targets(beta, foc))
    np.testing.assert_allclose(b, beta, rtol=1e-6)
    np.testing.assert_allclose(f, foc, rtol=1e-6)


def test_per_bscan_search_finds_known_optima():
    from oct_recon_af_v1_gb300 import learned as L
    opt = np.array([-6.1e7, -1.23e6, 0.0, 4.4e7])

    class Quad:
        def scores(self, beta, idx=None):
            o = opt if idx is None else opt[idx:idx + 1]
            return -((beta - o) / 1e7) ** 2

        def scores_grid(self, betas, idx=None):
            return np.stack([self.scores(b, idx) for b in betas])

    got, grid, S = L.search_per_bscan(Quad(), -8e7, 8e7, 41)
    assert S.shape == (41, 4)
    # the zoom stops at candidates 2e-5 x 8e7 apart; the parabolic step lands
    # on a quadratic's vertex
    np.testing.assert_allclose(got, opt, rtol=0, atol=1.0)
