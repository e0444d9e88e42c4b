"""Learned beta/focus estimator on the GB300 kernels.

The reference estimates the dispersion term and the focus by searches
(octrecon/estimation/dispersion.py:154-267, focus.py:191-218).  This module
adds a small CNN that predicts both from a B-scan in one forward pass, and
keeps the searches as its judge.

Input image of a B-scan: the scorer's trick (dispersion.py:17-20) - linearise
and Hann/rms-window once, then |ifft| at three probe dispersions (-p, 0, +p);
each is block-averaged to 256 x 256 (depth rows x A-scan columns, adaptive
average pooling of the magnitude, then 20 log10, as the preview's
block-average, estimation/preview.py:49-53) and the three channels of an
image are standardised together.  The magnitude of one reconstruction does
not reveal the sign of the residual dispersion; the +-p probes do.

Network (NCHW float32): 4 x [conv 3x3 (pad 1) -> ReLU -> 2x2 mean pool]
of 32 channels each, then dense 8192 -> 64 -> ReLU -> 2.  Outputs:
beta / BETA_SCALE and (focus - 500) / 400.  Every layer, its gradients, the
loss and Adam run in hand-written kernels (csrc/cnn.cu) through the C ABI;
torch only allocates the tensors.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import estimation as E
from . import geometry as G
from . import synthetic as S
from ._lib import Context

IMG = 256
Z_KEEP = 1000                  # depth bins kept (the crop of the spectrum model's workload)
FOCUS_CENTER, FOCUS_SCALE = 500.0, 400.0


def beta_scale() -> float:
    """Reference units (nm^2/rad) of beta_px = 5e-5, the training range's edge."""
    return S.beta_ref_from_px(5e-5)


def probe_betas(p_px: float = 3e-5):
    b = S.beta_ref_from_px(p_px)
    return np.array([-b, 0.0, b])


def _p(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


class ImageMaker:
    """Probe images of raw B-scans on the device (see the module docstring)."""

    def __init__(self, lambda_nm, apod_size: int, device: int = 0, probes=None):
        import torch
        self.torch = torch
        lam = np.asarray(lambda_nm, float)
        sg = G.build_spectral_geometry(lam, 0.0, 1.33)
        self.n = len(lam)
        self.apod = int(apod_size)
        self.ctx = Context(device)
        self.ctx.set_geometry(sg.sinc_idx, sg.sinc_w, np.ones(self.n, np.complex128))
        k_eq = 2 * np.pi / sg.lambda_eq_nm
        self.ctx.disp_set_dk2((k_eq - k_eq.mean()) ** 2)
        self.hann = E.hann_rms(self.n)
        self.probes = probe_betas() if probes is None else np.asarray(probes, float)

    def close(self):
        self.ctx.close()

    def load(self, raw, raw_dtype=None):
        """Linearise and window raw B-scans once: device tensor (B, interf, N)
        (int16 holding uint16 bits with raw_dtype U16, or int16/float32)."""
        self.ctx.follow_torch_stream()
        self.B, interf, _ = raw.shape
        self.nx = interf - self.apod
        self.device = raw.device
        self.ctx.disp_load(raw, self.apod, self.B, 1, self.hann, raw_dtype=raw_dtype)

    def render(self, beta_shift: float = 0.0, out=None):
        """(B, probes, 256, 256) float32 images of the loaded B-scans.  A shift
        b renders the probes at beta - b, i.e. the B-scans as if their spectra
        carried a compensating dispersion b (the scorer's phase trick)."""
        torch = self.torch
        self.ctx.follow_torch_stream()
        P = len(self.probes)
        if out is None:
            out = torch.empty((self.B, P, IMG, IMG), dtype=torch.float32, device=self.device)
        betas = np.ascontiguousarray(self.probes - float(beta_shift), dtype=np.float64)
        self.ctx._check(self.ctx.lib.octgb_disp_images(self.ctx.h, P, betas.ctypes.data, 0, self.B, Z_KEEP, _p(out),
                                                       1))
        return out

    def images(self, raw, out=None, raw_dtype=None):
        self.load(raw, raw_dtype)
        return self.render(0.0, out)


class BetaFocusNet:
    """The CNN (see the module docstring); parameters and Adam state are torch
    CUDA tensors, every computation a C-ABI call on the context's stream."""

    def __init__(self, ctx: Context, in_ch: int = 3, widths=(32, 32, 32, 32), img: int = IMG, hidden: int = 64,
                 seed: int = 0, device="cuda", train_tensor_cores: bool = False):
        """train_tensor_cores: train_step runs the convolutions, their weight
        and data gradients on the tensor cores (FP16 forward operands, BF16
        gradient operands, float32 accumulation) where the shape allows."""
        import torch
        self.torch = torch
        self.train_tensor_cores = bool(train_tensor_cores)
        self.ctx = ctx
        self.lib = ctx.lib
        self.img = img
        self.chans = [in_ch, *widths]
        self.hidden = hidden
        g = torch.Generator().manual_seed(int(seed))
        self.params = []
        for cin, cout in zip(self.chans[:-1], self.chans[1:]):
            w = torch.randn((cout, cin, 3, 3), generator=g) * math.sqrt(2.0 / (cin * 9))
            self.params += [w, torch.zeros(cout)]
        self.flat = widths[-1] * (img // 16) ** 2
        self.params += [torch.randn((hidden, self.flat), generator=g) * math.sqrt(2.0 / self.flat), torch.zeros(hidden),
                        torch.randn((2, hidden), generator=g) * math.sqrt(1.0 / hidden), torch.zeros(2)]
        self.params = [p.float().to(device).contiguous() for p in self.params]
        self.grads = [torch.zeros_like(p) for p in self.params]
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.step_count = 0
        self.wscratch = torch.empty(max(p.numel() for p in self.params[:8:2]), dtype=torch.float32, device=device)
        self.loss_dev = torch.zeros(1, dtype=torch.float64, device=device)
        self._acts = {}

    def _check(self, rc):
        self.ctx._check(rc)

    def _buffers(self, n):
        b = self._acts.get(n)
        if b is None:
            torch = self.torch
            dev = self.params[0].device
            pre, pooled = [], []
            h = self.img
            for cout in self.chans[1:]:
                pre.append(torch.empty((n, cout, h, h), dtype=torch.float32, device=dev))
                h //= 2
                pooled.append(torch.empty((n, cout, h, h), dtype=torch.float32, device=dev))
            b = {"pre": pre, "pooled": pooled,
                 "h_pre": torch.empty((n, self.hidden), dtype=torch.float32, device=dev),
                 "h": torch.empty((n, self.hidden), dtype=torch.float32, device=dev),
                 "out": torch.empty((n, 2), dtype=torch.float32, device=dev),
                 "dout": torch.empty((n, 2), dtype=torch.float32, device=dev),
                 "dh": torch.empty((n, self.hidden), dtype=torch.float32, device=dev),
                 "dflat": torch.empty((n, self.flat), dtype=torch.float32, device=dev),
                 "dpre": [torch.empty_like(t) for t in pre],
                 "dpooled": [torch.empty_like(t) for t in pooled[:-1]]}
            self._acts[n] = b
        return b

    @staticmethod
    def tc_supported(cin: int, cout: int, h: int, w: int) -> bool:
        """Shapes octgb_cnn_conv3x3_tc accepts."""
        if not (1 <= cin <= 32 and 32 <= cout <= 128 and cout % 32 == 0):
            return False
        return w % 128 == 0 if w >= 128 else (128 % w == 0 and h % (128 // w) == 0)

    def forward(self, x, tensor_cores: bool = False, fuse_pool=None):
        """x: (n, in_ch, img, img) float32 CUDA tensor -> (n, 2) predictions (a
        view of an internal buffer, valid until the next call).  Runs on
        torch's current stream (see Context.follow_torch_stream), after the
        work that produced x.  tensor_cores: the convolutions on the tensor
        cores (FP16 operands, float32 accumulation) where the shape allows.
        fuse_pool (default: tensor_cores): layers the fused convolution + ReLU
        + pooling kernel accepts keep no pre-activations (no backward after)."""
        if fuse_pool is None:
            fuse_pool = tensor_cores
        self.ctx.follow_torch_stream()
        n = x.shape[0]
        b = self._buffers(n)
        self._x = x
        cur = x
        h = self.img
        for i, (cin, cout) in enumerate(zip(self.chans[:-1], self.chans[1:])):
            w, bias = self.params[2 * i], self.params[2 * i + 1]
            if fuse_pool and tensor_cores and self.tc_supported(cin, cout, h, h) and h >= 128 and h % 2 == 0:
                # convolution, ReLU and pooling in one kernel (no pre-activations)
                self._check(self.lib.octgb_cnn_conv3x3_relu_pool_tc(self.ctx.h, _p(cur), _p(w), _p(bias),
                                                                    _p(b["pooled"][i]), n, cin, cout, h, h))
            else:
                conv = self.lib.octgb_cnn_conv3x3
                if tensor_cores and self.tc_supported(cin, cout, h, h):
                    conv = self.lib.octgb_cnn_conv3x3_tc
                self._check(conv(self.ctx.h, _p(cur), _p(w), _p(bias), _p(b["pre"][i]), n, cin, cout, h, h))
                self._check(self.lib.octgb_cnn_relu_pool(self.ctx.h, _p(b["pre"][i]), _p(b["pooled"][i]), n * cout,
                                                         h, h))
            cur = b["pooled"][i]
            h //= 2
        w1, b1, w2, b2 = self.params[8:12]
        self._check(self.lib.octgb_cnn_dense(self.ctx.h, _p(cur), _p(w1), _p(b1), _p(b["h_pre"]), _p(b["h"]), n,
                                             self.flat, self.hidden))
        self._check(self.lib.octgb_cnn_dense(self.ctx.h, _p(b["h"]), _p(w2), _p(b2), _p(b["out"]), None, n,
                                             self.hidden, 2))
        return b["out"]

    def predict(self, x):
        """Inference: forward with the convolutions on the tensor cores (layers
        of width >= 128 fused with their ReLU + pooling, so their
        pre-activations are not kept: no backward after predict)."""
        return self.forward(x, tensor_cores=True)

    def backward(self, dout):
        """Gradients of all parameters (self.grads) from d loss / d output."""
        n = dout.shape[0]
        b = self._buffers(n)
        g = self.grads
        w1, b1, w2, b2 = self.params[8:12]
        self._check(self.lib.octgb_cnn_dense_bwd(self.ctx.h, _p(b["h"]), _p(w2), _p(dout), None, _p(b["dh"]),
                                                 _p(g[10]), _p(g[11]), n, self.hidden, 2))
        self._check(self.lib.octgb_cnn_dense_bwd(self.ctx.h, _p(b["pooled"][-1]), _p(w1), _p(b["dh"]),
                                                 _p(b["h_pre"]), _p(b["dflat"]), _p(g[8]), _p(g[9]), n, self.flat,
                                                 self.hidden))
        dp = b["dflat"]
        h = self.img >> (len(self.chans) - 2)
        for i in reversed(range(len(self.chans) - 1)):
            cin, cout = self.chans[i], self.chans[i + 1]
            self._check(self.lib.octgb_cnn_relu_pool_bwd(self.ctx.h, _p(dp), _p(b["pre"][i]), _p(b["dpre"][i]),
                                                         n * cout, h, h))
            xin = self._x if i == 0 else b["pooled"][i - 1]
            dx = None if i == 0 else b["dpooled"][i - 1]
            bwd = self.lib.octgb_cnn_conv3x3_bwd_tc if self.train_tensor_cores else self.lib.octgb_cnn_conv3x3_bwd
            self._check(bwd(self.ctx.h, _p(xin), _p(self.params[2 * i]), _p(b["dpre"][i]), _p(dx), _p(g[2 * i]),
                            _p(g[2 * i + 1]), _p(self.wscratch), n, cin, cout, h, h))
            dp = dx
            h *= 2

    def loss_grad(self, pred, target):
        """MSE loss (device float64 scalar) and its gradient in the dout buffer."""
        b = self._buffers(pred.shape[0])
        self._check(self.lib.octgb_cnn_mse(self.ctx.h, _p(pred), _p(target), pred.numel(), _p(b["dout"]),
                                           _p(self.loss_dev)))
        return self.loss_dev, b["dout"]

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        self.step_count += 1
        for p, g, m, v in zip(self.params, self.grads, self.m, self.v):
            self._check(self.lib.octgb_cnn_adam(self.ctx.h, _p(p), _p(g), _p(m), _p(v), p.numel(), lr, beta1, beta2,
                                                eps, self.step_count))

    def train_step(self, x, target, lr: float):
        pred = self.forward(x, tensor_cores=self.train_tensor_cores, fuse_pool=False)
        loss, dout = self.loss_grad(pred, target)
        self.backward(dout)
        self.adam(lr)
        return loss


def targets(beta_ref, focus_px):
    """Network targets from the compensating beta (reference units) and focus (px)."""
    return np.stack([np.asarray(beta_ref, float) / beta_scale(),
                     (np.asarray(focus_px, float) - FOCUS_CENTER) / FOCUS_SCALE], -1).astype(np.float32)


def decode(pred):
    p = np.asarray(pred, float)
    return p[:, 0] * beta_scale(), p[:, 1] * FOCUS_SCALE + FOCUS_CENTER


# --------------------------------------------------------------------------- the judge
def search_per_bscan(scorer, lo: float, hi: float, n_grid: int = 41, points: int = 9):
    """The plain search of every B-scan on its own: coarse grid (one launch for
    all B-scans and betas), then each B-scan's optimum between the grid
    neighbours of its grid maximum, refined by rounds of `points` candidates
    scored in one launch (estimation.zoom_maximum) to 2e-5 of the largest
    |bound| - the per-B-scan part of estimate_dispersion (dispersion.py:
    213-238), with bounds spanning 0 (dispersion.py:178-181)."""
    grid = np.linspace(lo, hi, int(n_grid))
    S_ = scorer.scores_grid(grid)
    tol = max(abs(lo), abs(hi)) * 2e-5
    out = np.empty(S_.shape[1])
    for j in range(S_.shape[1]):
        i = int(np.argmax(S_[:, j]))
        a, b = grid[max(i - 1, 0)], grid[min(i + 1, len(grid) - 1)]
        x, sx, _ = E.zoom_maximum(lambda xs, j=j: scorer.scores_grid(xs, j)[:, 0], a, b, tol, points)
        out[j] = x if sx >= S_[i, j] else float(grid[i])
    return out, grid, S_


def focus_plain(ctx: Context, mag) -> np.ndarray:
    """Plain focus-band detector (the rules of estimation/focus.py:191-218 on a
    depth profile): 10 log10 of the profile over depths < z_keep, sigma-4
    smoothing minus a sigma-30 trend, the strongest MATLAB peak (0-based
    depth).  The profile is the x-mean of the magnitude: the spectrum model's
    reflectors are sparse, so the reference's x-median is the noise floor at
    every depth.  mag: (B, nX, N/2)."""
    med = ctx.xmean(mag)                                      # (B, N/2) float64
    out = np.empty(med.shape[0])
    for b, prof in enumerate(med[:, :Z_KEEP]):
        lp = 10 * np.log10(np.maximum(prof, 1e-30))
        detr = E.imgaussfilt_1d(lp, 4.0) - E.imgaussfilt_1d(lp, 30.0)
        pk = E.findpeaks_matlab(detr)
        pk = pk[pk >= E.Z_MIN_PIX]
        out[b] = float(pk[np.argmax(detr[pk])]) if pk.size else float(np.argmax(detr[E.Z_MIN_PIX:]) + E.Z_MIN_PIX)
    return out
