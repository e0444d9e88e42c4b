"""Seeded synthetic spectral-domain OCT spectra (uint16 camera counts).

No public dataset is involved: every workload of this package is generated here.
Spectrum model (one A-scan, N spectral pixels, j = 0..N-1, u = j/(N-1)):

  q_j      = (N-1) * (u + c2 * u * (1 - u))          position of raw pixel j on the
                                                     linear-k grid (c2 = 0.05)
  k_j      = kmax - (kmax - kmin) * q_j / (N-1)      k spans 2*pi/796 .. 2*pi/1010 nm
  lambda_j = 2*pi / k_j
  env_j    = A * exp(-4 ln2 (j - N/2)^2 / FWHM^2)    A = 20000, FWHM = 0.3 N
  s_j      = env_j * (1 + sum_r a_r cos(2 pi d_r q_j / N + beta_px (q_j - N/2)^2))
             + noise N(0, sigma)  -> rounded, clipped to [0, 65535]

with 5 reflectors per A-scan, depths d_r ~ U[50, 900] px, amplitudes
a_r ~ 10^U[-4, -2].  Apodisation (background) lines are env_j + noise.
`beta_px` is the dispersion in rad/px^2; the reconstruction's
`dispersion_quadratic_term` in nm^2/rad is beta_px / dk^2, dk = (kmax-kmin)/(N-1).

An optional confocal focus envelope multiplies each reflector amplitude by
exp(-((d_r - focus_px)/focus_width)^2) (used by the learned beta/focus workload).

The torch implementation runs on CPU or CUDA (large volumes are generated on the
device); the values for a given seed depend on the device's RNG.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

LAMBDA_MIN_NM = 796.0
LAMBDA_MAX_NM = 1010.0


@dataclass
class SpectrumParams:
    n: int = 2048
    chirp_c2: float = 0.05
    peak: float = 20000.0
    fwhm_frac: float = 0.30
    n_reflectors: int = 5
    depth_lo: float = 50.0
    depth_hi: float = 900.0
    log_amp_lo: float = -4.0
    log_amp_hi: float = -2.0
    beta_px: float = 1e-5
    noise_sigma: float = 20.0


def raw_position(p: SpectrumParams) -> np.ndarray:
    """q_j: raw pixel j's position on the linear-k grid (float64)."""
    u = np.arange(p.n, dtype=np.float64) / (p.n - 1)
    return (p.n - 1) * (u + p.chirp_c2 * u * (1.0 - u))


def lambda_nm(p: SpectrumParams | None = None) -> np.ndarray:
    """Per-pixel wavelength (nm) of the synthetic spectrometer."""
    p = p or SpectrumParams()
    kmax, kmin = 2 * np.pi / LAMBDA_MIN_NM, 2 * np.pi / LAMBDA_MAX_NM
    k = kmax - (kmax - kmin) * raw_position(p) / (p.n - 1)
    return 2 * np.pi / k


def dk_per_px(p: SpectrumParams | None = None) -> float:
    p = p or SpectrumParams()
    kmax, kmin = 2 * np.pi / LAMBDA_MIN_NM, 2 * np.pi / LAMBDA_MAX_NM
    return (kmax - kmin) / (p.n - 1)


def beta_ref_from_px(beta_px: float, p: SpectrumParams | None = None) -> float:
    """Dispersion in the reconstruction's units (nm^2/rad) for a beta in rad/px^2."""
    return beta_px / dk_per_px(p) ** 2


def envelope(p: SpectrumParams) -> np.ndarray:
    j = np.arange(p.n, dtype=np.float64)
    fwhm = p.fwhm_frac * p.n
    return p.peak * np.exp(-4.0 * np.log(2.0) * (j - p.n / 2) ** 2 / fwhm ** 2)


def generate(n_bscans: int, n_ascans: int, apod: int = 25, seed: int = 0, params: SpectrumParams | None = None,
             device="cpu", beta_px=None, focus_px=None, focus_width: float = 150.0, chunk: int = 16,
             precision: str = "float64"):
    """uint16-valued spectra (B, apod + nX, N) as a torch tensor of dtype int32 on
    `device` (torch has limited uint16 support): narrow with
    `generate_numpy` on the host or `u16_bits` on the device.

    beta_px / focus_px: scalars or per-B-scan arrays overriding the defaults.
    precision "float32" evaluates the model in float32 (fringe phases of up to
    ~6e3 rad then carry ~3e-4 rad of rounding, below 0.1 count of the result:
    far under the noise), for workloads of tens of thousands of B-scans."""
    import torch

    p = params or SpectrumParams()
    dev = torch.device(device)
    fdt = {"float64": torch.float64, "float32": torch.float32}[precision]
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    q = torch.as_tensor(raw_position(p), dtype=fdt, device=dev)
    env = torch.as_tensor(envelope(p), dtype=fdt, device=dev)
    N = p.n
    out = torch.empty((n_bscans, apod + n_ascans, N), dtype=torch.int32, device=dev)
    betas = np.broadcast_to(np.asarray(p.beta_px if beta_px is None else beta_px, float), (n_bscans,))
    foci = None if focus_px is None else np.broadcast_to(np.asarray(focus_px, float), (n_bscans,))
    qc = (q - N / 2) ** 2
    for b0 in range(0, n_bscans, chunk):
        b1 = min(n_bscans, b0 + chunk)
        nb = b1 - b0
        depth = p.depth_lo + (p.depth_hi - p.depth_lo) * torch.rand(
            (nb, n_ascans, p.n_reflectors), generator=g, device=dev, dtype=fdt)
        amp = 10.0 ** (p.log_amp_lo + (p.log_amp_hi - p.log_amp_lo) * torch.rand(
            (nb, n_ascans, p.n_reflectors), generator=g, device=dev, dtype=fdt))
        if foci is not None:
            f = torch.as_tensor(np.array(foci[b0:b1], dtype=np.float64), device=dev).to(fdt)[:, None, None]
            amp = amp * torch.exp(-((depth - f) / focus_width) ** 2)
        beta = torch.as_tensor(np.array(betas[b0:b1], dtype=np.float64), device=dev).to(fdt)[:, None, None]
        s = torch.ones((nb, n_ascans, N), dtype=fdt, device=dev)
        for r in range(p.n_reflectors):
            ph = (2 * np.pi / N) * depth[..., r:r + 1] * q + beta * qc
            s += amp[..., r:r + 1] * torch.cos(ph)
        s *= env
        s += p.noise_sigma * torch.randn((nb, n_ascans, N), generator=g, device=dev, dtype=fdt)
        bg = env + p.noise_sigma * torch.randn((nb, apod, N), generator=g, device=dev, dtype=fdt)
        out[b0:b1, :apod] = torch.clamp(torch.round(bg), 0, 65535).to(torch.int32)
        out[b0:b1, apod:] = torch.clamp(torch.round(s), 0, 65535).to(torch.int32)
    return out


def generate_numpy(n_bscans: int, n_ascans: int, apod: int = 25, seed: int = 0, **kw) -> np.ndarray:
    """Host uint16 array (B, apod + nX, N) from the CPU generator."""
    t = generate(n_bscans, n_ascans, apod, seed, device="cpu", **kw)
    return t.numpy().astype(np.uint16)


def u16_bits(t):
    """int16 tensor holding the uint16 bit patterns of an int32 tensor with
    values in [0, 65535]; pass it with raw_dtype=U16."""
    import torch
    return (t - 65536 * (t > 32767).to(t.dtype)).to(torch.int16)


def config1_layout(seed: int = 1, bscans: int = 270):
    """The tiled scan of the 2 x 2 tiles x 3 depths workload: tiles of 1000
    A-scans x `bscans` B-scans at 1 um pixels, centres +-0.45 mm (10 % lateral
    overlap), depths 0 / 0.15 / 0.30 mm, focus 400 + U[-30, 30] px per depth.
    Returns (stitching.ScanLayout, focus pixels)."""
    from .stitching import ScanLayout
    rng = np.random.default_rng(seed)
    ty = int(bscans) * 1e-3
    lay = ScanLayout(np.array([-0.45, 0.45]), np.array([-0.45 * ty, 0.45 * ty]), np.array([0.0, 0.15, 0.30]),
                     1000, int(bscans), 1.0, ty)
    return lay, 400.0 + rng.uniform(-30, 30, 3)
