"""Tile placement and focus-weighted stitching operators (host FP64 build,
device apply).

Host side builds, once per scan, the same operators as the reference:
  factor_z / MIN_WEIGHT / min_weight_threshold   octrecon/core/stitching.py:20-33
  linear_interp_matrix                           octrecon/core/stitching.py:36-51
  OpticalPathCorrection                          octrecon/core/stitching.py:54-78
  tiled_geometry                                 octrecon/core/geometry.py:146-202
  TileStitcher (r0:r1, c0:c1, Wz, WxT, fz)       octrecon/core/stitching.py:84-120
and uploads them as a compact 2-tap plan (octgb_stitch_plan); the device
applies OPC gather, focus weight, Wz and WxT and accumulates num/den
(octgb_row_add_batch), replacing TileStitcher.contribute (stitching.py:122-139).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .geometry import colon_matlab, linspace_matlab

CUTOFF_SIGMA = 3.0
MIN_WEIGHT = float(np.exp(-CUTOFF_SIGMA ** 2 / 2))


def min_weight_threshold(dtype=np.float32) -> float:
    """Weight below exp(-4.5) is NaN; a pixel covered by one tile at its floor
    weight sits exactly on the threshold and is kept, so allow 8 ulps of the
    accumulation type (stitching.py:24-28)."""
    return MIN_WEIGHT * (1.0 - 8 * float(np.finfo(dtype).eps))


def factor_z(n_rows: int, focus_pix_1based: float, focus_sigma: float) -> np.ndarray:
    """Focus weight exp(-(z - f)^2 / (2 sigma)^2) + exp(-4.5) on 1-based rows
    (yOCTProcessTiledScan_factorZ; the (2 sigma)^2 denominator is the legacy
    one, so the effective standard deviation is sqrt(2) * sigma)."""
    z = np.arange(1, n_rows + 1, dtype=float)
    return np.exp(-((z - focus_pix_1based) ** 2) / (2.0 * focus_sigma) ** 2) + MIN_WEIGHT


def linear_interp_matrix(src: np.ndarray, dst: np.ndarray) -> np.ndarray:
    """Dense W (len(dst), len(src)) with W @ v = interp1(src, v, dst, 'linear', 0)
    for strictly increasing src; queries within 1e-9 (relative position) of a
    node take the node value exactly, as MATLAB's interp2 does."""
    src = np.asarray(src, float)
    dst = np.asarray(dst, float)
    W = np.zeros((len(dst), len(src)))
    rows = np.flatnonzero((dst >= src[0]) & (dst <= src[-1]))
    q = dst[rows]
    j = np.clip(np.searchsorted(src, q, side="right") - 1, 0, len(src) - 2)
    t = (q - src[j]) / (src[j + 1] - src[j])
    t = np.where(np.abs(t) < 1e-9, 0.0, t)
    t = np.where(np.abs(1.0 - t) < 1e-9, 1.0, t)
    np.add.at(W, (rows, j), 1.0 - t)
    np.add.at(W, (rows, j + 1), t)
    return W


@dataclass
class OpticalPathCorrection:
    """Per (frame, A-scan) integer row shift round(P/dz) and P/dz for validity,
    P = p1 x + p2 y + p3 x^2 + p4 y^2 + p5 x y (um)."""
    shift: np.ndarray
    pdz: np.ndarray
    n_rows: int

    @classmethod
    def build(cls, poly, tile_x_mm, tile_y_mm, tile_z_mm):
        x, y, z = tile_x_mm * 1e3, tile_y_mm * 1e3, tile_z_mm * 1e3
        dz = (z[-1] - z[0]) / (len(z) - 1)
        X, Y = np.meshgrid(x, y)
        P = poly[0] * X + poly[1] * Y + poly[2] * X ** 2 + poly[3] * Y ** 2 + poly[4] * X * Y
        pdz = P / dz
        return cls(np.floor(pdz + 0.5).astype(np.int64), pdz, len(z))


@dataclass
class ScanLayout:
    """The scan description fields the tiled geometry needs (ScanInfo.json:
    xCenters_mm, yCenters_mm, zDepths, nX/nYPixelsInEachTile, tileRangeX/Y_mm,
    xOffset, yOffset)."""
    x_centers_mm: np.ndarray
    y_centers_mm: np.ndarray
    z_depths_mm: np.ndarray
    n_x_px: int
    n_y_px: int
    tile_range_x_mm: float
    tile_range_y_mm: float
    x_offset: float = 0.0
    y_offset: float = 0.0
    x_shift_mm: float = 0.0    # galvo phase-delay x correction already folded into tile x


@dataclass
class TiledGeometry:
    tile_x_mm: np.ndarray
    tile_y_mm: np.ndarray
    tile_z_mm: np.ndarray
    out_x_mm: np.ndarray
    out_y_mm: np.ndarray
    out_z_mm: np.ndarray
    focus_pix: np.ndarray


def tiled_geometry(si: ScanLayout, z_um_tile, focus_pix, output_pixel_size_um=None,
                   crop_z_range_mm=None) -> TiledGeometry:
    """Tile-local and output grids (yOCTProcessTiledScan_createDimStructure and
    yOCTProcessTiledScan.m 171-222; reference octrecon/core/geometry.py:146-202)."""
    zd = np.asarray(si.z_depths_mm, float)
    xc = np.asarray(si.x_centers_mm, float)
    yc = np.asarray(si.y_centers_mm, float)
    focus = np.asarray(focus_pix, float).ravel()
    if focus.size == 1:
        focus = np.full(len(zd), focus[0])
    if focus.size != len(zd):
        raise ValueError("focus_pix must be scalar or one value per zDepth")
    tx = (si.x_offset + si.tile_range_x_mm * linspace_matlab(-0.5, 0.5, si.n_x_px + 1))[:-1] - si.x_shift_mm
    ty = (si.y_offset + si.tile_range_y_mm * linspace_matlab(-0.5, 0.5, si.n_y_px + 1))[:-1]
    tz = np.asarray(z_um_tile, float) / 1e3
    if not np.any(np.isnan(focus)):
        ref = focus[0] if np.all(focus == focus[0]) else focus[int(np.argmin(np.abs(zd)))]
        tz = tz - tz[int(np.round(ref)) - 1]
    dx = tx[1] - tx[0]
    dy = ty[1] - ty[0] if len(ty) > 1 else 0.0
    dz = tz[1] - tz[0]
    x_all = colon_matlab(xc.min() + tx[0], dx, xc.max() + tx[-1] + dx / 2)
    y_all = colon_matlab(yc.min() + ty[0], dy, yc.max() + ty[-1] + dy / 2)
    z_all = colon_matlab(zd.min() + tz[0], dz, zd.max() + tz[-1] + dz / 2)
    zero = int(np.argmin(np.abs(z_all)))
    z_all = dz * (np.arange(1, len(z_all) + 1) - (zero + 1))
    if len(xc) == 1:
        x_all = tx.copy()
    if len(yc) == 1:
        y_all = ty.copy()
    if output_pixel_size_um is not None:
        px = np.round(np.mean(np.diff(x_all)) * 1e3 * 100) / 100
        py = np.round(np.mean(np.diff(y_all)) * 1e3 * 100) / 100 if len(y_all) >= 2 else px
        if not (px == py == output_pixel_size_um):
            raise ValueError(f"output pixel size {output_pixel_size_um} um must equal the scan pixel size "
                             f"({px}, {py}) um")
        z_all = colon_matlab(z_all[0], output_pixel_size_um * 1e-3, z_all.max())
    if crop_z_range_mm is not None and len(crop_z_range_mm):
        lo, hi = crop_z_range_mm
        z_all = z_all[~((z_all < lo) | (z_all > hi))]
        if z_all.size == 0:
            raise ValueError("crop_z_range_mm does not overlap the available z range")
    return TiledGeometry(tx, ty, tz, x_all, y_all, z_all, focus)


@dataclass
class TileStitcher:
    """Operators of one tile position (xi, zi); `plan` is the device plan id
    once uploaded (`upload`)."""
    empty: bool
    r0: int = 0
    r1: int = 0
    c0: int = 0
    c1: int = 0
    Wz: np.ndarray | None = None      # (nOutZ, R) float32 values
    WxT: np.ndarray | None = None     # (nTileX, C)
    fz: np.ndarray | None = None      # (R,)
    n_rows: int = 0
    plan: int | None = field(default=None, repr=False)

    @classmethod
    def build(cls, tg: TiledGeometry, xi_center_mm: float, z_depth_mm: float, focus_pix: float,
              focus_sigma: float, dtype=np.float32) -> "TileStitcher":
        nz = len(tg.tile_z_mm)
        x = tg.tile_x_mm + xi_center_mm
        z = tg.tile_z_mm + z_depth_mm
        if not np.isnan(focus_pix):
            z = z - tg.tile_z_mm[int(np.round(focus_pix)) - 1]
        x = x.copy()
        z = z.copy()
        # widen the end nodes so output points on the tile edge stay inside
        x[0] -= 1e-10
        x[-1] += 1e-10
        z[0] -= 1e-10
        z[-1] += 1e-10
        Wz = linear_interp_matrix(z, tg.out_z_mm)
        Wx = linear_interp_matrix(x, tg.out_x_mm)
        rows = np.flatnonzero(Wz.any(axis=0))
        cols = np.flatnonzero(Wx.any(axis=1))
        if rows.size == 0 or cols.size == 0:
            return cls(empty=True)
        r0, r1 = int(rows[0]), int(rows[-1]) + 1
        c0, c1 = int(cols[0]), int(cols[-1]) + 1
        fz = factor_z(nz, focus_pix, focus_sigma) if not np.isnan(focus_pix) else np.ones(nz)
        return cls(False, r0, r1, c0, c1, Wz[:, r0:r1].astype(dtype), Wx[c0:c1, :].T.astype(dtype),
                   fz[r0:r1].astype(dtype), nz)

    def upload(self, ctx, oc: OpticalPathCorrection | None = None) -> int:
        if self.empty:
            raise ValueError("empty tile position has no plan")
        self.plan = ctx.stitch_plan(self.n_rows, self.r0, self.r1, self.c0, self.c1, self.Wz, self.WxT, self.fz,
                                    None if oc is None else oc.shift, None if oc is None else oc.pdz)
        return self.plan
