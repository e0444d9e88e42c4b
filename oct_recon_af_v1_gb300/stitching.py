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


@dataclass
class Resampling:
    """MATLAB linear interpolation with 0 outside (interp1 / interp2
    'linear'), from strictly increasing source nodes to destination points,
    as a 2-tap plan: destination rows[k] = (1 - t[k]) v[j[k]] + t[k] v[j[k] + 1].
    A destination within 1e-9 (relative position) of a node takes the node
    value exactly, as MATLAB does.  This is the form the device applies; the
    dense matrix, the source rows and destination columns a tile touches
    follow from it."""
    rows: np.ndarray       # destination indices inside [src[0], src[-1]]
    j: np.ndarray          # left source node of each
    t: np.ndarray          # fraction towards the right node
    n_src: int
    n_dst: int

    @classmethod
    def between(cls, src, dst) -> "Resampling":
        src = np.asarray(src, float)
        dst = np.asarray(dst, float)
        rows = np.flatnonzero((dst >= src[0]) & (dst <= src[-1]))
        q = dst[rows]
        j = np.clip(np.searchsorted(src, q, side="right") - 1, 0, len(src) - 2)
        t = (q - src[j]) / (src[j + 1] - src[j])
        t = np.where(np.abs(t) < 1e-9, 0.0, t)
        t = np.where(np.abs(1.0 - t) < 1e-9, 1.0, t)
        return cls(rows, j, t, len(src), len(dst))

    def dense(self) -> np.ndarray:
        """W (n_dst, n_src) with W @ v the interpolated values."""
        W = np.zeros((self.n_dst, self.n_src))
        W[self.rows, self.j] += 1.0 - self.t
        W[self.rows, self.j + 1] += self.t
        return W

    def sources_used(self) -> np.ndarray:
        """Source nodes that carry a non-zero weight, increasing."""
        left = self.j[(1.0 - self.t) != 0]
        right = self.j[self.t != 0] + 1
        return np.unique(np.concatenate([left, right]))

    def targets_used(self) -> np.ndarray:
        """Destination points with a non-zero weight, increasing."""
        return self.rows[((1.0 - self.t) != 0) | (self.t != 0)]


def _placed_depths(tile_z_mm: np.ndarray, z_depth_mm: float, focus_pix: float) -> np.ndarray:
    """Tile rows in the output depth frame: the tile's depth added, then the
    focus row's own position subtracted (no shift without a focus)."""
    z = tile_z_mm + z_depth_mm
    return z if np.isnan(focus_pix) else z - tile_z_mm[int(np.round(focus_pix)) - 1]


def _edge_widened(nodes: np.ndarray) -> np.ndarray:
    """A copy of increasing nodes with the first moved 1e-10 down and the last
    1e-10 up."""
    out = np.array(nodes, float, copy=True)
    out[0] -= 1e-10
    out[-1] += 1e-10
    return out


def linear_interp_matrix(src: np.ndarray, dst: np.ndarray) -> np.ndarray:
    """Dense W (len(dst), len(src)) of Resampling.between(src, dst)
    (octrecon/core/stitching.py:36-51)."""
    return Resampling.between(src, dst).dense()


@dataclass
class OpticalPathCorrection:
    """Per (frame, A-scan) integer row shift round(P/dz) and P/dz for validity,
    P = p1 x + p2 y + p3 x^2 + p4 y^2 + p5 x y (um)."""
    shift: np.ndarray
    pdz: np.ndarray
    n_rows: int

    @classmethod
    def build(cls, poly, tile_x_mm, tile_y_mm, tile_z_mm):
        """poly = (p1 .. p5) in um over the tile's x / y pixels (um); the
        shift is in z pixels of the tile (octrecon/core/stitching.py:67-78)."""
        to_um = 1e3
        x, y, z = tile_x_mm * to_um, tile_y_mm * to_um, tile_z_mm * to_um
        z_step = (z[-1] - z[0]) / (len(z) - 1)
        X, Y = np.meshgrid(x, y)
        rows = _path_surface(poly, X, Y) / z_step
        return cls(np.floor(rows + 0.5).astype(np.int64), rows, len(z))


def _path_surface(poly, X, Y):
    """Optical path P(x, y) = p1 x + p2 y + p3 x^2 + p4 y^2 + p5 x y, the terms
    summed left to right and the cross term formed as (p5 x) y: the float64
    evaluation order the reference's expression has, so P is bit-identical."""
    terms = (poly[0] * X, poly[1] * Y, poly[2] * X ** 2, poly[3] * Y ** 2, poly[4] * X * Y)
    total = terms[0]
    for term in terms[1:]:
        total = total + term
    return total


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


def _tile_pixels(offset: float, extent_mm: float, n: int) -> np.ndarray:
    """Positions (mm) of a tile's n pixels along one lateral axis: n + 1
    MATLAB-linspace edges over the extent, centred on `offset`, the last edge
    dropped (yOCTProcessTiledScan_createDimStructure)."""
    return (offset + extent_mm * linspace_matlab(-0.5, 0.5, n + 1))[:-1]


def _covering_grid(centres: np.ndarray, local: np.ndarray, step: float) -> np.ndarray:
    """The grid (MATLAB colon, pitch `step`) from the first pixel of the lowest
    tile to the last pixel of the highest one, half a step of slack at the
    end (yOCTProcessTiledScan.m 171-185)."""
    return colon_matlab(centres.min() + local[0], step, centres.max() + local[-1] + step / 2)


def _focus_reference(focus: np.ndarray, depths_mm: np.ndarray) -> float:
    """The focus pixel the tile z axis is zeroed at: the common one, or the
    one of the depth closest to 0."""
    return focus[0] if np.all(focus == focus[0]) else focus[int(np.argmin(np.abs(depths_mm)))]


def _pixel_pitch_um(grid_mm: np.ndarray) -> float:
    """Mean pitch of an output grid in um, rounded to 0.01 um."""
    return np.round(np.mean(np.diff(grid_mm)) * 1e3 * 100) / 100


def tiled_geometry(si: ScanLayout, z_um_tile, focus_pix, output_pixel_size_um=None,
                   crop_z_range_mm=None) -> TiledGeometry:
    """Tile-local and output grids of a tiled scan (yOCTProcessTiledScan_
    createDimStructure and yOCTProcessTiledScan.m 171-222; reference
    octrecon/core/geometry.py:146-202).  The grids are built per axis: tile
    pixels, the covering output grid, then z re-zeroed at the focus, resampled
    to the output pixel size and cropped."""
    depths = np.asarray(si.z_depths_mm, float)
    x_centres = np.asarray(si.x_centers_mm, float)
    y_centres = np.asarray(si.y_centers_mm, float)
    focus = np.asarray(focus_pix, float).ravel()
    if focus.size == 1:
        focus = np.full(len(depths), focus[0])
    if focus.size != len(depths):
        raise ValueError("focus_pix must be scalar or one value per zDepth")
    # lateral axes: tile pixels and the grid covering every tile centre
    tile_x = _tile_pixels(si.x_offset, si.tile_range_x_mm, si.n_x_px) - si.x_shift_mm
    tile_y = _tile_pixels(si.y_offset, si.tile_range_y_mm, si.n_y_px)
    out_x = tile_x.copy() if len(x_centres) == 1 else _covering_grid(x_centres, tile_x, tile_x[1] - tile_x[0])
    y_step = tile_y[1] - tile_y[0] if len(tile_y) > 1 else 0.0
    out_y = tile_y.copy() if len(y_centres) == 1 else _covering_grid(y_centres, tile_y, y_step)
    # depth: the tile axis zeroed at the focus row, the covering grid zeroed at
    # its sample closest to 0
    tile_z = np.asarray(z_um_tile, float) / 1e3
    if not np.any(np.isnan(focus)):
        tile_z = tile_z - tile_z[int(np.round(_focus_reference(focus, depths))) - 1]
    z_step = tile_z[1] - tile_z[0]
    cover_z = _covering_grid(depths, tile_z, z_step)
    zero = int(np.argmin(np.abs(cover_z)))
    out_z = z_step * (np.arange(1, len(cover_z) + 1) - (zero + 1))
    if output_pixel_size_um is not None:
        pitch_x = _pixel_pitch_um(out_x)
        pitch_y = _pixel_pitch_um(out_y) if len(out_y) >= 2 else pitch_x
        if not (pitch_x == pitch_y == output_pixel_size_um):
            raise ValueError(f"output pixel size {output_pixel_size_um} um must equal the scan pixel size "
                             f"({pitch_x}, {pitch_y}) um")
        out_z = colon_matlab(out_z[0], output_pixel_size_um * 1e-3, out_z.max())
    if crop_z_range_mm is not None and len(crop_z_range_mm):
        lo, hi = crop_z_range_mm
        out_z = out_z[~((out_z < lo) | (out_z > hi))]
        if out_z.size == 0:
            raise ValueError("crop_z_range_mm does not overlap the available z range")
    return TiledGeometry(tile_x, tile_y, tile_z, out_x, out_y, out_z, focus)


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
        """The tile at lateral centre xi_center_mm and depth z_depth_mm
        (octrecon/core/stitching.py:84-120): its pixels placed in the output
        frame (z shifted so the focus row sits at the tile's depth), the end
        nodes widened by 1e-10 mm so output points on a tile edge stay inside,
        then one 2-tap resampling plan per axis; the source rows the depth
        plan touches give r0:r1, the output columns the lateral plan reaches
        give c0:c1."""
        depth_nodes = _edge_widened(_placed_depths(tg.tile_z_mm, z_depth_mm, focus_pix))
        lateral_nodes = _edge_widened(tg.tile_x_mm + xi_center_mm)
        along_z = Resampling.between(depth_nodes, tg.out_z_mm)
        along_x = Resampling.between(lateral_nodes, tg.out_x_mm)
        rows, cols = along_z.sources_used(), along_x.targets_used()
        if rows.size == 0 or cols.size == 0:
            return cls(empty=True)
        r0, r1 = int(rows[0]), int(rows[-1]) + 1
        c0, c1 = int(cols[0]), int(cols[-1]) + 1
        n_rows = len(tg.tile_z_mm)
        weight = factor_z(n_rows, focus_pix, focus_sigma) if not np.isnan(focus_pix) else np.ones(n_rows)
        return cls(False, r0, r1, c0, c1, along_z.dense()[:, r0:r1].astype(dtype),
                   along_x.dense()[c0:c1, :].T.astype(dtype), weight[r0:r1].astype(dtype), n_rows)

    def upload(self, ctx, oc: OpticalPathCorrection | None = None) -> int:
        if self.empty:
            raise ValueError("empty tile position has no plan")
        self.plan = ctx.stitch_plan(self.n_rows, self.r0, self.r1, self.c0, self.c1, self.Wz, self.WxT, self.fz,
                                    None if oc is None else oc.shift, None if oc is None else oc.pdz)
        return self.plan
