"""Oracle: per-view height maps -> UTM point lists -> DSMs -> fused DSM (test infrastructure
only).

The reference turns each view's depth map into a UTM point list in pixel order
(aggregate_2p5d_util.py:75-98), rasterises it with produce_dsm_from_points
(produce_dsm.py:46-58: proj_to_grid, then cv2.medianBlur(float32, 3)) and fuses an AOI's
per-view DSMs (aggregate_2p5d.py:65-81).  The synthetic views place pixel (i, j) of a
W x H height map by an affine map in fixed point (units of 2^-28 m):
    easting  = (e0 + ej*(2j+1-W) + ei*(2i+1-H)) * 2^-28
    northing = (n0 + nj*(2j+1-W) + ni*(2i+1-H)) * 2^-28
with the pixel's height; the integers stay below 2^53, so these are exact float64 values.
"""
import numpy as np

from . import blur, fuse, raster

FRAC_BITS = 28


def map_points(heights, affine):
    """(H*W, 3) float64 (easting, northing, height) of a (H, W) float32 height map, rows in
    pixel order (index i*W + j)."""
    H, W = heights.shape
    dj = (2 * np.arange(W, dtype=np.int64) + 1 - W)[None, :]
    di = (2 * np.arange(H, dtype=np.int64) + 1 - H)[:, None]
    e = affine['e0'] + affine['ej'] * dj + affine['ei'] * di
    n = affine['n0'] + affine['nj'] * dj + affine['ni'] * di
    assert np.abs(e).max() < 2 ** 53 and np.abs(n).max() < 2 ** 53
    scale = 2.0 ** -FRAC_BITS
    east = e.astype(np.float64) * scale
    north = n.astype(np.float64) * scale
    return np.stack([east.ravel(), north.ravel(), heights.astype(np.float64).ravel()], axis=1)


def view_dsm(heights, affine, grid):
    """produce_dsm_from_points of one view: proj_to_grid, float32, 3x3 median blur."""
    pts = map_points(heights, affine)
    dsm = raster.proj_to_grid(pts, grid['xoff'], grid['yoff'], grid['xres'], grid['yres'], grid['xsize'],
                              grid['ysize'])
    return blur.median_blur3x3(dsm.astype(np.float32))


def fused_dsm(view_dsms, median_blur=True):
    """The AOI's fusion over its per-view DSMs (stacked in view order)."""
    return fuse.fuse_dsms(np.stack(view_dsms, axis=2), median_blur=median_blur)
