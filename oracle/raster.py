"""Oracle: max-height rasterisation onto the DSM grid (test infrastructure only).

Restates ``proj_to_grid`` (lib/proj_to_grid.py:41-81):

1. FP64 binning  row = floor((yoff - y) / xres), col = floor((x - xoff) / yres)
   (the reference passes the resolutions crossed; both are equal at every call site),
   points outside 0<=row<ysize, 0<=col<xsize dropped (NaN/inf coordinates included).
2. Per-cell ``nanmax`` of the heights through ``numpy_groupies.aggregate`` (version
   0.9.9, not installed here).  The reference's pinned environment has numba, so
   ``npg.aggregate`` is the numba implementation: NaN values are skipped, the first
   non-NaN value of a cell seeds it and later values replace it only when strictly
   greater (so -inf survives and the first of two equal zeros keeps its sign); cells
   without a value get the fill value NaN.
3. Non-propagating hole fill: every NaN cell with at least one non-NaN 3x3 neighbour
   (read from the pre-fill grid) becomes ``np.median`` of those neighbours.

``hole_fill_loop`` keeps the reference's per-cell loop; ``hole_fill`` is a vectorised
restatement checked equal to it by the tests.
"""
import numpy as np


def bin_points(points, xoff, yoff, xresolution, yresolution, xsize, ysize):
    """(cell index int64, height float64) of the points that land inside the grid."""
    with np.errstate(invalid='ignore', over='ignore'):
        row = np.floor((yoff - points[:, 1]) / xresolution)
        col = np.floor((points[:, 0] - xoff) / yresolution)
        inside = (row >= 0) & (col >= 0) & (row < ysize) & (col < xsize)
    idx = row[inside].astype(np.int64) * xsize + col[inside].astype(np.int64)
    return idx, points[inside, 2]


def group_nanmax(idx, val, size):
    """numpy_groupies 0.9.9 ``aggregate(..., func='nanmax', fill_value=nan)`` (numba
    flavour), sequential over the input order: NaN values skipped, empty cells NaN,
    otherwise the maximum; when the maximum is zero its sign is that of the first zero
    of the cell in input order (a later equal value never replaces the current one)."""
    out = np.full(size, np.nan)
    good = ~np.isnan(val)
    idx = idx[good]
    val = val[good]
    best = np.full(size, -np.inf)
    np.maximum.at(best, idx, val)
    present = np.zeros(size, dtype=bool)
    present[idx] = True
    out[present] = best[present]
    zero = val == 0
    zcells, zfirst = np.unique(idx[zero], return_index=True)
    is_zero_max = out[zcells] == 0
    out[zcells[is_zero_max]] = val[zero][zfirst[is_zero_max]]
    return out


def nanmax_grid(points, xoff, yoff, xresolution, yresolution, xsize, ysize):
    idx, val = bin_points(points, xoff, yoff, xresolution, yresolution, xsize, ysize)
    return group_nanmax(idx, val, xsize * ysize).reshape(ysize, xsize)


def hole_fill_loop(dsm):
    """lib/proj_to_grid.py:64-79, cell by cell (slow; small grids only)."""
    src = dsm.copy()
    out = dsm.copy()
    H, W = src.shape
    for r, c in np.argwhere(np.isnan(src)):
        neigh = []
        for j in range(r - 1, r + 2):
            for k in range(c - 1, c + 2):
                if 0 <= j < H and 0 <= k < W and not np.isnan(src[j, k]):
                    neigh.append(src[j, k])
        if neigh:
            out[r, c] = np.median(neigh)
    return out


def hole_fill(dsm):
    """Vectorised form of ``hole_fill_loop``.

    For a NaN cell with n valid neighbours (sorted s_0..s_{n-1}) numpy's median is
    (0 + s_{n//2}) / 1 for odd n and ((0 + s_{n/2-1}) + s_{n/2}) / 2 for even n (the
    0 is the identity the sum reduction starts from).
    """
    H, W = dsm.shape
    pad = np.full((H + 2, W + 2), np.nan)
    pad[1:-1, 1:-1] = dsm
    holes = np.argwhere(np.isnan(dsm))
    if holes.size == 0:
        return dsm.copy()
    r = holes[:, 0] + 1
    c = holes[:, 1] + 1
    neigh = np.stack([pad[r + dj, c + dk] for dj in (-1, 0, 1) for dk in (-1, 0, 1)], axis=1)
    n = np.sum(~np.isnan(neigh), axis=1)
    s = np.sort(neigh, axis=1)          # NaN sorts last
    out = dsm.copy()
    has = n > 0
    nn = n[has]
    ss = s[has]
    rows = np.arange(ss.shape[0])
    hi = ss[rows, nn // 2]
    lo = ss[rows, np.maximum(nn // 2 - 1, 0)]
    with np.errstate(invalid='ignore', over='ignore'):
        even = ((0.0 + lo) + hi) / 2.0
        odd = (0.0 + hi) / 1.0
    med = np.where(nn % 2 == 0, even, odd)
    out[holes[has, 0], holes[has, 1]] = med
    return out


def proj_to_grid(points, xoff, yoff, xresolution, yresolution, xsize, ysize, propagate=False,
                 loop=False):
    """float64 (ysize, xsize) DSM of lib/proj_to_grid.py:41-81."""
    dsm = nanmax_grid(points, xoff, yoff, xresolution, yresolution, xsize, ysize)
    return hole_fill_loop(dsm) if loop else hole_fill(dsm)
