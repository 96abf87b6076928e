"""Oracle: fusion of per-view DSMs (test infrastructure only).

``fuse_numpy`` runs the numpy calls of aggregate_2p5d.py:68-78 in order on an
(H, W, V) float32 stack: cells with <= 2 measurements rejected, per-cell nanmedian,
MAD = nanmedian of |x - median|, samples with |x - median| > MAD rejected, nanmean of
the rest.  ``fuse_explicit`` spells out the arithmetic numpy performs for those calls
(the recipe the CUDA kernel follows) and is checked bit-for-bit against
``fuse_numpy`` by the tests:

* nanmedian of n valid values (masked-array median): sorted s, lo = s[(n-1)//2],
  hi = s[n//2], median = ((0 + lo) + hi) / 2 in float32 (odd n: lo == hi);
* nanmean: NaN -> 0, float32 sum in numpy's pairwise order over the V slots in view
  order, started from the reduction identity 0; then f32(f64(sum) / count).
"""
import warnings

import numpy as np


def fuse_numpy(all_dsm):
    a = np.array(all_dsm, dtype=np.float32, copy=True)
    cnt = a.shape[2]
    with warnings.catch_warnings():
        warnings.simplefilter('ignore', RuntimeWarning)
        num = cnt - np.sum(np.isnan(a), axis=2, keepdims=True)
        a[np.tile(num <= 2, (1, 1, cnt))] = np.nan
        med = np.nanmedian(a, axis=2, keepdims=True)
        mad = np.nanmedian(np.abs(a - med), axis=2, keepdims=True)
        a[np.abs(a - med) > mad] = np.nan
        return np.nanmean(a, axis=2)


def pairwise_sum_f32(v):
    """numpy's float32 pairwise summation of a 1-D contiguous block."""
    n = v.size
    f = np.float32
    if n < 8:
        res = f(0.0)
        for x in v:
            res = f(res + x)
        return res
    if n <= 128:
        r = [f(x) for x in v[:8]]
        i = 8
        while i < n - (n % 8):
            for j in range(8):
                r[j] = f(r[j] + v[i + j])
            i += 8
        res = f(f(f(r[0] + r[1]) + f(r[2] + r[3])) + f(f(r[4] + r[5]) + f(r[6] + r[7])))
        while i < n:
            res = f(res + v[i])
            i += 1
        return res
    n2 = n // 2
    n2 -= n2 % 8
    return f(pairwise_sum_f32(v[:n2]) + pairwise_sum_f32(v[n2:]))


def _median_f32(s):
    n = s.size
    lo = s[(n - 1) // 2]
    hi = s[n // 2]
    return np.float32(np.float32(np.float32(0.0) + lo) + hi) / np.float32(2.0)


def fuse_cell(x):
    """Explicit per-cell recipe; x is the float32 vector of one cell's V views."""
    f = np.float32
    x = np.asarray(x, dtype=np.float32)
    valid = ~np.isnan(x)
    n = int(valid.sum())
    if n <= 2:
        return f(np.nan)
    s = np.sort(x[valid])
    with np.errstate(invalid='ignore', over='ignore'):
        med = _median_f32(s)
        d = np.abs(x - med).astype(np.float32)
        dv = d[~np.isnan(d)]
        mad = _median_f32(np.sort(dv)) if dv.size else f(np.nan)
        keep = valid & ~(d > mad)
    vals = np.where(keep, x, f(0.0)).astype(np.float32)
    tot = f(f(0.0) + pairwise_sum_f32(vals))
    count = int(keep.sum())
    with np.errstate(invalid='ignore', divide='ignore'):
        return f(np.float64(tot) / np.float64(count)) if count else f(np.nan)


def fuse_explicit(all_dsm):
    a = np.asarray(all_dsm, dtype=np.float32)
    H, W, V = a.shape
    out = np.empty((H, W), dtype=np.float32)
    for i in range(H):
        for j in range(W):
            out[i, j] = fuse_cell(a[i, j])
    return out


def fuse_dsms(all_dsm, median_blur=True):
    """aggregate_2p5d.py:65-81: fused (H, W) float32 DSM, optionally 3x3 median blurred."""
    from .blur import median_blur3x3
    out = fuse_numpy(all_dsm)
    return median_blur3x3(out) if median_blur else out
