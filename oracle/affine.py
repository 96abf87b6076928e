"""Oracle: affine camera fit (test infrastructure only).

Restates ``solve_affine`` (lib/solve_affine.py:37-72) as ``approx_affine_latlonalt``
calls it (camera_approx.py:112-137): the kept points' (x, y, z) = (lat, lon, alt) and
pixels give the 2N x 8 system [x y z 1 0 0 0 0; 0 0 0 0 x y z 1] p = [col; row], solved by
numpy's least squares (LAPACK gelsd, rcond=-1); P is p as 2 x 4.
"""
import numpy as np


def solve_affine(xx, yy, zz, col, row, keep_mask=None):
    xx, yy, zz, col, row = (np.asarray(a, dtype=np.float64).reshape(-1, 1) for a in (xx, yy, zz, col, row))
    if keep_mask is not None:
        k = np.asarray(keep_mask).reshape(-1)
        xx, yy, zz, col, row = (a[k] for a in (xx, yy, zz, col, row))
    n = xx.shape[0]
    ones = np.ones((n, 1))
    zeros = np.zeros((n, 4))
    A = np.vstack((np.hstack((xx, yy, zz, ones, zeros)), np.hstack((zeros, xx, yy, zz, ones))))
    b = np.vstack((col, row))
    return np.linalg.lstsq(A, b, rcond=-1)[0].reshape((2, 4))


def affine_project(P, xx, yy, zz):
    """(col, row) of points under the affine camera P (2 x 4)."""
    X = np.stack([np.ravel(xx), np.ravel(yy), np.ravel(zz), np.ones(np.size(xx))])
    out = P @ X
    return out[0], out[1]
