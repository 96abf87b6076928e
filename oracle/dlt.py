"""Oracle: perspective (DLT) fit to RPC projections (test infrastructure only).

Restates ``solve_perspective`` and ``factorize`` (lib/solve_perspective.py:38-126) and
``check_perspective_error`` (lib/check_error.py:37-121) with numpy/scipy, plus the
camera parameter vector of camera_approx.py:178-182.
"""
import numpy as np
from scipy import linalg

from .quat import quaternion_from_rotation


def factorize(P):
    """K, R, t of a 3x4 camera (lib/solve_perspective.py:38-79).

    RQ of the left 3x3 block; K's diagonal made positive by flipping K/R signs
    (all three when an odd number is negative, else in pairs); K scaled to K[2,2]=1;
    R's determinant made +1 by negating R and P; t solved from K t = P[:, 3].
    """
    P = np.array(P[:3, :4], dtype=np.float64)
    K, R = linalg.rq(P[:, :3])
    negative = [K[i, i] < 0 for i in range(3)]
    if sum(negative) in (1, 3):
        K, R = -K, -R
    d = np.ones(3)
    if K[0, 0] < 0 and K[1, 1] < 0:
        d = np.array([-1.0, -1.0, 1.0])
    elif K[0, 0] < 0 and K[2, 2] < 0:
        d = np.array([-1.0, 1.0, -1.0])
    elif K[1, 1] < 0 and K[2, 2] < 0:
        d = np.array([1.0, -1.0, -1.0])
    F = np.diag(d)
    K = K @ F
    R = F @ R
    s = K[2, 2]
    K = K / s
    P = P / s
    if np.linalg.det(R) < 0.0:
        R = -R
        P = -P
    t = linalg.lstsq(K, P[:, 3:4])[0]
    return K, R, t


def dlt_matrix(xx, yy, zz, col, row):
    """The 2N x 12 DLT system of lib/solve_perspective.py:98-110."""
    n = xx.size
    X = np.hstack((xx.reshape(-1, 1), yy.reshape(-1, 1), zz.reshape(-1, 1), np.ones((n, 1))))
    c = col.reshape(-1, 1)
    r = row.reshape(-1, 1)
    Z = np.zeros((n, 4))
    return np.vstack((np.hstack((X, Z, -c * X)), np.hstack((Z, X, -r * X))))


def solve_perspective(xx, yy, zz, col, row, keep_mask=None):
    """(K, R, t) of the perspective camera closest to the correspondences in the
    algebraic (DLT) sense: the right singular vector of the smallest singular value."""
    sizes = [a.size for a in (xx, yy, zz, col, row)]
    assert all(s == sizes[0] for s in sizes)
    if keep_mask is not None:
        m = np.asarray(keep_mask).reshape(-1)
        xx, yy, zz, col, row = (a.reshape(-1)[m] for a in (xx, yy, zz, col, row))
    A = dlt_matrix(xx, yy, zz, col, row)
    _, _, vh = linalg.svd(A, full_matrices=False)
    P = np.real(vh[11, :]).reshape(3, 4)
    return factorize(P)


def perspective_error(xx, yy, zz, col, row, K, R, t, keep_mask=None):
    """(mean, median, max) pixel reprojection error and (mean, median, max) metric
    inverse-projection error, as lib/check_error.py:37-121 defines them."""
    if keep_mask is not None:
        m = np.asarray(keep_mask).reshape(-1)
        xx, yy, zz, col, row = (a.reshape(-1)[m].reshape(-1, 1) for a in (xx, yy, zz, col, row))
    else:
        xx, yy, zz, col, row = (a.reshape(-1, 1) for a in (xx, yy, zz, col, row))
    n = xx.size
    ones = np.ones((n, 1))
    cam = np.hstack((xx, yy, zz)) @ R.T + np.tile(t.T, (n, 1))
    P_hat = K @ np.hstack((R, t))
    h = np.hstack((xx, yy, zz, ones)) @ P_hat.T
    est_col = h[:, 0:1] / h[:, 2:3]
    est_row = h[:, 1:2] / h[:, 2:3]
    proj_err = np.sqrt((est_row - row) ** 2 + (est_col - col) ** 2)
    ray = np.hstack((col, row, ones)) @ np.linalg.inv(K.T)
    scale = (cam * ray).sum(axis=1, keepdims=True) / (ray * ray).sum(axis=1, keepdims=True)
    inv_err = np.sqrt(((ray * scale - cam) ** 2).sum(axis=1, keepdims=True))
    return (float(np.mean(proj_err)), float(np.median(proj_err)), float(np.max(proj_err)),
            float(np.mean(inv_err)), float(np.median(inv_err)), float(np.max(inv_err)))


def camera_params(width, height, K, R, t):
    """[w, h, fx, fy, cx, cy, s, qw, qx, qy, qz, tx, ty, tz] (camera_approx.py:178-182)."""
    q = quaternion_from_rotation(R)
    return [width, height, K[0, 0], K[1, 1], K[0, 2], K[1, 2], K[0, 1],
            q[0], q[1], q[2], q[3], t[0, 0], t[1, 0], t[2, 0]]


def reproject(K, R, t, xx, yy, zz):
    """(col, row) of ENU points through K [R | t]."""
    P = K @ np.hstack((R, t))
    X = np.hstack((xx.reshape(-1, 1), yy.reshape(-1, 1), zz.reshape(-1, 1), np.ones((xx.size, 1))))
    h = X @ P.T
    return h[:, 0] / h[:, 2], h[:, 1] / h[:, 2]
