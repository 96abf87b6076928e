"""Oracle: RPC projection (test infrastructure only).

Restates ``apply_poly`` (lib/rpc_model.py:40-63), ``apply_rfm`` (:66-79) and
``RPCModel.projection`` (:160-168) in FP64 numpy.  The accumulation grouping below is
the reference's line-by-line grouping: the FP64 result depends on it, and the golden
vectors check this restatement bit-for-bit against the reference module.
"""
import numpy as np

# RPC00B monomial order, x = normalised latitude, y = longitude, z = altitude.  Each
# inner tuple is one accumulation line of lib/rpc_model.py:53-62; the letters give the
# multiplication order applied to the coefficient.
POLY_LINES = (
    ((0, ''),),
    ((1, 'y'), (2, 'x'), (3, 'z')),
    ((4, 'yx'), (5, 'yz'), (6, 'xz')),
    ((7, 'yy'), (8, 'xx'), (9, 'zz')),
    ((10, 'xyz'),),
    ((11, 'yyy'),),
    ((12, 'yxx'), (13, 'yzz'), (14, 'yyx')),
    ((15, 'xxx'),),
    ((16, 'xzz'), (17, 'yyz'), (18, 'xxz')),
    ((19, 'zzz'),),
)


def apply_poly(poly, x, y, z):
    var = {'x': x, 'y': y, 'z': z}
    out = 0
    for line in POLY_LINES:
        line_sum = None
        for k, mono in line:
            term = poly[k]
            for ch in mono:
                term = term * var[ch]
            line_sum = term if line_sum is None else line_sum + term
        out = out + line_sum
    return out


def apply_rfm(num, den, x, y, z):
    return apply_poly(num, x, y, z) / apply_poly(den, x, y, z)


def projection(meta, lat, lon, alt):
    """(col, row) of lat/lon/alt through the RPC camera ``meta`` (a meta_dict)."""
    r = meta['rpc']
    c_lon = (lon - r['lonOff']) / r['lonScale']
    c_lat = (lat - r['latOff']) / r['latScale']
    c_alt = (alt - r['altOff']) / r['altScale']
    c_col = apply_rfm(r['colNum'], r['colDen'], c_lat, c_lon, c_alt)
    c_row = apply_rfm(r['rowNum'], r['rowDen'], c_lat, c_lon, c_alt)
    return c_col * r['colScale'] + r['colOff'], c_row * r['rowScale'] + r['rowOff']


def in_image(meta, col, row):
    """keep mask of camera_approx.py:170-174."""
    return (col >= 0) & (row >= 0) & (col < meta['width']) & (row < meta['height'])


def projection_normalized(meta, x, y, z):
    """(col, row) for points already in the camera's normalised frame (FP64)."""
    r = meta['rpc']
    c_col = apply_rfm(r['colNum'], r['colDen'], x, y, z)
    c_row = apply_rfm(r['rowNum'], r['rowDen'], x, y, z)
    return c_col * r['colScale'] + r['colOff'], c_row * r['rowScale'] + r['rowOff']


def inverse_projection(meta, col, row, alt, return_normalized=False, max_iter=1000):
    """RPCModel.inverse_projection (lib/rpc_model.py:170-249): (lon, lat, alt) of image
    points at given altitudes.  Newton-like iteration in the normalised frame from
    lon = lat = -1, with finite-difference directions of step 2 in the first iteration and
    0.1 after; every point is updated until all of them reproject within sqrt(1e-18) of
    their target (one shared iteration count).  Returns the iteration count as well."""
    r = meta['rpc']
    c_col = (col - r['colOff']) / r['colScale']
    c_row = (row - r['rowOff']) / r['rowScale']
    c_alt = (alt - r['altOff']) / r['altScale']
    shape = np.shape(c_col)
    c_col, c_row, c_alt = (np.ravel(a).astype(np.float64) for a in (c_col, c_row, c_alt))
    lon = -np.ones(c_col.size)
    lat = -np.ones(c_col.size)
    eps = 2.0

    def frames(lat, lon, eps):
        x0 = apply_rfm(r['colNum'], r['colDen'], lat, lon, c_alt)
        y0 = apply_rfm(r['rowNum'], r['rowDen'], lat, lon, c_alt)
        x1 = apply_rfm(r['colNum'], r['colDen'], lat, lon + eps, c_alt)
        y1 = apply_rfm(r['rowNum'], r['rowDen'], lat, lon + eps, c_alt)
        x2 = apply_rfm(r['colNum'], r['colDen'], lat + eps, lon, c_alt)
        y2 = apply_rfm(r['rowNum'], r['rowDen'], lat + eps, lon, c_alt)
        return x0, y0, x1, y1, x2, y2

    x0, y0, x1, y1, x2, y2 = frames(lat, lon, eps)
    it = 0
    while not np.all((x0 - c_col) ** 2 + (y0 - c_row) ** 2 < 1e-18):
        if it >= max_iter:
            raise RuntimeError('inverse projection did not converge')
        e1x, e1y = x1 - x0, y1 - y0
        e2x, e2y = x2 - x0, y2 - y0
        ux, uy = c_col - x0, c_row - y0
        a1 = (ux * e1x + uy * e1y) / (e1x * e1x + e1y * e1y)
        a2 = (ux * e2x + uy * e2y) / (e2x * e2x + e2y * e2y)
        lon = lon + a1 * eps
        lat = lat + a2 * eps
        eps = 0.1
        x0, y0, x1, y1, x2, y2 = frames(lat, lon, eps)
        it += 1
    if return_normalized:
        return lon.reshape(shape), lat.reshape(shape), c_alt.reshape(shape), it
    return ((lon * r['lonScale'] + r['lonOff']).reshape(shape), (lat * r['latScale'] + r['latOff']).reshape(shape),
            alt, it)
