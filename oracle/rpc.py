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
