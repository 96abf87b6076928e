"""Oracle (test infrastructure only): CPU restatement of the depth map -> UTM points chain.

Reference: ``aggregate_2p5d_util.py:75-98`` (``convert_depth_map_worker``): depth <= 0 becomes
NaN, every pixel (col, row, 1, depth) goes through the view's 4x4 inverse projection matrix
with a homogeneous divide, pixels whose z is NaN are dropped (pixel order kept), ENU is
converted to lat/lon/alt (``coordinate_system.py:41-50`` -> ``pymap3d.enu2geodetic``) and
lat/lon to UTM (``lib/latlon_utm_converter.py:38-52`` -> ``utm.from_latlon`` for the zone,
``pyproj.Proj(proj='utm', ellps='WGS84')`` for the projection).

The three third-party libraries are pinned in the reference's ``requirements.txt`` and are
absent here: pymap3d==1.7.15, utm==0.4.2, pyproj==2.4.0 (PROJ 6).  Their published
algorithms are restated:

* ENU -> ECEF: the rotation of (east, north, up) by the origin's latitude/longitude plus the
  origin's ECEF position (pymap3d ``enu2ecef``).
* ECEF -> geodetic: You, Rey-Jer (2000), "Transformation of Cartesian to Geodetic
  Coordinates without Iterations", J. Surveying Eng. 126(1): reduced latitude from the
  confocal-ellipsoid semi-minor axis, one closed-form correction, then latitude, longitude
  and height (the method pymap3d's ``ecef2geodetic`` names).
* UTM zone: 6-degree zones from -180 with the Norway (32V) and Svalbard exceptions
  (utm ``latlon_to_zone_number``).
* Transverse Mercator: Krueger's series in the third flattening n to order n^6 (Krueger
  1912; coefficients as tabulated by Karney 2011, "Transverse Mercator with an accuracy of a
  few nanometers", J. Geodesy 85), k0 = 0.9996, false easting 500 km, false northing
  10,000 km in the south.  PROJ 6's default ``utm`` is this series (Poder/Engsager).

Parity against pymap3d/pyproj themselves is unpinned (they are not installed).  The
restatement is pinned by identities instead: the series on the central meridian equals the
numerically integrated meridian arc (which fixes every alpha_j and the rectifying radius),
the forward and inverse series invert each other, and ENU -> geodetic inverts the textbook
geodetic -> ENU conversion.
"""
import numpy as np

WGS84_A = 6378137.0
WGS84_F = 1.0 / 298.257223563
WGS84_B = WGS84_A * (1.0 - WGS84_F)
WGS84_E2 = WGS84_F * (2.0 - WGS84_F)
UTM_K0 = 0.9996
UTM_FE = 500000.0
UTM_FN_SOUTH = 10000000.0

_N = WGS84_F / (2.0 - WGS84_F)          # third flattening


def _series():
    n = _N
    n2, n3, n4, n5, n6 = n * n, n ** 3, n ** 4, n ** 5, n ** 6
    alpha = [
        n / 2 - 2 * n2 / 3 + 5 * n3 / 16 + 41 * n4 / 180 - 127 * n5 / 288 + 7891 * n6 / 37800,
        13 * n2 / 48 - 3 * n3 / 5 + 557 * n4 / 1440 + 281 * n5 / 630 - 1983433 * n6 / 1935360,
        61 * n3 / 240 - 103 * n4 / 140 + 15061 * n5 / 26880 + 167603 * n6 / 181440,
        49561 * n4 / 161280 - 179 * n5 / 168 + 6601661 * n6 / 7257600,
        34729 * n5 / 80640 - 3418889 * n6 / 1995840,
        212378941 * n6 / 319334400,
    ]
    beta = [
        n / 2 - 2 * n2 / 3 + 37 * n3 / 96 - n4 / 360 - 81 * n5 / 512 + 96199 * n6 / 604800,
        n2 / 48 + n3 / 15 - 437 * n4 / 1440 + 46 * n5 / 105 - 1118711 * n6 / 3870720,
        17 * n3 / 480 - 37 * n4 / 840 - 209 * n5 / 4480 + 5569 * n6 / 90720,
        4397 * n4 / 161280 - 11 * n5 / 504 - 830251 * n6 / 7257600,
        4583 * n5 / 161280 - 108847 * n6 / 3991680,
        20648693 * n6 / 638668800,
    ]
    rect = WGS84_A / (1 + n) * (1 + n2 / 4 + n4 / 64 + n6 / 256)
    return np.array(alpha), np.array(beta), rect


ALPHA, BETA, RECT_A = _series()


def geodetic_to_ecef(lat, lon, alt):
    phi, lam = np.radians(lat), np.radians(lon)
    s = np.sin(phi)
    nu = WGS84_A / np.sqrt(1.0 - WGS84_E2 * s * s)
    return ((nu + alt) * np.cos(phi) * np.cos(lam), (nu + alt) * np.cos(phi) * np.sin(lam),
            (nu * (1.0 - WGS84_E2) + alt) * s)


def enu_to_ecef(e, n, u, lat0, lon0, alt0):
    """pymap3d ``enu2ecef``: rotate (e, n, u) into ECEF axes and add the origin."""
    x0, y0, z0 = geodetic_to_ecef(lat0, lon0, alt0)
    phi, lam = np.radians(lat0), np.radians(lon0)
    t = np.cos(phi) * u - np.sin(phi) * n
    w = np.sin(phi) * u + np.cos(phi) * n
    du = np.cos(lam) * t - np.sin(lam) * e
    dv = np.sin(lam) * t + np.cos(lam) * e
    return x0 + du, y0 + dv, z0 + w


def ecef_to_geodetic(x, y, z):
    """You (2000): (x, y, z) metres -> (lat, lon) degrees, alt metres."""
    a, b = WGS84_A, WGS84_B
    x, y, z = (np.asarray(v, dtype=np.float64) for v in (x, y, z))
    r = np.sqrt(x * x + y * y + z * z)
    E = np.sqrt(a * a - b * b)
    u = np.sqrt(0.5 * (r * r - E * E) + 0.5 * np.sqrt((r * r - E * E) ** 2 + 4.0 * E * E * z * z))
    Q = np.hypot(x, y)
    huE = np.hypot(u, E)
    with np.errstate(divide='ignore', invalid='ignore'):
        beta = np.arctan(huE / u * z / Q)
        eps = ((b * u - a * huE + E * E) * np.sin(beta)) / (a * huE / np.cos(beta) - E * E * np.cos(beta))
    beta = beta + eps
    lat = np.arctan(a / b * np.tan(beta))
    lon = np.arctan2(y, x)
    alt = np.hypot(z - b * np.sin(beta), Q - a * np.cos(beta))
    inside = x * x / (a * a) + y * y / (a * a) + z * z / (b * b) < 1.0
    alt = np.where(inside, -alt, alt)
    return np.degrees(lat), np.degrees(lon), alt


def enu_to_geodetic(e, n, u, lat0, lon0, alt0):
    """``coordinate_system.local_to_global`` -> pymap3d ``enu2geodetic``."""
    return ecef_to_geodetic(*enu_to_ecef(e, n, u, lat0, lon0, alt0))


def utm_zone(lat, lon):
    """utm 0.4.2 ``latlon_to_zone_number`` (scalar)."""
    if 56 <= lat < 64 and 3 <= lon < 12:
        return 32
    if 72 <= lat <= 84 and lon >= 0:
        if lon < 9:
            return 31
        if lon < 21:
            return 33
        if lon < 33:
            return 35
        if lon < 42:
            return 37
    return int((lon + 180) / 6) + 1


def central_meridian(zone):
    return (zone - 1) * 6 - 180 + 3


def geodetic_to_utm(lat, lon, zone, south):
    """Krueger series transverse Mercator: (lat, lon) degrees -> (east, north) metres."""
    e = np.sqrt(WGS84_E2)
    phi = np.radians(np.asarray(lat, dtype=np.float64))
    dlam = np.radians(np.asarray(lon, dtype=np.float64) - central_meridian(zone))
    tau = np.tan(phi)
    sig = np.sinh(e * np.arctanh(e * tau / np.sqrt(1.0 + tau * tau)))
    taup = tau * np.sqrt(1.0 + sig * sig) - sig * np.sqrt(1.0 + tau * tau)
    xip = np.arctan2(taup, np.cos(dlam))
    etap = np.arcsinh(np.sin(dlam) / np.sqrt(taup * taup + np.cos(dlam) ** 2))
    xi, eta = xip.copy(), etap.copy()
    for j in range(1, 7):
        xi = xi + ALPHA[j - 1] * np.sin(2 * j * xip) * np.cosh(2 * j * etap)
        eta = eta + ALPHA[j - 1] * np.cos(2 * j * xip) * np.sinh(2 * j * etap)
    east = UTM_FE + UTM_K0 * RECT_A * eta
    north = UTM_K0 * RECT_A * xi + (UTM_FN_SOUTH if south else 0.0)
    return east, north


def utm_to_geodetic(east, north, zone, south):
    """Inverse Krueger series (beta coefficients) with Newton iteration on the conformal
    latitude: (east, north) metres -> (lat, lon) degrees.  Used to check the forward series."""
    e = np.sqrt(WGS84_E2)
    xi = (np.asarray(north, dtype=np.float64) - (UTM_FN_SOUTH if south else 0.0)) / (UTM_K0 * RECT_A)
    eta = (np.asarray(east, dtype=np.float64) - UTM_FE) / (UTM_K0 * RECT_A)
    xip, etap = xi.copy(), eta.copy()
    for j in range(1, 7):
        xip = xip - BETA[j - 1] * np.sin(2 * j * xi) * np.cosh(2 * j * eta)
        etap = etap - BETA[j - 1] * np.cos(2 * j * xi) * np.sinh(2 * j * eta)
    taup = np.sin(xip) / np.sqrt(np.sinh(etap) ** 2 + np.cos(xip) ** 2)
    dlam = np.arctan2(np.sinh(etap), np.cos(xip))
    tau = taup.copy()
    for _ in range(6):                     # Newton on tau' (tau), Karney 2011 eqs. 19-21
        sig = np.sinh(e * np.arctanh(e * tau / np.sqrt(1.0 + tau * tau)))
        tp = tau * np.sqrt(1.0 + sig * sig) - sig * np.sqrt(1.0 + tau * tau)
        d = (taup - tp) / np.sqrt(1.0 + tp * tp) * (1.0 + (1.0 - WGS84_E2) * tau * tau) / (
            (1.0 - WGS84_E2) * np.sqrt(1.0 + tau * tau))
        tau = tau + d
    return np.degrees(np.arctan(tau)), np.degrees(dlam) + central_meridian(zone)


def latlon_to_eastnorth(lat, lon):
    """``lib/latlon_utm_converter.latlon_to_eastnorh``: zone and hemisphere from the first
    point, all points projected in that zone.  Returns (east, north, zone, south)."""
    lat = np.asarray(lat, dtype=np.float64)
    lon = np.asarray(lon, dtype=np.float64)
    assert np.all(lat >= 0) or np.all(lat < 0)
    first_lat, first_lon = float(lat.reshape(-1)[0]), float(lon.reshape(-1)[0])
    south = first_lat < 0
    zone = utm_zone(first_lat, first_lon)
    east, north = geodetic_to_utm(lat, lon, zone, south)
    return east, north, zone, south


def depth_to_enu(depth_map, inv_proj_mat):
    """``aggregate_2p5d_util.py:78-91``: (H, W) float32 depth -> (valid ENU points (N, 3),
    valid mask (H*W,)).  Pixel order is row-major; the arithmetic is FP64 as in numpy."""
    depth = np.array(depth_map, dtype=np.float32, copy=True)
    depth[depth <= 0.0] = np.nan
    h, w = depth.shape
    row, col = np.meshgrid(np.arange(h), np.arange(w), indexing='ij')
    tmp = np.vstack((col.reshape(1, -1), row.reshape(1, -1), np.ones((1, w * h)), depth.reshape(1, -1)))
    tmp = np.dot(np.asarray(inv_proj_mat, dtype=np.float64), tmp)
    with np.errstate(divide='ignore', invalid='ignore'):
        tmp[0, :] /= tmp[3, :]
        tmp[1, :] /= tmp[3, :]
        tmp[2, :] /= tmp[3, :]
    valid = np.logical_not(np.isnan(tmp[2, :]))
    return tmp[0:3, valid].T, valid


def depth_to_points(depth_map, inv_proj_mat, lat0, lon0, alt0):
    """``aggregate_2p5d_util.py:78-98``: UTM points (N, 3) [east, north, alt] of the valid
    pixels, plus (zone, south)."""
    enu, _ = depth_to_enu(depth_map, inv_proj_mat)
    lat, lon, alt = enu_to_geodetic(enu[:, 0], enu[:, 1], enu[:, 2], lat0, lon0, alt0)
    east, north, zone, south = latlon_to_eastnorth(lat, lon)
    return np.stack([east, north, alt], axis=1), zone, south


def read_array(path):
    """COLMAP dense array (``colmap/read_dense.py:36-51``): ASCII "width&height&channels&"
    then float32 in column-major (width, height, channels) order -> (height, width[, ch])."""
    with open(path, 'rb') as f:
        raw = f.read()
    pos, fields = 0, []
    while len(fields) < 3:
        amp = raw.index(b'&', pos)
        fields.append(int(raw[pos:amp]))
        pos = amp + 1
    w, h, c = fields
    arr = np.frombuffer(raw[pos:], dtype=np.float32).reshape((w, h, c), order='F')
    return np.transpose(arr, (1, 0, 2)).squeeze()
