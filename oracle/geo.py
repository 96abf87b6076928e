"""Oracle (test infrastructure only): CPU restatement of the depth map -> UTM points chain.

Reference: ``aggregate_2p5d_util.py:75-98`` (``convert_depth_map_worker``): depth <= 0 becomes
NaN, every pixel (col, row, 1, depth) goes through the view's 4x4 inverse projection matrix
with a homogeneous divide, pixels whose z is NaN are dropped (pixel order kept), ENU is
converted to lat/lon/alt (``coordinate_system.py:41-50`` -> ``pymap3d.enu2geodetic``) and
lat/lon to UTM (``lib/latlon_utm_converter.py:38-52`` -> ``utm.from_latlon`` for the zone,
``pyproj.Proj(proj='utm', ellps='WGS84')`` for the projection).

The three third-party libraries are pinned in the reference's ``requirements.txt`` and are
absent here: pymap3d==1.7.15, utm==0.4.2, pyproj==2.4.0 (which bundles PROJ 6.2).  Their
published source is restated step by step (same formulas, same order of operations):

* ENU -> ECEF: pymap3d 1.7.15 ``enu2geodetic`` (pymap3d/enu.py) calls ``enu2ecef``, which
  adds ``enu2uvw``'s rotation of (east, north, up) by the origin's latitude/longitude to
  the origin's ``geodetic2ecef`` (pymap3d/ecef.py): N = a^2 / sqrt(a^2 cos^2 lat +
  b^2 sin^2 lat), x = (N + h) cos lat cos lon, y = (N + h) cos lat sin lon,
  z = (N (b/a)^2 + h) sin lat, with the WGS-84 ellipsoid a = 6378137, f = 1/298.257223563,
  b = a (1 - f).
* ECEF -> geodetic: pymap3d's ``ecef2geodetic`` (pymap3d/ecef.py), the method of You,
  Rey-Jer (2000), "Transformation of Cartesian to Geodetic Coordinates without
  Iterations", J. Surveying Eng. 126(1): reduced latitude from the confocal ellipsoid's
  semi-minor axis u, one closed-form correction, latitude atan(a/b tan beta), height
  hypot(z - b sin beta, Q - a cos beta), negated inside the ellipsoid.
* UTM zone: utm 0.4.2 ``latlon_to_zone_number`` (6-degree zones from -180 with the Norway
  32V and Svalbard exceptions), taken from the first point.
* Transverse Mercator: ``pyproj.Proj(proj='utm', ellps='WGS84', zone=z, south=s)`` runs
  PROJ 6.2's ``utm``, which is the Poder/Engsager extended transverse Mercator
  (src/projections/tmerc.cpp, the former etmerc): pyproj converts degrees with pi/180;
  PROJ subtracts lam0 = (zone - 1 + 0.5) pi / 30 - pi; the geodetic latitude becomes the
  Gaussian (conformal) latitude by the 6-term trig series ``cbg`` summed by Clenshaw
  (``gatg``); the spherical transverse Mercator step (atan2 / hypot / asinh(tan)); the
  6-term Krueger series ``gtu`` summed by complex Clenshaw (``clenS``); x = a Qn Ce + x0,
  y = a Qn Cn + y0 with Qn = k0 / (1 + n) (1 + n^2/4 + n^4/64 + n^6/256), k0 = 0.9996,
  x0 = 500 km, y0 = 10,000 km in the south.

What pins this restatement: the libraries themselves cannot run here, so the oracle is
pinned to their published code paths as restated above, plus checks that do not depend on
the restatement: the series on the central meridian equals the numerically integrated
meridian arc (fixing every coefficient and the rectifying radius), an independent
closed-form transverse Mercator (Karney 2011, "Transverse Mercator with an accuracy of a
few nanometers", J. Geodesy 85: exact conformal latitude, direct series) agrees with the
PROJ path to nanometres, the forward and inverse series invert each other, and ENU ->
geodetic inverts geodetic -> ENU.
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
    """pymap3d 1.7.15 ``geodetic2ecef`` (``get_radius_normal`` for N)."""
    a, b = WGS84_A, WGS84_B
    phi, lam = np.radians(lat), np.radians(lon)
    N = a ** 2 / np.sqrt(a ** 2 * np.cos(phi) ** 2 + b ** 2 * np.sin(phi) ** 2)
    return ((N + alt) * np.cos(phi) * np.cos(lam), (N + alt) * np.cos(phi) * np.sin(lam),
            (N * (b / a) ** 2 + alt) * np.sin(phi))


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


def _proj_coefficients():
    """PROJ 6's etmerc set-up: the 6-term series geodetic -> Gaussian latitude (``cbg``),
    spherical -> ellipsoidal N, E (``gtu``, Krueger's alpha) and Qn, from the third
    flattening n (Engsager and Poder 2007)."""
    n = _N
    cbg = [n * (-2 + n * (2 / 3 + n * (4 / 3 + n * (-82 / 45 + n * (32 / 45 + n * (4642 / 4725)))))),
           n ** 2 * (5 / 3 + n * (-16 / 15 + n * (-13 / 9 + n * (904 / 315 + n * (-1522 / 945))))),
           n ** 3 * (-26 / 15 + n * (34 / 21 + n * (8 / 5 + n * (-12686 / 2835)))),
           n ** 4 * (1237 / 630 + n * (-12 / 5 + n * (-24832 / 14175))),
           n ** 5 * (-734 / 315 + n * (109598 / 31185)),
           n ** 6 * (444337 / 155925)]
    gtu = [n * (0.5 + n * (-2 / 3 + n * (5 / 16 + n * (41 / 180 + n * (-127 / 288 + n * (7891 / 37800)))))),
           n ** 2 * (13 / 48 + n * (-3 / 5 + n * (557 / 1440 + n * (281 / 630 + n * (-1983433 / 1935360))))),
           n ** 3 * (61 / 240 + n * (-103 / 140 + n * (15061 / 26880 + n * (167603 / 181440)))),
           n ** 4 * (49561 / 161280 + n * (-179 / 168 + n * (6601661 / 7257600))),
           n ** 5 * (34729 / 80640 + n * (-3418889 / 1995840)),
           n ** 6 * (212378941 / 319334400)]
    n2 = n * n
    qn = UTM_K0 / (1 + n) * (1 + n2 * (1 / 4 + n2 * (1 / 64 + n2 / 256)))
    return np.array(cbg), np.array(gtu), qn


PROJ_CBG, PROJ_GTU, PROJ_QN = _proj_coefficients()


def _clenshaw_sin(p, B):
    """B + sum_k p[k] sin(2 (k+1) B) by Clenshaw's recurrence (PROJ ``gatg``)."""
    two_cos = 2.0 * np.cos(2.0 * B)
    h1, h2, h = p[-1], 0.0, 0.0
    for k in range(len(p) - 2, -1, -1):
        h = -h2 + two_cos * h1 + p[k]
        h2, h1 = h1, h
    return B + h * np.sin(2.0 * B)


def _clenshaw_complex(a, arg_r, arg_i):
    """(Re, Im) of sum_k a[k] sin((k+1) (arg_r + i arg_i)) by complex Clenshaw (PROJ
    ``clenS``)."""
    sin_r, cos_r = np.sin(arg_r), np.cos(arg_r)
    sinh_i, cosh_i = np.sinh(arg_i), np.cosh(arg_i)
    r = 2.0 * cos_r * cosh_i
    i = -2.0 * sin_r * sinh_i
    hr, hi, hr1, hi1 = a[-1], 0.0, 0.0, 0.0
    for k in range(len(a) - 2, -1, -1):
        hr2, hi2 = hr1, hi1
        hr1, hi1 = hr, hi
        hr = -hr2 + r * hr1 - i * hi1 + a[k]
        hi = -hi2 + i * hr1 + r * hi1
    r = sin_r * cosh_i
    i = cos_r * sinh_i
    return r * hr - i * hi, r * hi + i * hr


def geodetic_to_utm(lat, lon, zone, south):
    """PROJ 6.2 ``utm`` (etmerc forward) as pyproj 2.4 calls it: (lat, lon) degrees ->
    (east, north) metres."""
    deg = np.pi / 180.0
    lam0 = (zone - 1 + 0.5) * np.pi / 30.0 - np.pi
    phi = np.asarray(lat, dtype=np.float64) * deg
    lam = np.asarray(lon, dtype=np.float64) * deg - lam0
    cn = _clenshaw_sin(PROJ_CBG, phi)                       # Gaussian latitude
    sin_cn, cos_cn = np.sin(cn), np.cos(cn)
    sin_ce, cos_ce = np.sin(lam), np.cos(lam)
    cn = np.arctan2(sin_cn, cos_ce * cos_cn)
    ce = np.arctan2(sin_ce * cos_cn, np.hypot(sin_cn, cos_cn * cos_ce))
    ce = np.arcsinh(np.tan(ce))
    dcn, dce = _clenshaw_complex(PROJ_GTU, 2.0 * cn, 2.0 * ce)
    cn = cn + dcn
    ce = ce + dce
    east = WGS84_A * (PROJ_QN * ce) + UTM_FE
    north = WGS84_A * (PROJ_QN * cn) + (UTM_FN_SOUTH if south else 0.0)
    return east, north


def geodetic_to_utm_karney(lat, lon, zone, south):
    """Independent closed-form transverse Mercator (Karney 2011: exact conformal latitude,
    Krueger's series summed directly): (lat, lon) degrees -> (east, north) metres.  Checks
    the PROJ path."""
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
