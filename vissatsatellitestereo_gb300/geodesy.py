"""WGS-84 geodetic -> ENU conversion (input preparation for the perspective fit).

The reference converts its lat/lon/alt sample grid to a local ENU frame with
``pymap3d.geodetic2enu`` (``lib/latlonalt_enu_converter.py:36-39``), origin at the AOI
centre latitude/longitude and the lowest altitude (``coordinate_system.py:45-47``).
pymap3d is not available here, so this is the textbook conversion written out in
FP64: geodetic -> ECEF with the WGS-84 prime-vertical radius, then the ECEF offset
from the origin rotated into east/north/up.
"""
import numpy as np

WGS84_A = 6378137.0
WGS84_F = 1.0 / 298.257223563
WGS84_E2 = WGS84_F * (2.0 - WGS84_F)


def geodetic_to_ecef(lat, lon, alt):
    phi = np.radians(lat)
    lam = np.radians(lon)
    sphi = np.sin(phi)
    n = WGS84_A / np.sqrt(1.0 - WGS84_E2 * sphi * sphi)
    x = (n + alt) * np.cos(phi) * np.cos(lam)
    y = (n + alt) * np.cos(phi) * np.sin(lam)
    z = (n * (1.0 - WGS84_E2) + alt) * sphi
    return x, y, z


def geodetic_to_enu(lat, lon, alt, lat0, lon0, alt0):
    """(east, north, up) metres of lat/lon/alt about the origin (lat0, lon0, alt0)."""
    x, y, z = geodetic_to_ecef(lat, lon, alt)
    x0, y0, z0 = geodetic_to_ecef(lat0, lon0, alt0)
    dx, dy, dz = x - x0, y - y0, z - z0
    phi0 = np.radians(lat0)
    lam0 = np.radians(lon0)
    sp, cp = np.sin(phi0), np.cos(phi0)
    sl, cl = np.sin(lam0), np.cos(lam0)
    east = -sl * dx + cl * dy
    t = cl * dx + sl * dy
    north = -sp * t + cp * dz
    up = cp * t + sp * dz
    return east, north, up
