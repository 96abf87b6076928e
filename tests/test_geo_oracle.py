"""The depth map -> UTM chain's oracle and host logic, on the CPU.

pymap3d 1.7.15, utm 0.4.2 and pyproj 2.4.0 (the reference's geodesy) are absent, so the
oracle's restatements are pinned by identities: the transverse Mercator series on the
central meridian equals the numerically integrated meridian arc (which fixes every series
coefficient and the rectifying radius), forward and inverse series invert each other, and
ENU -> geodetic inverts the textbook geodetic -> ENU conversion.  The depth -> ENU stage and
the COLMAP array format are pinned by fixtures made with the reference's own code
(``tests/golden/make_golden.py --sections depth``).
"""
import os

import numpy as np
import pytest

from oracle import geo

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def test_transverse_mercator_matches_meridian_arc():
    quad = pytest.importorskip('scipy.integrate').quad
    a, e2 = geo.WGS84_A, geo.WGS84_E2
    for lat in np.linspace(-84.0, 84.0, 29):
        arc = quad(lambda p: a * (1 - e2) / (1 - e2 * np.sin(p) ** 2) ** 1.5, 0.0, np.radians(lat),
                   epsabs=1e-12, epsrel=1e-15, limit=200)[0]
        east, north = geo.geodetic_to_utm(np.array([lat]), np.array([27.0]), 35, False)
        assert east[0] == 500000.0
        assert abs(north[0] - geo.UTM_K0 * arc) < 2e-8, lat


def test_transverse_mercator_round_trip_and_conformality():
    rng = np.random.default_rng(3)
    lat = rng.uniform(-80.0, 84.0, 20000)
    lon = geo.central_meridian(31) + rng.uniform(-3.5, 3.5, 20000)
    east, north = geo.geodetic_to_utm(lat, lon, 31, False)
    la, lo = geo.utm_to_geodetic(east, north, 31, False)
    assert np.abs(la - lat).max() < 1e-12 and np.abs(lo - lon).max() < 1e-12
    # conformal: equal scale along the meridian and the parallel
    a, e2 = geo.WGS84_A, geo.WGS84_E2
    for phi, dl in ((45.0, 1.0), (-20.0, 2.5), (60.0, -3.0)):
        h = 1e-6
        e0, n0 = geo.geodetic_to_utm(np.array([phi]), np.array([3.0 + dl]), 31, False)
        e1, n1 = geo.geodetic_to_utm(np.array([phi + h]), np.array([3.0 + dl]), 31, False)
        e2_, n2 = geo.geodetic_to_utm(np.array([phi]), np.array([3.0 + dl + h]), 31, False)
        s = np.sin(np.radians(phi))
        M = a * (1 - e2) / (1 - e2 * s * s) ** 1.5
        nu = a / np.sqrt(1 - e2 * s * s)
        k1 = np.hypot(e1 - e0, n1 - n0)[0] / (M * np.radians(h))
        k2 = np.hypot(e2_ - e0, n2 - n0)[0] / (nu * np.cos(np.radians(phi)) * np.radians(h))
        assert abs(k1 - k2) < 1e-7


def test_enu_to_geodetic_inverts_geodetic_to_enu():
    from vissatsatellitestereo_gb300.geodesy import geodetic_to_enu
    # the reference's own demonstration case (lib/latlonalt_enu_converter.py __main__)
    e, n, u = geodetic_to_enu(-34.450, -58.579, 20.31, -34.448, -58.577, -30.0)
    lat, lon, alt = geo.enu_to_geodetic(e, n, u, -34.448, -58.577, -30.0)
    assert abs(lat + 34.450) < 1e-12 and abs(lon + 58.579) < 1e-12 and abs(alt - 20.31) < 1e-8
    rng = np.random.default_rng(4)
    lat0, lon0, alt0 = 39.7, -84.1, -30.0
    la = lat0 + rng.uniform(-0.05, 0.05, 5000)
    lo = lon0 + rng.uniform(-0.05, 0.05, 5000)
    al = rng.uniform(-100.0, 500.0, 5000)
    e, n, u = geodetic_to_enu(la, lo, al, lat0, lon0, alt0)
    la2, lo2, al2 = geo.enu_to_geodetic(e, n, u, lat0, lon0, alt0)
    assert np.abs(la2 - la).max() < 1e-13 and np.abs(lo2 - lo).max() < 1e-13 and np.abs(al2 - al).max() < 1e-8


def test_utm_zone_rule():
    from vissatsatellitestereo_gb300.coordinate_system import utm_zone
    assert utm_zone(47.9941214, 7.8509671) == 32          # lib/latlon_utm_converter.py __main__
    assert utm_zone(60.0, 5.0) == 32                       # Norway
    assert utm_zone(78.0, 15.0) == 33 and utm_zone(78.0, 35.0) == 37   # Svalbard
    assert utm_zone(-33.9, 18.4) == 34 and utm_zone(39.77, -84.05) == 16
    rng = np.random.default_rng(5)
    for la, lo in zip(rng.uniform(-80, 84, 2000), rng.uniform(-180, 179.99, 2000)):
        assert utm_zone(la, lo) == geo.utm_zone(la, lo)


def test_depth_to_enu_matches_reference_block():
    g = np.load(os.path.join(GOLDEN, 'depth_enu.npz'))
    for v in range(2):
        enu, valid = geo.depth_to_enu(g[f'v{v}_depth'], g[f'v{v}_inv_proj'])
        assert np.array_equal(valid, g[f'v{v}_valid'])
        np.testing.assert_allclose(enu, g[f'v{v}_points4'][:, :3], rtol=1e-14, atol=1e-9)
        assert valid.sum() < valid.size                      # holes, NaN and inf planted


def test_colmap_arrays_match_reference_reader():
    from vissatsatellitestereo_gb300 import io_formats
    g = np.load(os.path.join(GOLDEN, 'colmap_arrays.npz'))
    for name in ('depth', 'normal'):
        path = os.path.join(GOLDEN, f'colmap_{name}.bin')
        ours = io_formats.read_array(path)
        assert ours.shape == g[f'{name}_read'].shape and np.array_equal(ours, g[f'{name}_read'])
        assert np.array_equal(geo.read_array(path), g[f'{name}_read'])


def test_colmap_array_writer_bytes(tmp_path):
    from vissatsatellitestereo_gb300 import io_formats
    g = np.load(os.path.join(GOLDEN, 'colmap_arrays.npz'))
    for name in ('depth', 'normal'):
        out = tmp_path / f'{name}.bin'
        io_formats.write_array(g[f'{name}_written'], str(out))
        assert out.read_bytes() == open(os.path.join(GOLDEN, f'colmap_{name}.bin'), 'rb').read()


def test_inv_proj_mats_round_trip(tmp_path):
    from vissatsatellitestereo_gb300 import io_formats
    rng = np.random.default_rng(6)
    mats = {f'{i:04d}.png': rng.normal(0.0, 1e5, (4, 4)) for i in range(5)}
    path = tmp_path / 'inv_proj_mats.txt'
    io_formats.write_inv_proj_mats(mats, str(path))
    back = io_formats.read_inv_proj_mats(str(path))
    assert list(back) == list(mats)
    for k in mats:
        assert np.array_equal(back[k], mats[k])


def test_synthetic_depth_case_lands_on_the_grid():
    from vissatsatellitestereo_gb300 import synth

    def utm(la, lo, z, s):
        e, n = geo.geodetic_to_utm(np.array([la]), np.array([lo]), z, s)
        return float(e[0]), float(n[0])

    case = synth.make_depth_case(11, 2, 64, 64, utm, aoi_m=200.0, n_boxes=10)
    aoi = case.aoi
    lat0 = (aoi['lat_min'] + aoi['lat_max']) / 2
    lon0 = (aoi['lon_min'] + aoi['lon_max']) / 2
    d = synth.depth_map_torch(case, 0).numpy()
    pts, zone, south = geo.depth_to_points(d, case.inv_proj[0], lat0, lon0, aoi['alt_min'])
    assert zone == aoi['zone_number'] and not south
    assert 0.75 < len(pts) / d.size < 0.95
    inside = ((pts[:, 0] >= aoi['ul_easting']) & (pts[:, 0] < aoi['ul_easting'] + aoi['width']) &
              (pts[:, 1] <= aoi['ul_northing']) & (pts[:, 1] > aoi['ul_northing'] - aoi['height']))
    assert inside.mean() > 0.5
    assert -32.0 < pts[:, 2].min() and pts[:, 2].max() < 60.0


def test_aoi_host_logic(tmp_path):
    """aoi.json read from a work dir like coordinate_system.py:42-47, the ENU origin (centre
    latitude/longitude, lowest altitude), a fast-path box that holds the AOI's ENU extent,
    and produce_dsm's grid (int(width / 0.5) + 1 cells from the upper-left corner)."""
    import json
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import aoi_grid
    from vissatsatellitestereo_gb300.coordinate_system import aoi_enu_box, aoi_origin, load_aoi
    from vissatsatellitestereo_gb300.geodesy import geodetic_to_enu
    aoi = {'lat_min': 39.76, 'lat_max': 39.78, 'lon_min': -84.06, 'lon_max': -84.04, 'alt_min': -30.0,
           'alt_max': 120.0, 'ul_easting': 752374.0, 'ul_northing': 4406693.0, 'width': 713.0, 'height': 651.0,
           'zone_number': 16, 'hemisphere': 'N'}
    (tmp_path / 'aoi.json').write_text(json.dumps(aoi))
    assert load_aoi(str(tmp_path)) == aoi
    lat0, lon0, alt0 = aoi_origin(str(tmp_path))
    assert (lat0, lon0, alt0) == ((39.76 + 39.78) / 2.0, (-84.06 + -84.04) / 2.0, -30.0)   # :44-46
    lo, hi = aoi_enu_box(aoi)
    for la in (aoi['lat_min'], aoi['lat_max']):
        for lo_ in (aoi['lon_min'], aoi['lon_max']):
            for al in (aoi['alt_min'], aoi['alt_max']):
                e, n, u = geodetic_to_enu(la, lo_, al, lat0, lon0, alt0)
                assert lo[0] < e < hi[0] and lo[1] < n < hi[1] and lo[2] < u < hi[2]
    assert aoi_grid(aoi) == (752374.0, 4406693.0, 0.5, 0.5, 1427, 1303)


def test_ecef_to_geodetic_matches_an_independent_iteration():
    """You (2000), as restated, against the textbook fixed-point iteration on the latitude
    (tan(phi) = (z + e^2 nu sin(phi)) / p, run to convergence) over the globe, poles and
    equator included.  The published method applies one closed-form correction, so its
    latitude error grows with the height above the ellipsoid: ~2e-9 m at terrain heights
    (the depth-map points), ~1e-6 m at 10-100 km, ~2e-3 m at 700 km; heights stay exact."""
    rng = np.random.default_rng(9)
    lat = np.concatenate([rng.uniform(-89.9, 89.9, 3000), [89.999, -89.999, 0.0, 45.0]])
    lon = np.concatenate([rng.uniform(-180.0, 180.0, 3000), [10.0, -20.0, 0.0, 179.9]])
    alt = np.concatenate([rng.uniform(-400.0, 8000.0, 2000), rng.uniform(1e4, 7e5, 1000), [0.0, 100.0, 0.0, 6e5]])
    x, y, z = geo.geodetic_to_ecef(lat, lon, alt)
    la, lo, al = geo.ecef_to_geodetic(x, y, z)
    a, e2 = geo.WGS84_A, geo.WGS84_E2
    p = np.hypot(x, y)
    phi = np.arctan2(z, p * (1.0 - e2))
    for _ in range(20):
        nu = a / np.sqrt(1.0 - e2 * np.sin(phi) ** 2)
        phi = np.arctan2(z + e2 * nu * np.sin(phi), p)
    nu = a / np.sqrt(1.0 - e2 * np.sin(phi) ** 2)
    h = np.where(np.abs(np.cos(phi)) > 1e-3, p / np.cos(phi) - nu, z / np.sin(phi) - nu * (1.0 - e2))
    dlat_m = np.abs(np.degrees(phi) - la) * 111320.0                    # metres along the meridian
    terrain, high, sat = alt <= 8000.0, (alt > 8000.0) & (alt <= 1e5), alt > 1e5
    assert dlat_m[terrain].max() < 1e-8 and dlat_m[high].max() < 5e-6 and dlat_m[sat].max() < 5e-3
    assert np.abs(h - al).max() < 1e-6
    assert np.abs(lo - lon).max() < 1e-10
    assert (np.abs(la - lat) * 111320.0)[terrain].max() < 1e-8 and np.abs(al - alt).max() < 1e-6


def test_proj_path_matches_closed_form_transverse_mercator():
    """The restated PROJ 6.2 utm path (Gaussian latitude by Clenshaw, complex Clenshaw of
    Krueger's series) against an independent closed form (exact conformal latitude, direct
    series) over the UTM domain of every latitude band, both hemispheres' false northings."""
    rng = np.random.default_rng(11)
    lat = rng.uniform(-80.0, 84.0, 100000)
    for zone in (1, 21, 33, 60):
        lon = geo.central_meridian(zone) + rng.uniform(-3.5, 3.5, lat.size)
        for south in (False, True):
            e1, n1 = geo.geodetic_to_utm(lat, lon, zone, south)
            e2, n2 = geo.geodetic_to_utm_karney(lat, lon, zone, south)
            assert np.abs(e1 - e2).max() < 2e-8 and np.abs(n1 - n2).max() < 2e-8
