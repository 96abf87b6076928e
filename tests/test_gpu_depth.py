"""Depth maps -> UTM points -> DSMs on the GPU against the oracle (``oracle/geo.py``).

Tolerances: the device geodesy (FP64 chain, and the validated polynomial fast path) agrees
with the oracle's numpy restatement within 1e-6 m in easting, northing and altitude (the
fast path's plan-time bound is 2.5e-7 m; 1e-6 m is 3e-6 px at 0.3 m).  Everything integer
-- point count, pixel order, DSM bits -- is exact: the fused DSM equals the points path's
DSM and the oracle's proj_to_grid + blur of the GPU's own points bit for bit.
"""
import os

import numpy as np
import pytest
import torch

from conftest import same_bits
from oracle import geo
from oracle.blur import median_blur3x3
from oracle.raster import proj_to_grid

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
TOL_M = 1e-6


def _utm(la, lo, z, s):
    e, n = geo.geodetic_to_utm(np.array([la]), np.array([lo]), z, s)
    return float(e[0]), float(n[0])


def _origin(aoi):
    return (aoi['lat_min'] + aoi['lat_max']) / 2, (aoi['lon_min'] + aoi['lon_max']) / 2, aoi['alt_min']


@pytest.fixture(scope='module')
def case():
    from vissatsatellitestereo_gb300 import synth
    return synth.make_depth_case(21, 3, 200, 264, _utm, aoi_m=300.0, n_boxes=40)


def _oracle_points(depth, M, aoi):
    pts, zone, south = geo.depth_to_points(depth, M, *_origin(aoi))
    return pts


def test_plan_validates_fast_path(case):
    from vissatsatellitestereo_gb300.coordinate_system import aoi_enu_box, aoi_origin, plan_for
    aoi = case.aoi
    plan = plan_for(*aoi_origin(aoi), aoi['zone_number'], False, aoi_enu_box(aoi))
    assert plan.fast_enabled and plan.max_err_m <= 2.5e-7


def test_enu_to_geodetic_and_utm_vs_oracle():
    from vissatsatellitestereo_gb300.coordinate_system import enu_to_geodetic, latlon_to_eastnorh
    rng = np.random.default_rng(7)
    e, n, u = rng.uniform(-3000, 3000, 4000), rng.uniform(-3000, 3000, 4000), rng.uniform(-50, 900, 4000)
    for origin in ((39.77, -84.05, -30.0), (-33.9, 18.4, 12.0), (64.1, -21.9, 0.0)):
        lat, lon, alt = enu_to_geodetic(e, n, u, *origin)
        la, lo, al = geo.enu_to_geodetic(e, n, u, *origin)
        assert np.abs(lat - la).max() < 1e-11 and np.abs(lon - lo).max() < 1e-11 and np.abs(alt - al).max() < TOL_M
        east, north = latlon_to_eastnorh(lat, lon)
        ea, no, zone, south = geo.latlon_to_eastnorth(lat, lon)
        assert np.abs(east - ea).max() < TOL_M and np.abs(north - no).max() < TOL_M


def test_latlon_to_eastnorth_hemisphere_assert():
    from vissatsatellitestereo_gb300.coordinate_system import latlon_to_eastnorh
    with pytest.raises(AssertionError):
        latlon_to_eastnorh(np.array([0.001, -0.001]), np.array([10.0, 10.0]))


@pytest.mark.parametrize('mode', ['fast', 'exact'])
def test_depth_to_points_vs_oracle(case, mode):
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import depth_map_to_points
    for v in range(3):
        d = synth.depth_map_torch(case, v).numpy()
        ours = depth_map_to_points(d, case.inv_proj[v], case.aoi, mode=mode)
        ref = _oracle_points(d, case.inv_proj[v], case.aoi)
        assert ours.shape == ref.shape
        assert np.abs(ours - ref).max() < TOL_M, (v, mode, np.abs(ours - ref).max(axis=0))


def test_depth_to_points_on_reference_enu_golden():
    """Depth maps with holes, NaN and inf: the valid count and order of the reference's own
    depth -> ENU block, and UTM within tolerance of the oracle's geodesy of its ENU points."""
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import depth_map_to_points
    g = np.load(os.path.join(GOLDEN, 'depth_enu.npz'))
    aoi = eval(str(g['aoi']))
    for v in range(2):
        ours = depth_map_to_points(g[f'v{v}_depth'], g[f'v{v}_inv_proj'], aoi)
        enu = g[f'v{v}_points4'][:, :3]
        assert ours.shape[0] == enu.shape[0] == int(g[f'v{v}_valid'].sum())
        lat, lon, alt = geo.enu_to_geodetic(enu[:, 0], enu[:, 1], enu[:, 2], *_origin(aoi))
        east, north, _, _ = geo.latlon_to_eastnorth(lat, lon)
        assert np.abs(ours - np.stack([east, north, alt], 1)).max() < TOL_M


def test_depth_to_points_edges():
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import depth_map_to_points
    case = synth.make_depth_case(23, 1, 37, 29, _utm, aoi_m=80.0, n_boxes=5)
    d = synth.depth_map_torch(case, 0).numpy()
    M = case.inv_proj[0]
    empty = depth_map_to_points(np.full_like(d, -1e20), M, case.aoi)
    assert empty.shape == (0, 3)
    one = depth_map_to_points(d[:1, :1], M, case.aoi)
    assert np.abs(one - _oracle_points(d[:1, :1], M, case.aoi)).max() < TOL_M
    ragged = d[:, :23].copy()                    # width not a multiple of the 8-pixel runs
    ragged[::3, ::2] = 0.0
    ragged[5, 5] = np.nan
    ragged[6, 6] = np.inf
    ours = depth_map_to_points(ragged, M, case.aoi)
    ref = _oracle_points(ragged, M, case.aoi)
    assert ours.shape == ref.shape and np.abs(ours - ref).max() < TOL_M
    # device input stays on the device
    dev = depth_map_to_points(torch.from_numpy(ragged).cuda(), M, case.aoi)
    assert dev.is_cuda and np.array_equal(dev.cpu().numpy(), ours)


def test_points_outside_the_fast_box_take_the_fp64_chain(case):
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import depth_map_to_points
    d = synth.depth_map_torch(case, 1).numpy()
    small = ((-40.0, -40.0, -5.0), (40.0, 40.0, 100.0))       # most of the scene lies outside
    part = depth_map_to_points(d, case.inv_proj[1], case.aoi, box=small)
    none = depth_map_to_points(d, case.inv_proj[1], case.aoi, box=None)
    ref = _oracle_points(d, case.inv_proj[1], case.aoi)
    assert np.abs(part - ref).max() < TOL_M and np.abs(none - ref).max() < TOL_M


@pytest.mark.parametrize('mode', ['fast', 'exact'])
def test_fused_dsm_equals_points_path_and_oracle(case, mode):
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import aoi_grid, depth_map_to_points, dsm_from_depth_maps
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    depths = [synth.depth_map_torch(case, v, 'cuda') for v in range(3)]
    grid = aoi_grid(case.aoi)
    fused = dsm_from_depth_maps(depths, list(case.inv_proj), case.aoi, mode=mode)
    pts = [depth_map_to_points(d, case.inv_proj[v], case.aoi, mode=mode) for v, d in enumerate(depths)]
    offs = torch.tensor(np.cumsum([0] + [p.shape[0] for p in pts]), dtype=torch.int64)
    two_step = dsm_from_points(torch.cat(pts), offs, *grid)
    torch.cuda.synchronize()
    assert same_bits(fused.cpu().numpy(), two_step.cpu().numpy())
    for v in range(3):
        ref = median_blur3x3(proj_to_grid(pts[v].cpu().numpy(), *grid).astype(np.float32))
        assert same_bits(fused[v].cpu().numpy(), ref), v
    assert np.isfinite(fused.cpu().numpy()).mean() > 0.6      # 200-row views cover ~260 of 300 m


def test_fused_dsm_on_a_grid_across_a_binade_falls_back():
    """An AOI whose easting range crosses 2^19 m cannot take the fused binning (its grid
    leaves the origin's binade); the wrapper goes through the points and gives the oracle's
    DSM of them."""
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import aoi_grid, depth_map_to_points, dsm_from_depth_maps
    case = synth.make_depth_case(25, 1, 96, 96, _utm, aoi_m=100.0, lon0=-86.7164, n_boxes=5)
    grid = aoi_grid(case.aoi)
    assert grid[0] < 2.0 ** 19 < grid[0] + grid[4] * grid[2]
    d = synth.depth_map_torch(case, 0, 'cuda')
    pts = depth_map_to_points(d, case.inv_proj[0], case.aoi).cpu().numpy()
    out = dsm_from_depth_maps([d], [case.inv_proj[0]], case.aoi)
    ref = median_blur3x3(proj_to_grid(pts, *grid).astype(np.float32))
    assert same_bits(out[0].cpu().numpy(), ref)
    assert np.isfinite(ref).mean() > 0.5


def test_equator_straddling_aoi_asserts_like_the_reference():
    """The reference asserts that all points lie in one hemisphere
    (lib/latlon_utm_converter.py:40); an AOI across the equator raises the same way, and
    its plan keeps the fast path off (the box spans both hemispheres)."""
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import depth_map_to_points
    from vissatsatellitestereo_gb300.coordinate_system import aoi_enu_box, aoi_origin, plan_for
    case = synth.make_depth_case(27, 1, 64, 64, _utm, aoi_m=400.0, lat0=0.0005, lon0=10.0, n_boxes=5)
    plan = plan_for(*aoi_origin(case.aoi), case.aoi['zone_number'], False, aoi_enu_box(case.aoi))
    assert not plan.fast_enabled
    with pytest.raises(AssertionError):
        depth_map_to_points(synth.depth_map_torch(case, 0).numpy(), case.inv_proj[0], case.aoi)


def test_depth_entry_points_reject_bad_arguments():
    import ctypes
    from vissatsatellitestereo_gb300 import _lib, synth
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import depth_map_to_points
    from vissatsatellitestereo_gb300.coordinate_system import GeoPlan
    with pytest.raises(_lib.VsError) as e:
        GeoPlan(39.0, -84.0, 0.0, 0, False)               # zone 0
    assert e.value.status == _lib.VS_ERR_ARG
    case = synth.make_depth_case(28, 1, 16, 16, _utm, aoi_m=40.0, n_boxes=2)
    d = synth.depth_map_torch(case, 0, 'cuda')
    bad = case.inv_proj[0].copy()
    bad[0, 0] = np.nan
    with pytest.raises(ValueError):
        depth_map_to_points(d, bad, case.aoi)
    plan = GeoPlan(39.77, -84.05, -30.0, 16, False)
    pts = torch.empty((256, 3), dtype=torch.float64, device='cuda')
    n = torch.zeros(1, dtype=torch.int64, device='cuda')
    ws = torch.empty(_lib.lib().vs_depth_to_points_workspace_size(16, 16), dtype=torch.uint8, device='cuda')
    m = np.ascontiguousarray(case.inv_proj[0])
    args = (d.data_ptr(), 16, 16, m.ctypes.data_as(ctypes.c_void_p), plan.handle)
    tail = (pts.data_ptr(), n.data_ptr(), None, ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream)
    assert _lib.lib().vs_depth_to_points(*args, 7, *tail) == _lib.VS_ERR_ARG          # bad mode
    assert _lib.lib().vs_depth_to_points(*args, _lib.VS_GEO_FAST, *tail[:3], ws.data_ptr(), 16,
                                         tail[-1]) == _lib.VS_ERR_WORKSPACE
    assert _lib.lib().vs_depth_to_points(*args, _lib.VS_GEO_FAST, *tail) == _lib.VS_OK
