"""Parity of the CUDA path with the oracle and the golden vectors (GB300).

Tolerances: RPC projection exact mode bit-identical, fast mode |d| < 1e-4 px inside the
normalised cube; fitted cameras: reprojected pixels within 1e-3 px of the reference's
camera and error statistics within 1e-3 (px / m); rasterisation and fusion
bit-identical (NaN payloads aside).
"""
import ast

import numpy as np
import pytest
import torch

from conftest import same_bits
from oracle import blur, dlt, fuse, raster, rpc

pytestmark = pytest.mark.gpu

PX_TOL = 1e-3


@pytest.fixture(scope='module', autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from vissatsatellitestereo_gb300.build import build
    build()


def _meta(z, key):
    return ast.literal_eval(str(z[key]))


# ---- (a) projection -------------------------------------------------------------------
@pytest.mark.parametrize('cam', ['cam0', 'cam1', 'cam2'])
def test_rpc_exact_is_bit_identical_to_reference(golden, cam):
    from vissatsatellitestereo_gb300.rpc_model import RPCModel
    z = golden('rpc_projection.npz')
    m = RPCModel(_meta(z, f'{cam}_meta'))
    col, row = m.projection(z[f'{cam}_lat'], z[f'{cam}_lon'], z[f'{cam}_alt'])
    assert col.shape == z[f'{cam}_col'].shape
    assert same_bits(col, z[f'{cam}_col'])
    assert same_bits(row, z[f'{cam}_row'])


@pytest.mark.parametrize('cam', ['cam0', 'cam1', 'cam2'])
def test_rpc_fast_within_tolerance(golden, cam):
    from vissatsatellitestereo_gb300.rpc_model import RPCModel
    z = golden('rpc_projection.npz')
    m = RPCModel(_meta(z, f'{cam}_meta'), mode='fast')
    col, row = m.projection(z[f'{cam}_lat'], z[f'{cam}_lon'], z[f'{cam}_alt'])
    ref_c, ref_r = z[f'{cam}_col'], z[f'{cam}_row']
    grid = slice(0, ref_c.shape[0] - 4)           # the grid; the last 4 rows are NaN/inf/far-off probes
    assert np.max(np.abs(col[grid] - ref_c[grid])) < 1e-4
    assert np.max(np.abs(row[grid] - ref_r[grid])) < 1e-4
    assert np.isnan(col[-4]) and np.isnan(row[-3]) and not np.isfinite(col[-2])


def test_rpc_broadcast_and_device_tensors():
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.rpc_model import RPCModel
    meta = synth.make_rpc_meta(5, 2048, 2048)
    r = meta['rpc']
    lat = r['latOff'] + np.linspace(-0.04, 0.04, 7).reshape(7, 1)
    lon = r['lonOff'] + np.linspace(-0.04, 0.04, 5).reshape(1, 5)
    alt = np.float64(r['altOff'])
    m = RPCModel(meta)
    col, row = m.projection(lat, lon, alt)
    ref_c, ref_r = rpc.projection(meta, lat, lon, alt)
    assert col.shape == (7, 5) and same_bits(col, ref_c) and same_bits(row, ref_r)
    dc, dr = m.projection(torch.tensor(lat, device='cuda'), torch.tensor(lon, device='cuda'), alt)
    assert isinstance(dc, torch.Tensor) and dc.is_cuda and same_bits(dc.cpu().numpy(), ref_c)
    e_c, e_r = m.projection(np.zeros((0, 1)), np.zeros((0, 1)), np.zeros((0, 1)))
    assert e_c.shape == (0, 1)


def test_project_cameras_batch_shared_and_per_view():
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.rpc_model import project_cameras
    metas = [synth.make_rpc_meta(30 + i, 4096, 4096) for i in range(4)]
    grids = [synth.rpc_sample_grid(m, 33, 7) for m in metas]
    # per view grids
    lat = np.stack([g.lat.ravel() for g in grids])
    lon = np.stack([g.lon.ravel() for g in grids])
    alt = np.stack([g.alt.ravel() for g in grids])
    for mode in ('exact', 'fast'):
        col, row, keep = project_cameras(metas, lat, lon, alt, mode=mode, shared=False, keep=True)
        for v, m in enumerate(metas):
            rc, rr = rpc.projection(m, lat[v], lon[v], alt[v])
            tol = 0 if mode == 'exact' else 1e-4
            assert np.max(np.abs(col[v].cpu().numpy() - rc)) <= tol
            assert np.max(np.abs(row[v].cpu().numpy() - rr)) <= tol
            assert np.array_equal(keep[v].cpu().numpy().astype(bool), rpc.in_image(m, rc, rr))
    # shared grid (camera 0's grid through all cameras)
    col, row = project_cameras(metas, lat[0], lon[0], alt[0], mode='exact', shared=True)
    for v, m in enumerate(metas):
        rc, _ = rpc.projection(m, lat[0], lon[0], alt[0])
        assert same_bits(col[v].cpu().numpy(), rc)


# ---- (b) perspective fit -------------------------------------------------------------
@pytest.mark.parametrize('cam', ['cam0', 'cam1'])
def test_solve_perspective_matches_reference(golden, cam):
    from vissatsatellitestereo_gb300.solve_perspective import solve_perspective
    from vissatsatellitestereo_gb300.check_error import check_perspective_error
    z = golden('perspective_fit.npz')
    g = {k: z[f'{cam}_{k}'] for k in ('x', 'y', 'z', 'col', 'row', 'keep', 'K', 'R', 't', 'err')}
    K, R, t = solve_perspective(g['x'], g['y'], g['z'], g['col'], g['row'], g['keep'])
    assert K.shape == (3, 3) and R.shape == (3, 3) and t.shape == (3, 1)
    assert abs(np.linalg.det(R) - 1.0) < 1e-9 and K[2, 2] == 1.0 and np.all(np.diag(K) > 0)
    m = g['keep'].ravel()
    c0, r0 = dlt.reproject(g['K'], g['R'], g['t'], g['x'][m], g['y'][m], g['z'][m])
    c1, r1 = dlt.reproject(K, R, t, g['x'][m], g['y'][m], g['z'][m])
    assert np.max(np.hypot(c1 - c0, r1 - r0)) < PX_TOL
    err = check_perspective_error(g['x'], g['y'], g['z'], g['col'], g['row'], K, R, t, g['keep'])
    np.testing.assert_allclose(err, g['err'], rtol=0, atol=PX_TOL)
    # the statistics kernel on the reference's own camera (per-point errors are computed in
    # compensated FP32 in the fit's normalised frame: |error| <~ 1e-4 px)
    err_ref_cam = check_perspective_error(g['x'], g['y'], g['z'], g['col'], g['row'], g['K'], g['R'], g['t'],
                                          g['keep'])
    np.testing.assert_allclose(err_ref_cam, g['err'], rtol=0, atol=PX_TOL)


def test_solve_perspective_size_mismatch_asserts():
    from vissatsatellitestereo_gb300.solve_perspective import solve_perspective
    with pytest.raises(AssertionError):
        solve_perspective(np.zeros(5), np.zeros(5), np.zeros(4), np.zeros(5), np.zeros(5))


def test_solve_perspective_degenerate_reports():
    from vissatsatellitestereo_gb300.solve_perspective import solve_perspective_batch
    z = np.zeros(10)
    K, R, t, st = solve_perspective_batch(z, z, z, z.reshape(1, -1), z.reshape(1, -1), np.zeros((1, 10), bool))
    assert int(st[0]) != 0     # no kept points: degenerate, reported instead of raising


@pytest.mark.parametrize('mode', ['exact', 'fast'])
def test_camera_approx_batch_matches_reference_loop(mode):
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.camera_approx import approx_perspective_enu, params_to_krt
    metas = [synth.make_rpc_meta(700 + i, s, s) for i, s in enumerate((2048, 4096, 4096, 8192))]
    grids = [synth.rpc_sample_grid(m, 41, 9) for m in metas]
    st = lambda f: np.stack([getattr(g, f).ravel() for g in grids])
    params, err, status = approx_perspective_enu(metas, st('lat'), st('lon'), st('alt'), st('x'), st('y'), st('z'),
                                                 mode=mode, shared_points=False)
    params, err, status = params.cpu().numpy(), err.cpu().numpy(), status.cpu().numpy()
    assert np.all(status == 0)
    for v, (m, g) in enumerate(zip(metas, grids)):
        col, row = rpc.projection(m, g.lat, g.lon, g.alt)
        keep = rpc.in_image(m, col, row)
        K, R, t = dlt.solve_perspective(g.x, g.y, g.z, col, row, keep)
        ref_err = dlt.perspective_error(g.x, g.y, g.z, col, row, K, R, t, keep)
        K2, R2, t2 = params_to_krt(params[v])
        k = keep.ravel()
        c0, r0 = dlt.reproject(K, R, t, g.x[k], g.y[k], g.z[k])
        c1, r1 = dlt.reproject(K2, R2, t2, g.x[k], g.y[k], g.z[k])
        assert np.max(np.hypot(c1 - c0, r1 - r0)) < PX_TOL
        np.testing.assert_allclose(err[v], ref_err, rtol=0, atol=PX_TOL)
        ref_params = dlt.camera_params(m['width'], m['height'], K, R, t)
        np.testing.assert_allclose(params[v][:2], ref_params[:2])
        # R (and so q) is weakly determined for a near-affine camera (focal length ~1e5-1e6
        # px): rotation, focal length and translation trade off with sub-1e-3 px effect.  The
        # fit is pinned through the reprojection above; q only has to agree to 1e-4.
        np.testing.assert_allclose(params[v][7:11], ref_params[7:11], atol=1e-4)


# ---- (c) rasterisation -----------------------------------------------------------------
def test_proj_to_grid_golden_bit_exact(golden):
    from vissatsatellitestereo_gb300.proj_to_grid import proj_to_grid
    z = golden('proj_to_grid.npz')
    xoff, yoff, xres, yres, xsize, ysize = z['grid']
    dsm = proj_to_grid(z['points'], xoff, yoff, xres, yres, int(xsize), int(ysize))
    assert same_bits(dsm, z['dsm'])


@pytest.mark.parametrize('case', ['small', 'straddle', 'local_origin', 'negative'])
def test_proj_to_grid_matches_oracle(case):
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.proj_to_grid import proj_to_grid
    rng = np.random.default_rng(11)
    if case == 'small':
        scene, view = synth.small_raster_case()
        pts = synth.view_points(scene, view)
        g = scene.grid
        args = (g.xoff, g.yoff, g.xres, g.yres, g.xsize, g.ysize)
    elif case == 'straddle':      # northing grid crossing 2^22: both exponents present
        n = 200000
        pts = np.stack([rng.uniform(1000.0, 1300.0, n), rng.uniform(4194304.0 - 150, 4194304.0 + 150, n),
                        rng.normal(0, 10, n)], 1)
        args = (1000.0, 4194304.0 + 140, 0.37, 0.37, 700, 700)
    elif case == 'local_origin':  # origin at 0: no fast path
        n = 100000
        pts = np.stack([rng.uniform(-5, 120, n), rng.uniform(-120, 5, n), rng.normal(0, 10, n)], 1)
        args = (0.0, 0.0, 0.5, 0.5, 230, 230)
    else:                         # negative offsets
        n = 100000
        pts = np.stack([rng.uniform(-3000, -2800, n), rng.uniform(-7000, -6800, n), rng.normal(0, 10, n)], 1)
        args = (-3000.0, -6800.0, 0.25, 0.25, 800, 800)
    pts[rng.random(len(pts)) < 0.05, 2] = np.nan
    ref = raster.proj_to_grid(pts, *args)
    got = proj_to_grid(pts, *args)
    assert same_bits(got, ref)


def test_proj_to_grid_edge_cases():
    from vissatsatellitestereo_gb300.proj_to_grid import proj_to_grid
    args = (354052.25, 6182702.5, 0.5, 0.5, 4, 3)
    empty = proj_to_grid(np.zeros((0, 3)), *args)
    assert empty.shape == (3, 4) and np.all(np.isnan(empty))
    pts = np.array([[354052.25, 6182702.5, 1.0],        # UL corner -> cell (0, 0)
                    [354052.25 + 0.5, 6182702.5, -0.0],  # (0, 1): -0 first ...
                    [354052.25 + 0.7, 6182702.4, 0.0],   # ... then +0: sign of the first stays
                    [354052.25 + 1.2, 6182702.5 - 1.2, -np.inf],
                    [354052.25 + 1.9, 6182702.5 - 1.0, 0.0],   # (2, 3): +0 then -0
                    [354052.25 + 1.8, 6182702.5 - 1.1, -0.0]])
    ref = raster.proj_to_grid(pts, *args)
    got = proj_to_grid(pts, *args)
    assert same_bits(got, ref)
    assert np.signbit(got[0, 1]) and not np.signbit(got[2, 3])


def test_dsm_from_points_batch_matches_oracle():
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    grid = synth.DsmGrid(synth.EXPLORER_UL_EASTING, synth.EXPLORER_UL_NORTHING, 0.3, 0.3, 300, 260)
    scene = synth.make_scene(77, grid, 40, 3.0, 80.0)
    views = synth.make_views(78, scene, 3, 400, 440, 0.1, 0.3, 0.5)
    clouds = [synth.view_points(scene, v) for v in views]
    clouds[1] = clouds[1][:-7]    # ragged view sizes
    offsets = np.cumsum([0] + [len(c) for c in clouds])
    pts = np.concatenate(clouds)
    out = dsm_from_points(pts, offsets, grid.xoff, grid.yoff, grid.xres, grid.yres, grid.xsize, grid.ysize)
    out = out.cpu().numpy()
    for v, c in enumerate(clouds):
        ref = blur.median_blur3x3(raster.proj_to_grid(c, grid.xoff, grid.yoff, grid.xres, grid.yres,
                                                      grid.xsize, grid.ysize).astype(np.float32))
        assert same_bits(out[v], ref), v


def test_dsm_from_points_overlap_matches_serial_and_oracle():
    """Epilogues on a second stream overlapped with the next view's binning (rotating key
    grids, alternating first-zero arrays): identical to the serial call and the oracle,
    with signed zeros in the same cells of consecutive views."""
    import torch
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    grid = synth.DsmGrid(synth.EXPLORER_UL_EASTING, synth.EXPLORER_UL_NORTHING, 0.3, 0.3, 200, 170)
    scene = synth.make_scene(79, grid, 30, 3.0, 80.0)
    views = synth.make_views(80, scene, 7, 260, 300, 0.1, 0.3, 0.5)
    clouds = [synth.view_points(scene, v) for v in views]
    for v, c in enumerate(clouds):
        # a region of non-positive heights whose cell maxima are zeros: the sign of a
        # cell's first zero alternates view by view
        c[:6000, 2] = -np.abs(c[:6000, 2]) - 1.0
        c[:6000:2, 2] = -0.0 if v % 2 else 0.0
        c[1:6000:4, 2] = 0.0 if v % 2 else -0.0
    clouds[3] = clouds[3][:-13]
    offsets = np.cumsum([0] + [len(c) for c in clouds])
    pts = np.concatenate(clouds)
    args = (grid.xoff, grid.yoff, grid.xres, grid.yres, grid.xsize, grid.ysize)
    side = torch.cuda.Stream()
    over = dsm_from_points(pts, offsets, *args, epilogue_stream=side).cpu().numpy()
    serial = dsm_from_points(pts, offsets, *args).cpu().numpy()
    assert same_bits(over, serial)
    for v, c in enumerate(clouds):
        ref = blur.median_blur3x3(raster.proj_to_grid(c, *args).astype(np.float32))
        assert same_bits(over[v], ref), v
        assert (over[v] == 0).any()


@pytest.mark.parametrize('ctas', [0, 3, 5])
def test_dsm_from_points_pipelined_matches_serial_and_oracle(ctas):
    """One launch per view bins view v while its other CTAs run view v-1's epilogue
    (vs_dsm_from_points_pipelined): identical to the serial call and the oracle, with signed
    zeros alternating view by view, an empty view, a one-point view, odd view offsets and
    more views than key grids; at full occupancy and with the CTAs per SM capped (the
    48-register build at 5 or fewer)."""
    from vissatsatellitestereo_gb300 import _lib, synth
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    grid = synth.DsmGrid(synth.EXPLORER_UL_EASTING, synth.EXPLORER_UL_NORTHING, 0.3, 0.3, 230, 170)
    scene = synth.make_scene(83, grid, 30, 3.0, 80.0)
    views = synth.make_views(84, scene, 8, 260, 300, 0.1, 0.3, 0.5)
    clouds = [synth.view_points(scene, v) for v in views]
    for v, c in enumerate(clouds):
        c[:6000, 2] = -np.abs(c[:6000, 2]) - 1.0
        c[:6000:2, 2] = -0.0 if v % 2 else 0.0
        c[1:6000:4, 2] = 0.0 if v % 2 else -0.0
    clouds[2] = clouds[2][:0]
    clouds[3] = clouds[3][:1]
    clouds[5] = clouds[5][:-13]
    offsets = np.cumsum([0] + [len(c) for c in clouds])
    pts = torch.from_numpy(np.concatenate(clouds)).cuda()
    offs = torch.from_numpy(offsets).cuda()
    args = (grid.xoff, grid.yoff, grid.xres, grid.yres, grid.xsize, grid.ysize)
    serial = dsm_from_points(pts, offs, *args).cpu().numpy()
    _lib.lib().vs_set_binning_ctas_per_sm(ctas)
    try:
        pipe = dsm_from_points(pts, offs, *args, pipelined=True)
        again = dsm_from_points(pts, offs, *args, pipelined=True)     # the counters start from zero per call
        torch.cuda.synchronize()
    finally:
        _lib.lib().vs_set_binning_ctas_per_sm(0)
    pipe = pipe.cpu().numpy()
    assert same_bits(pipe, serial)
    assert same_bits(again.cpu().numpy(), serial)
    assert np.isnan(pipe[2]).all()
    for v, c in enumerate(clouds):
        ref = blur.median_blur3x3(raster.proj_to_grid(c, *args).astype(np.float32))
        assert same_bits(pipe[v], ref), v


def test_dsm_from_points_with_l2_persisting_key_grids():
    """An L2 set-aside with persisting access-policy windows over the key grids
    (vs_set_l2_persisting) leaves every DSM bit-identical: the serial, overlapped and
    pipelined forms and proj_to_grid; a request above the device's maximum is clamped, and
    0 releases the reservation."""
    from vissatsatellitestereo_gb300 import _lib, synth
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    from vissatsatellitestereo_gb300.proj_to_grid import proj_to_grid
    grid = synth.DsmGrid(synth.EXPLORER_UL_EASTING, synth.EXPLORER_UL_NORTHING, 0.3, 0.3, 210, 190)
    scene = synth.make_scene(85, grid, 25, 3.0, 80.0)
    views = synth.make_views(86, scene, 4, 240, 280, 0.1, 0.3, 0.5)
    clouds = [synth.view_points(scene, v) for v in views]
    offsets = np.cumsum([0] + [len(c) for c in clouds])
    pts = torch.from_numpy(np.concatenate(clouds)).cuda()
    offs = torch.from_numpy(offsets).cuda()
    args = (grid.xoff, grid.yoff, grid.xres, grid.yres, grid.xsize, grid.ysize)
    ref = dsm_from_points(pts, offs, *args).cpu().numpy()
    ref_grid = proj_to_grid(clouds[0], *args)
    L = _lib.lib()
    try:
        assert L.vs_set_l2_persisting(64 << 20) == _lib.VS_OK, L.vs_last_error()
        outs = [dsm_from_points(pts, offs, *args), dsm_from_points(pts, offs, *args, epilogue_stream=torch.cuda.Stream()),
                dsm_from_points(pts, offs, *args, pipelined=True)]
        got_grid = proj_to_grid(clouds[0], *args)
        torch.cuda.synchronize()
        assert L.vs_set_l2_persisting(1 << 40) == _lib.VS_OK, L.vs_last_error()      # clamped
    finally:
        assert L.vs_set_l2_persisting(0) == _lib.VS_OK, L.vs_last_error()
    for o in outs:
        assert same_bits(o.cpu().numpy(), ref)
    assert same_bits(got_grid, ref_grid)


@pytest.mark.parametrize('case', ['straddle', 'local_origin', 'single_view'])
def test_dsm_from_points_pipelined_other_grids(case):
    """Grids outside the fast binning's precondition (a northing axis across 2^22, an origin
    at 0) take the per-view kernels inside the pipelined call; a single view has one
    binning-only and one epilogue-only launch.  All equal the oracle."""
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    rng = np.random.default_rng(12)
    if case == 'straddle':
        n = 120000
        mk = lambda: np.stack([rng.uniform(1000.0, 1300.0, n), rng.uniform(4194304.0 - 150, 4194304.0 + 150, n),
                               rng.normal(0, 10, n)], 1)
        args = (1000.0, 4194304.0 + 140, 0.37, 0.37, 700, 700)
        clouds = [mk(), mk()]
    elif case == 'local_origin':
        n = 80000
        mk = lambda: np.stack([rng.uniform(-5, 120, n), rng.uniform(-120, 5, n), rng.normal(0, 10, n)], 1)
        args = (0.0, 0.0, 0.5, 0.5, 230, 230)
        clouds = [mk(), mk(), mk()]
    else:
        n = 150001
        clouds = [np.stack([rng.uniform(354052.0, 354112.0, n), rng.uniform(6182640.0, 6182702.0, n),
                            rng.normal(20, 10, n)], 1)]
        args = (354052.25, 6182702.5, 0.3, 0.3, 197, 205)
    for c in clouds:
        c[rng.random(len(c)) < 0.05, 2] = np.nan
    offsets = np.cumsum([0] + [len(c) for c in clouds])
    pts = torch.from_numpy(np.concatenate(clouds)).cuda()
    got = dsm_from_points(pts, torch.from_numpy(offsets).cuda(), *args, pipelined=True).cpu().numpy()
    for v, c in enumerate(clouds):
        ref = blur.median_blur3x3(raster.proj_to_grid(c, *args).astype(np.float32))
        assert same_bits(got[v], ref), v


def test_dsm_from_points_host_pipeline_equals_device_path():
    """Host points copied view by view into a 3-buffer device ring on a second stream
    (vs_dsm_from_points_host): bit-identical to the device-input call, with an empty view, a
    one-point view, odd view offsets and more views than ring buffers."""
    import torch
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    grid = synth.DsmGrid(synth.EXPLORER_UL_EASTING, synth.EXPLORER_UL_NORTHING, 0.3, 0.3, 180, 150)
    scene = synth.make_scene(81, grid, 25, 3.0, 80.0)
    views = synth.make_views(82, scene, 6, 200, 230, 0.1, 0.3, 0.5)
    clouds = [synth.view_points(scene, v) for v in views]
    clouds[1] = clouds[1][:0]
    clouds[2] = clouds[2][:1]
    clouds[4] = clouds[4][:-3]
    offsets = np.cumsum([0] + [len(c) for c in clouds])
    pts = np.concatenate(clouds)
    args = (grid.xoff, grid.yoff, grid.xres, grid.yres, grid.xsize, grid.ysize)
    dev = dsm_from_points(torch.from_numpy(pts).cuda(), torch.from_numpy(offsets).cuda(), *args)
    pinned = torch.from_numpy(pts).pin_memory()
    host = dsm_from_points(pinned, torch.from_numpy(offsets), *args)
    torch.cuda.synchronize()
    assert same_bits(host.cpu().numpy(), dev.cpu().numpy())
    assert np.isnan(host[1].cpu().numpy()).all()


def _blur_image(rng, H, W):
    img = rng.integers(-3, 4, (H, W)).astype(np.float32)       # many ties
    u = rng.random((H, W))
    img[u < 0.25] = np.nan
    img[(u >= 0.25) & (u < 0.3)] = -0.0
    img[(u >= 0.3) & (u < 0.33)] = np.inf
    img[(u >= 0.33) & (u < 0.36)] = -np.inf
    return img


BLUR_SHAPES = [(1, 1), (1, 2), (1, 9), (9, 1), (2, 2), (3, 5), (5, 6), (4, 7), (6, 10), (7, 13), (33, 70), (40, 1),
               (1, 41)]


@pytest.mark.parametrize('H,W', BLUR_SHAPES)
def test_median_blur_cv2_network_shapes(H, W):
    """The standalone blur and the fusion's blur against OpenCV's network (scalar and SSE
    columns, the 1-D path) on images full of NaN, ties, signed zeros and infinities."""
    from vissatsatellitestereo_gb300.aggregate_2p5d import fuse_dsms
    from vissatsatellitestereo_gb300.proj_to_grid import median_blur3x3
    rng = np.random.default_rng(H * 100 + W)
    img = np.stack([_blur_image(rng, H, W) for _ in range(3)])
    got = median_blur3x3(img)
    for b in range(3):
        assert same_bits(got[b], blur.median_blur3x3(img[b])), b
    # the fusion's final blur: 3 identical views fuse to the view itself
    stack = np.repeat(img[0][:, :, None], 3, axis=2)
    assert same_bits(fuse_dsms(stack, median_blur=True), blur.median_blur3x3(fuse.fuse_numpy(stack)))


@pytest.mark.parametrize('H,W', BLUR_SHAPES)
def test_dsm_epilogue_cv2_network_shapes(H, W):
    """The fused rasterisation epilogue (nanmax, hole fill, blur in shared memory) on grids
    of every shape class, including 1-wide and 1-high grids."""
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    rng = np.random.default_rng(H * 1000 + W)
    xoff, yoff, res = 354000.0, 6182000.0, 1.0
    n = max(4 * H * W // 3, 1)
    pts = np.empty((n, 3))
    pts[:, 0] = xoff + rng.uniform(0, W, n)
    pts[:, 1] = yoff - rng.uniform(0, H, n)
    pts[:, 2] = rng.integers(-2, 3, n).astype(np.float64)
    pts[rng.random(n) < 0.1, 2] = -0.0
    pts[rng.random(n) < 0.05, 2] = np.inf
    args = (xoff, yoff, res, res, W, H)
    got = dsm_from_points(pts, np.array([0, n]), *args).cpu().numpy()[0]
    assert same_bits(got, blur.median_blur3x3(raster.proj_to_grid(pts, *args).astype(np.float32)))


@pytest.mark.parametrize('H,W', [(33, 70), (64, 64), (70, 33), (5, 6)])
def test_dsm_epilogue_sorted_column_path(H, W):
    """Tiles whose staged values hold no NaN and no zero take the sorted-column median in
    the epilogue; with ties and infinities it must still equal OpenCV's network bit for bit."""
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    rng = np.random.default_rng(H * 7 + W)
    xoff, yoff, res = 354000.0, 6182000.0, 1.0
    n = 16 * H * W                                 # dense: no empty cells, so no hole fill
    pts = np.empty((n, 3))
    pts[:, 0] = xoff + rng.uniform(0, W, n)
    pts[:, 1] = yoff - rng.uniform(0, H, n)
    pts[:, 2] = rng.choice([-3.5, -1.0, 1.0, 2.5, 7.0, np.inf, -np.inf], n, p=[0.2, 0.2, 0.2, 0.2, 0.1, 0.05, 0.05])
    args = (xoff, yoff, res, res, W, H)
    ref = blur.median_blur3x3(raster.proj_to_grid(pts, *args).astype(np.float32))
    assert not np.isnan(raster.proj_to_grid(pts, *args)).any()       # every cell covered: the fast path
    got = dsm_from_points(pts, np.array([0, n]), *args).cpu().numpy()[0]
    assert same_bits(got, ref)


def test_median_blur_matches_oracle():
    from vissatsatellitestereo_gb300.proj_to_grid import median_blur3x3
    rng = np.random.default_rng(3)
    img = rng.normal(0, 5, (3, 37, 53)).astype(np.float32)
    img[rng.random(img.shape) < 0.3] = np.nan
    img[0, 0, :3] = [np.inf, -np.inf, -0.0]
    got = median_blur3x3(img)
    for b in range(3):
        assert same_bits(got[b], blur.median_blur3x3(img[b]))
    got64 = median_blur3x3(img[0].astype(np.float64))
    assert same_bits(got64, blur.median_blur3x3(img[0]))
    one = median_blur3x3(np.float32([[7.0]]))
    assert one[0, 0] == 7.0


# ---- (d) fusion -----------------------------------------------------------------------
@pytest.mark.parametrize('V', [9, 50])
def test_fusion_golden_bit_exact(golden, V):
    from vissatsatellitestereo_gb300.aggregate_2p5d import fuse_dsms
    z = golden('fusion.npz')
    stack = z[f'v{V}_stack']
    assert same_bits(fuse_dsms(stack, median_blur=False), z[f'v{V}_fused'])
    assert same_bits(fuse_dsms(stack, median_blur=True), blur.median_blur3x3(z[f'v{V}_fused']))
    dev = torch.tensor(np.moveaxis(stack, 2, 0).copy(), device='cuda')
    assert same_bits(fuse_dsms(dev, median_blur=False, layout='vhw').cpu().numpy(), z[f'v{V}_fused'])


@pytest.mark.parametrize('V', [1, 2, 3, 4, 7, 8, 12, 16, 17, 33, 60, 64, 65, 129, 200])
def test_fusion_matches_numpy(V):
    from vissatsatellitestereo_gb300.aggregate_2p5d import fuse_dsms
    rng = np.random.default_rng(V)
    a = rng.normal(30, 10, (24, 20, V)).astype(np.float32)
    a[rng.random(a.shape) < rng.uniform(0.0, 0.8, (24, 20, 1))] = np.nan
    a[0, 0, :] = np.float32(-0.0)
    if V > 3:
        a[1, 1, :3] = np.inf
        a[2, 2, :] = np.float32(3e38)
        a[3, 3, :] = np.where(np.arange(V) % 2 == 0, np.float32(1e7), np.float32(-1e7 + 0.37))
        a[4, 4, :] = np.inf                                   # infinite median
        a[5, 5, :V // 2] = -np.inf                            # -inf below a finite median
        a[6, 6, :] = np.float32(5.0) + np.float32(0.25) * (np.arange(V) % 5 - 2)   # tied deviations
        a[7, 7, :] = np.where(np.arange(V) < (2 * V) // 3, np.inf, np.float32(1.5))  # +inf majority
        a[8, 8, :] = np.where(np.arange(V) % 3 == 0, np.float32(-2.5), np.float32(7.25))
    with np.errstate(invalid='ignore'):
        ref = fuse.fuse_numpy(a)
    assert same_bits(fuse_dsms(a, median_blur=False), ref)
