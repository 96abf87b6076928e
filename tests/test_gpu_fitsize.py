"""Perspective fit at the benchmarked sizes against the reference's own fits (GB300).

``tests/golden/perspective_fit_fullsize.npz`` holds K, R, t and the six error statistics
that the reference's ``solve_perspective`` and ``check_perspective_error``
(lib/solve_perspective.py:82-126, lib/check_error.py:37-121) produced on the 200x200x20
grids of the 50-view workload (2048, 4096 and 8192 px cameras), on the single-camera
101x101x21 grid, and on one 200x200x20 grid shared by three cameras -- the reference's
own call pattern (camera_approx.py:158-176).  The grids are regenerated here; the fixture's
strided sample of each grid proves it is the grid the reference fitted.

Bar: the GPU camera reprojects every kept point within 1e-3 px of the reference camera,
and the GPU error statistics are within 1e-3 (px and m) of the reference's, in both fit
modes (double-float projection and FP64 projection), through the drop-in
``solve_perspective``/``check_perspective_error`` and through the batched
``approx_perspective_enu`` with per-view and shared grids.
"""
import ast
import sys

import numpy as np
import pytest
import torch

from conftest import GOLDEN
from oracle import dlt, rpc
from oracle.quat import quaternion_from_rotation

pytestmark = pytest.mark.gpu

PX_TOL = 1e-3
CASES = ['cfg1_2048', 'cfg1_4096', 'cfg1_8192', 'cfg0', 'shared']


@pytest.fixture(scope='module', autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from vissatsatellitestereo_gb300.build import build
    build()


@pytest.fixture(scope='module')
def problems(golden):
    """name -> (grid, [(meta, col, row, keep, K, R, t, err)], shared)"""
    from vissatsatellitestereo_gb300 import synth
    sys.path.insert(0, GOLDEN)
    from fit_cases import fit_cases
    z = golden('perspective_fit_fullsize.npz')
    out = {}
    for name, metas, n_xy, n_z, shared in fit_cases():
        g = synth.rpc_sample_grid(metas[0], n_xy, n_z)
        assert np.array_equal(np.hstack((g.lat, g.lon, g.alt, g.x, g.y, g.z))[::997], z[f'{name}_probe'])
        cams = []
        for c, meta in enumerate(metas):
            key = f'{name}_cam{c}'
            assert ast.literal_eval(str(z[f'{key}_meta'])) == meta
            col, row = rpc.projection(meta, g.lat, g.lon, g.alt)
            keep = rpc.in_image(meta, col, row)
            assert int(keep.sum()) == int(z[f'{key}_kept'])
            cams.append((meta, col, row, keep, z[f'{key}_K'], z[f'{key}_R'], z[f'{key}_t'], z[f'{key}_err']))
        out[name] = (g, cams, shared)
    return out


def _reprojection_gap(g, keep, K_ref, R_ref, t_ref, K, R, t):
    k = keep.ravel()
    c0, r0 = dlt.reproject(K_ref, R_ref, t_ref, g.x[k], g.y[k], g.z[k])
    c1, r1 = dlt.reproject(K, R, t, g.x[k], g.y[k], g.z[k])
    return float(np.max(np.hypot(c1 - c0, r1 - r0)))


@pytest.mark.parametrize('case', CASES)
def test_drop_in_fit_and_error_at_size(problems, case):
    from vissatsatellitestereo_gb300.check_error import check_perspective_error
    from vissatsatellitestereo_gb300.solve_perspective import solve_perspective
    g, cams, _ = problems[case]
    for meta, col, row, keep, K_ref, R_ref, t_ref, err_ref in cams:
        K, R, t = solve_perspective(g.x, g.y, g.z, col, row, keep)
        assert abs(np.linalg.det(R) - 1.0) < 1e-9 and K[2, 2] == 1.0
        assert _reprojection_gap(g, keep, K_ref, R_ref, t_ref, K, R, t) < PX_TOL
        err = check_perspective_error(g.x, g.y, g.z, col, row, K, R, t, keep)
        np.testing.assert_allclose(err, err_ref, rtol=0, atol=PX_TOL)


@pytest.mark.parametrize('mode', ['fast', 'exact'])
@pytest.mark.parametrize('case', CASES)
def test_camera_approx_at_size(problems, case, mode):
    from vissatsatellitestereo_gb300.camera_approx import approx_perspective_enu, params_to_krt
    g, cams, shared = problems[case]
    metas = [c[0] for c in cams]
    V = len(metas)
    if shared:
        cols = [g.lat.ravel(), g.lon.ravel(), g.alt.ravel(), g.x.ravel(), g.y.ravel(), g.z.ravel()]
    else:
        cols = [np.stack([a.ravel()] * V) for a in (g.lat, g.lon, g.alt, g.x, g.y, g.z)]
    params, err, status = approx_perspective_enu(metas, *cols, mode=mode, shared_points=shared)
    params, err, status = params.cpu().numpy(), err.cpu().numpy(), status.cpu().numpy()
    assert np.all(status == 0), status
    for v, (meta, col, row, keep, K_ref, R_ref, t_ref, err_ref) in enumerate(cams):
        K, R, t = params_to_krt(params[v])
        assert _reprojection_gap(g, keep, K_ref, R_ref, t_ref, K, R, t) < PX_TOL, (case, mode, v)
        np.testing.assert_allclose(err[v], err_ref, rtol=0, atol=PX_TOL)
        assert params[v][0] == meta['width'] and params[v][1] == meta['height']
        # pyquaternion 0.9.5 Quaternion(matrix=R) of the reference's own R: the same branch
        # (so the same sign) and close values.  R itself is only determined up to what the
        # DLT's ill-conditioning lets K and R trade against each other at equal reprojection
        # (a few 1e-6 here), so the bar on the values is 1e-4.
        q, q_ref = params[v][7:11], quaternion_from_rotation(R_ref)
        assert np.argmax(np.abs(q)) == np.argmax(np.abs(q_ref)) and np.dot(q, q_ref) > 0.999
        np.testing.assert_allclose(q, q_ref, rtol=0, atol=1e-4)
