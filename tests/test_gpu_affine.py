"""Affine camera fit (solve_affine, approx_affine_latlonalt) on the GPU against the
reference's golden vectors and the oracle restatement of lib/solve_affine.py:37-72.
Tolerance: the fitted cameras' predictions within 1e-6 px of LAPACK's solution."""
import ast

import numpy as np
import pytest

from oracle import affine as oaff
from oracle import rpc as orpc

pytestmark = pytest.mark.gpu
TOL_PX = 1e-6


def _pred_diff(P0, P1, x, y, z):
    c0, r0 = oaff.affine_project(P0, x, y, z)
    c1, r1 = oaff.affine_project(P1, x, y, z)
    return np.max(np.hypot(c1 - c0, r1 - r0))


@pytest.mark.parametrize('i', [0, 1])
def test_solve_affine_matches_reference_golden(golden, i):
    from vissatsatellitestereo_gb300.solve_affine import solve_affine
    z = golden('affine_fit.npz')
    lat, lon, alt = z[f'cam{i}_lat'], z[f'cam{i}_lon'], z[f'cam{i}_alt']
    keep = z[f'cam{i}_keep']
    P = solve_affine(lat, lon, alt, z[f'cam{i}_col'], z[f'cam{i}_row'], keep)
    assert P.shape == (2, 4)
    k = keep.ravel()
    assert _pred_diff(z[f'cam{i}_P'], P, lat[k], lon[k], alt[k]) < TOL_PX


def test_camera_approx_affine_matches_oracle_per_view():
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.solve_affine import approx_affine_latlonalt
    metas = [synth.make_rpc_meta(1200 + v, s, s) for v, s in enumerate((2048, 4096, 8192))]
    g = synth.rpc_sample_grid(metas[0], 30, 8)        # one grid shared by the views, as the reference
    params, status = approx_affine_latlonalt(metas, g.lat.ravel(), g.lon.ravel(), g.alt.ravel())
    params, status = params.cpu().numpy(), status.cpu().numpy()
    for v, m in enumerate(metas):
        col, row = orpc.projection(m, g.lat, g.lon, g.alt)
        keep = orpc.in_image(m, col, row)
        if keep.sum() < 4:
            assert status[v] != 0
            continue
        assert status[v] == 0
        P = oaff.solve_affine(g.lat, g.lon, g.alt, col, row, keep)
        assert params[v, 0] == m['width'] and params[v, 1] == m['height']
        k = keep.ravel()
        assert _pred_diff(P, params[v, 2:].reshape(2, 4), g.lat.ravel()[k], g.lon.ravel()[k], g.alt.ravel()[k]) < TOL_PX


def test_degenerate_views_report_status():
    from vissatsatellitestereo_gb300.solve_affine import solve_affine, solve_affine_batch
    x = np.arange(10.0)
    P, st = solve_affine_batch(np.stack([x, x]), np.stack([x, x]), np.stack([x, x]), np.stack([x, x]),
                               np.stack([x, x]), keep_mask=np.stack([np.ones(10, bool), np.arange(10) < 3]))
    st = st.cpu().numpy()
    assert st[0] != 0 and st[1] != 0             # collinear points; 3 kept points
    rng = np.random.default_rng(0)
    a = rng.normal(size=(4, 50))
    P = solve_affine(a[0], a[1], a[2], 3 * a[0] - a[2] + 7, a[1] + 2 * a[2] - 1)
    assert np.allclose(P, [[3, 0, -1, 7], [0, 1, 2, -1]], atol=1e-9)
    with pytest.raises(AssertionError):
        solve_affine(a[0], a[1], a[2][:10], a[0], a[1])
