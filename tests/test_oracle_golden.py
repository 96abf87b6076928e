"""The oracle against the golden vectors made from the reference's own code (CPU)."""
import ast
import sys

import numpy as np
import pytest

from conftest import GOLDEN, same_bits
from oracle import blur, dlt, fuse, raster, rpc


def _meta(z, key):
    return ast.literal_eval(str(z[key]))


@pytest.mark.parametrize('cam', ['cam0', 'cam1', 'cam2'])
def test_rpc_projection_bit_exact(golden, cam):
    z = golden('rpc_projection.npz')
    meta = _meta(z, f'{cam}_meta')
    with np.errstate(all='ignore'):
        col, row = rpc.projection(meta, z[f'{cam}_lat'], z[f'{cam}_lon'], z[f'{cam}_alt'])
    assert same_bits(col, z[f'{cam}_col'])
    assert same_bits(row, z[f'{cam}_row'])


@pytest.mark.parametrize('cam', ['cam0', 'cam1'])
def test_perspective_fit_matches_reference(golden, cam):
    z = golden('perspective_fit.npz')
    g = {k: z[f'{cam}_{k}'] for k in ('x', 'y', 'z', 'col', 'row', 'keep', 'K', 'R', 't', 'err')}
    K, R, t = dlt.solve_perspective(g['x'], g['y'], g['z'], g['col'], g['row'], g['keep'])
    np.testing.assert_allclose(K, g['K'], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(R, g['R'], rtol=0, atol=1e-9)
    m = g['keep'].ravel()
    c0, r0 = dlt.reproject(g['K'], g['R'], g['t'], g['x'][m], g['y'][m], g['z'][m])
    c1, r1 = dlt.reproject(K, R, t, g['x'][m], g['y'][m], g['z'][m])
    assert np.max(np.hypot(c1 - c0, r1 - r0)) < 1e-6
    err = dlt.perspective_error(g['x'], g['y'], g['z'], g['col'], g['row'], K, R, t, g['keep'])
    np.testing.assert_allclose(err, g['err'], rtol=0, atol=1e-6)


def test_proj_to_grid_bit_exact(golden):
    z = golden('proj_to_grid.npz')
    xoff, yoff, xres, yres, xsize, ysize = z['grid']
    args = (z['points'], xoff, yoff, xres, yres, int(xsize), int(ysize))
    assert same_bits(raster.proj_to_grid(*args), z['dsm'])
    assert same_bits(raster.proj_to_grid(*args, loop=True), z['dsm'])


@pytest.mark.parametrize('V', [9, 50])
def test_fusion_bit_exact(golden, V):
    z = golden('fusion.npz')
    stack, ref = z[f'v{V}_stack'], z[f'v{V}_fused']
    assert same_bits(fuse.fuse_numpy(stack), ref)
    assert same_bits(fuse.fuse_explicit(stack), ref)


def test_hole_fill_vectorised_equals_loop():
    rng = np.random.default_rng(7)
    d = rng.normal(0, 3, (40, 50))
    d[rng.random(d.shape) < 0.45] = np.nan
    d[3, 3], d[3, 5], d[8, 8], d[8, 10] = -0.0, -0.0, np.inf, -np.inf
    assert same_bits(raster.hole_fill(d), raster.hole_fill_loop(d))


def _blur_image(seed, H, W):
    rng = np.random.default_rng(seed)
    img = rng.integers(-3, 4, (H, W)).astype(np.float32)       # many ties
    u = rng.random((H, W))
    img[u < 0.25] = np.nan
    img[(u >= 0.25) & (u < 0.3)] = -0.0
    img[(u >= 0.3) & (u < 0.33)] = np.inf
    img[(u >= 0.33) & (u < 0.36)] = -np.inf
    return img


@pytest.mark.parametrize('H,W', [(1, 1), (1, 7), (7, 1), (2, 2), (3, 5), (5, 6), (4, 9), (6, 13), (3, 37)])
def test_median_blur_vectorised_equals_pixel_loop(H, W):
    for seed in range(4):
        img = _blur_image(seed, H, W)
        assert same_bits(blur.median_blur3x3(img), blur.median_blur3x3_loop(img))


def test_median_blur_sse_columns():
    """cv::medianBlur's row loop: column 0 scalar, then 4 columns at a time from column 1
    while j <= W - 5, the rest scalar."""
    assert not blur.vector_columns(5).any()
    assert blur.vector_columns(6).tolist() == [False, True, True, True, True, False]
    assert blur.vector_columns(10).tolist() == [False] + [True] * 8 + [False]
    assert blur.vector_columns(2000).sum() == 1996


def test_median_blur_finite_values_and_nan_rules():
    img = np.arange(25, dtype=np.float32).reshape(5, 5)
    out = blur.median_blur3x3(img)
    assert out[2, 2] == 12 and out[0, 0] == 1   # replicate border: {0,0,1,0,0,1,5,5,6}
    rng = np.random.default_rng(3)
    img = rng.permutation(64 * 64).astype(np.float32).reshape(64, 64)
    pad = np.pad(img, 1, mode='edge')
    win = np.stack([pad[dj:dj + 64, dk:dk + 64] for dj in range(3) for dk in range(3)])
    assert same_bits(blur.median_blur3x3(img), np.sort(win, axis=0)[4])    # distinct finite: the median
    # the scalar op never moves a NaN (every comparison with it is false), so in a scalar
    # column a NaN centre comes out as NaN whatever its neighbours are
    img = np.ones((4, 12), dtype=np.float32)
    img[1, 0] = img[2, 11] = np.nan
    out = blur.median_blur3x3(img)
    assert np.isnan(out[1, 0]) and np.isnan(out[2, 11])
    assert np.sum(np.isnan(out)) >= 2


def test_inverse_projection_oracle_matches_reference_golden(golden):
    """RPCModel.inverse_projection (lib/rpc_model.py:170-249) on 1-D inputs, bit-exact."""
    z = golden('rpc_inverse.npz')
    for i in range(3):
        meta = ast.literal_eval(str(z[f'cam{i}_meta']))
        col, row, alt = z[f'cam{i}_col'], z[f'cam{i}_row'], z[f'cam{i}_alt']
        lon, lat, alt_out, it = rpc.inverse_projection(meta, col, row, alt)
        assert same_bits(lon, z[f'cam{i}_lon']) and same_bits(lat, z[f'cam{i}_lat']) and it > 0
        ln, lt, an, _ = rpc.inverse_projection(meta, col, row, alt, return_normalized=True)
        assert same_bits(ln, z[f'cam{i}_lon_n']) and same_bits(lt, z[f'cam{i}_lat_n'])
        assert same_bits(an, z[f'cam{i}_alt_n'])


def test_affine_oracle_matches_reference_golden(golden):
    """solve_affine (lib/solve_affine.py:37-72) on lat/lon/alt grids."""
    from oracle import affine
    z = golden('affine_fit.npz')
    for i in range(2):
        P = affine.solve_affine(z[f'cam{i}_lat'], z[f'cam{i}_lon'], z[f'cam{i}_alt'], z[f'cam{i}_col'],
                                z[f'cam{i}_row'], z[f'cam{i}_keep'])
        ref = z[f'cam{i}_P']
        k = z[f'cam{i}_keep'].ravel()
        c0, r0 = affine.affine_project(ref, z[f'cam{i}_lat'][k], z[f'cam{i}_lon'][k], z[f'cam{i}_alt'][k])
        c1, r1 = affine.affine_project(P, z[f'cam{i}_lat'][k], z[f'cam{i}_lon'][k], z[f'cam{i}_alt'][k])
        # LAPACK builds may differ in the last bits; the fitted camera may not
        assert np.max(np.hypot(c1 - c0, r1 - r0)) < 1e-6
        assert ast.literal_eval(str(z[f'cam{i}_meta']))['width'] > 0


def _fit_cases():
    sys.path.insert(0, GOLDEN)
    from fit_cases import fit_cases
    return fit_cases()


@pytest.mark.parametrize('case', ['cfg1_2048', 'cfg1_4096', 'cfg1_8192', 'cfg0', 'shared'])
def test_perspective_fit_at_benchmark_sizes(golden, case):
    """The oracle's SVD fit against the reference's own fit at the benchmarked grid sizes
    (200x200x20 per view; 101x101x21; one grid shared by three cameras)."""
    from vissatsatellitestereo_gb300 import synth
    z = golden('perspective_fit_fullsize.npz')
    name, metas, n_xy, n_z, shared = next(c for c in _fit_cases() if c[0] == case)
    g = synth.rpc_sample_grid(metas[0], n_xy, n_z)
    assert np.array_equal(np.hstack((g.lat, g.lon, g.alt, g.x, g.y, g.z))[::997], z[f'{case}_probe'])
    for c, meta in enumerate(metas):
        key = f'{case}_cam{c}'
        assert _meta(z, f'{key}_meta') == meta
        col, row = rpc.projection(meta, g.lat, g.lon, g.alt)
        keep = rpc.in_image(meta, col, row)
        assert int(keep.sum()) == int(z[f'{key}_kept'])
        K, R, t = dlt.solve_perspective(g.x, g.y, g.z, col, row, keep)
        k = keep.ravel()
        c0, r0 = dlt.reproject(z[f'{key}_K'], z[f'{key}_R'], z[f'{key}_t'], g.x[k], g.y[k], g.z[k])
        c1, r1 = dlt.reproject(K, R, t, g.x[k], g.y[k], g.z[k])
        assert np.max(np.hypot(c1 - c0, r1 - r0)) < 1e-6
        err = dlt.perspective_error(g.x, g.y, g.z, col, row, K, R, t, keep)
        np.testing.assert_allclose(err, z[f'{key}_err'], rtol=0, atol=1e-6)
