"""Precision form of the RPC projection (monomial x coefficient contraction) against the
FP64 oracle of lib/rpc_model.py:40-79,164-168, through the C ABI.

Tolerances (max |error| in pixels, cameras with line/sample scale 2048):
  fp32, bf16x6: 1e-3 px (the projection bar of the path);
  tf32x3: 1.5e-3 px -- two tf32 pieces leave a coefficient residual and a dropped lo*lo
  product of up to 2**-22 relative each, ~5e-4 px apiece on the linear terms, on top of
  the FP32 accumulation and output rounding shared with fp32;
  bf16x3: 0.06 px -- two bf16 pieces keep ~17 significant bits of a factor, so the
  linear terms alone leave ~2048 * 2**-16 = 0.03 px in the worst case;
  bf16x3_lin: 1e-3 px -- the same split for the higher-order terms (coefficients ~1e-3, so
  ~1e-5 px), the constant and linear terms in FP32 as in fp32.
"""
import numpy as np
import pytest
import torch

from oracle import rpc as orpc

pytestmark = pytest.mark.gpu

TOL = {'fp32': 1e-3, 'tf32x3': 1.5e-3, 'bf16x6': 1e-3, 'bf16x3': 0.06, 'bf16x3_lin': 1e-3}


def cube_points(n, seed):
    rng = np.random.default_rng(seed)
    pts = rng.uniform(-1.0, 1.0, (3, n)).astype(np.float32)
    corners = np.array(np.meshgrid([-1.0, 0.0, 1.0], [-1.0, 0.0, 1.0], [-1.0, 0.0, 1.0])).reshape(3, -1)
    return np.ascontiguousarray(np.concatenate([corners.astype(np.float32), pts], axis=1))


def oracle_colrow(metas, pts):
    x, y, z = (pts[i].astype(np.float64) for i in range(3))
    out = np.empty((len(metas), 2, pts.shape[1]))
    for c, m in enumerate(metas):
        out[c, 0], out[c, 1] = orpc.projection_normalized(m, x, y, z)
    return out


@pytest.fixture(scope='module')
def cameras50():
    from vissatsatellitestereo_gb300 import synth
    return [synth.make_rpc_meta(1000 + v, 4096, 4096) for v in range(50)]


@pytest.mark.parametrize('variant', ['fp32', 'bf16x3', 'tf32x3', 'bf16x6', 'bf16x3_lin'])
def test_cube_variant_against_oracle(cameras50, variant):
    from vissatsatellitestereo_gb300.rpc_model import project_cube
    pts = cube_points(20000, 7)
    want = oracle_colrow(cameras50, pts)
    got = project_cube(cameras50, pts, variant=variant).cpu().numpy().astype(np.float64)
    err = np.abs(got - want)
    assert np.isfinite(got).all()
    assert err.max() <= TOL[variant], (variant, err.max())


def test_cube_split_forms_are_more_accurate_than_one_bf16_piece(cameras50):
    """bf16x6 recovers what bf16x3 drops: its error is far below bf16x3's."""
    from vissatsatellitestereo_gb300.rpc_model import project_cube
    pts = cube_points(4096, 11)
    want = oracle_colrow(cameras50, pts)
    e3 = np.abs(project_cube(cameras50, pts, 'bf16x3').cpu().numpy() - want).max()
    e6 = np.abs(project_cube(cameras50, pts, 'bf16x6').cpu().numpy() - want).max()
    assert e6 < e3 / 10, (e3, e6)


@pytest.mark.parametrize('variant', ['fp32', 'bf16x3', 'tf32x3', 'bf16x6', 'bf16x3_lin'])
@pytest.mark.parametrize('n_cams,n', [(1, 1), (3, 37), (5, 1000), (2, 16), (7, 65)])
def test_cube_odd_cameras_ragged_points_no_stray_writes(variant, n_cams, n):
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.rpc_model import project_cube
    metas = [synth.make_rpc_meta(50 + v, 4096, 4096) for v in range(n_cams)]
    pts = cube_points(n, n_cams * 100 + n)[:, :n]
    size = n_cams * 2 * n
    buf = torch.full((size + 4096,), 12345.0, dtype=torch.float32, device='cuda')
    out = buf[:size].view(n_cams, 2, n)
    project_cube(metas, pts, variant=variant, out=out)
    assert (buf[size:] == 12345.0).all()
    err = np.abs(out.cpu().numpy() - oracle_colrow(metas, pts)).max()
    assert err <= TOL[variant], err


def test_cube_agrees_with_the_exact_projection_kernel(cameras50):
    """The cube form evaluated at denormalised points matches vs_rpc_project (FP64, exact)."""
    from vissatsatellitestereo_gb300.rpc_model import project_cameras, project_cube
    pts = cube_points(3000, 3)
    metas = cameras50[:6]
    lat = np.stack([pts[0].astype(np.float64) * m['rpc']['latScale'] + m['rpc']['latOff'] for m in metas])
    lon = np.stack([pts[1].astype(np.float64) * m['rpc']['lonScale'] + m['rpc']['lonOff'] for m in metas])
    alt = np.stack([pts[2].astype(np.float64) * m['rpc']['altScale'] + m['rpc']['altOff'] for m in metas])
    col, row = project_cameras(metas, lat, lon, alt, mode='exact', shared=False)
    got = project_cube(metas, pts, 'tf32x3').cpu().numpy()
    assert np.abs(got[:, 0] - col.cpu().numpy()).max() <= TOL['tf32x3']
    assert np.abs(got[:, 1] - row.cpu().numpy()).max() <= TOL['tf32x3']


def test_cube_empty_and_errors(cameras50):
    from vissatsatellitestereo_gb300 import _lib
    from vissatsatellitestereo_gb300.rpc_model import project_cube
    out = project_cube(cameras50[:3], np.zeros((3, 0), np.float32), 'bf16x3')
    assert out.shape == (3, 2, 0)
    with pytest.raises(ValueError):
        project_cube(cameras50[:3], np.zeros((2, 5), np.float32))
    with pytest.raises(ValueError):
        project_cube(cameras50[:3], np.zeros((3, 5), np.float32), variant='fp16')
    too_many = cameras50 * 3          # 150 > VS_CUBE_MAX_CAMERAS
    with pytest.raises(_lib.VsError):
        project_cube(too_many, np.zeros((3, 5), np.float32))


@pytest.mark.parametrize('variant,twin', [('bf16x3_tc', 'bf16x3'), ('bf16x3_lin_tc', 'bf16x3_lin')])
@pytest.mark.parametrize('n_cams,n', [(50, 20000), (3, 37), (1, 1), (7, 300), (64, 1000), (49, 129), (63, 256)])
def test_cube_tcgen05_variant(variant, twin, n_cams, n):
    """The tcgen05 kernels (TMEM accumulators, overlapped epilogue): within the bound of
    their split scheme against the oracle (BF16X3 0.06 px, LIN 1e-3 px), within 2e-3 px of
    the mma.sync kernel with the same split, and no write outside colrow."""
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.rpc_model import project_cube
    metas = [synth.make_rpc_meta(3000 + v, 4096, 4096) for v in range(n_cams)]
    pts = cube_points(n, 17 + n_cams)[:, :n]
    size = n_cams * 2 * n
    buf = torch.full((size + 4096,), 12345.0, dtype=torch.float32, device='cuda')
    tc = buf[:size].view(n_cams, 2, n)
    project_cube(metas, pts, variant=variant, out=tc)
    assert (buf[size:] == 12345.0).all()
    ref = project_cube(metas, pts, variant=twin).cpu().numpy()
    got = tc.cpu().numpy()
    assert np.abs(got - oracle_colrow(metas, pts)).max() <= TOL[twin]
    assert np.abs(got - ref).max() <= 2e-3


def test_cube_tcgen05_rejects_too_many_cameras(cameras50):
    from vissatsatellitestereo_gb300 import _lib
    from vissatsatellitestereo_gb300.rpc_model import project_cube
    with pytest.raises(_lib.VsError):
        project_cube(cameras50 + cameras50[:20], np.zeros((3, 5), np.float32), variant='bf16x3_tc')


@pytest.mark.parametrize('variant', ['bf16x3_tc', 'bf16x3_lin_tc'])
def test_cube_tcgen05_timeout_is_reported(variant):
    """A CTA whose bounded wait for the tensor cores runs out sets the error word; the call's
    status query returns VS_ERR_TIMEOUT and the context stays usable.  The wait limit is
    set to 0 polls, so every CTA gives up at its first wait; it still waits, with the full
    limit, for its coefficient copy and any committed MMA before freeing its memory.  No
    device fault is involved."""
    from vissatsatellitestereo_gb300 import _lib, synth
    from vissatsatellitestereo_gb300.rpc_model import project_cube, project_cube_status
    metas = [synth.make_rpc_meta(3100 + v, 4096, 4096) for v in range(5)]
    pts = cube_points(3000, 23)
    L = _lib.lib()
    try:
        L.vs_set_tc_wait_limit(0)
        with pytest.raises(_lib.VsError) as e:
            project_cube(metas, pts, variant=variant)
        assert e.value.status == _lib.VS_ERR_TIMEOUT
        project_cube(metas, pts, variant=variant, check=False)
        with pytest.raises(_lib.VsError):
            project_cube_status(len(metas), variant)
    finally:
        L.vs_set_tc_wait_limit(1 << 24)
    got = project_cube(metas, pts, variant=variant).cpu().numpy()      # status clean again
    assert np.abs(got - oracle_colrow(metas, pts)).max() <= TOL['bf16x3' if variant == 'bf16x3_tc' else 'bf16x3_lin']
    project_cube_status(len(metas), variant)
    assert project_cube(metas, pts, variant='fp32') is not None
