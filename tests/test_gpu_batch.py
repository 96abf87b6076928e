"""Batched form over many AOIs (height maps -> per-view DSMs -> fused DSMs) against the
oracle restatement of aggregate_2p5d_util.py:75-98 + produce_dsm.py:46-58 +
aggregate_2p5d.py:65-81, through the C ABI.  Bit-exact (NaN payloads aside)."""
import numpy as np
import pytest
import torch

from conftest import same_bits
from oracle import maps as omaps

pytestmark = pytest.mark.gpu


def build_batch(specs, maps, affines, rows_per_item=8, pad=0):
    from vissatsatellitestereo_gb300.batch import AoiBatch, AoiGrid, MapAffine, MapView
    grids, views = [], []
    for s, ms, afs in zip(specs, maps, affines):
        grids.append(AoiGrid(s.xoff, s.yoff, s.res, s.res, s.xsize, s.ysize))
        vs = []
        for m, a in zip(ms, afs):
            H, W = m.shape
            store = np.full((H, W + pad), 7.0, dtype=np.float32)
            store[:, :W] = m
            vs.append(MapView(torch.from_numpy(store).cuda(), W, H, MapAffine(**a)))
        views.append(vs)
    return AoiBatch(grids, views, rows_per_item=rows_per_item)


def oracle_results(specs, maps, affines):
    per_view, fused = [], []
    for s, ms, afs in zip(specs, maps, affines):
        g = {'xoff': s.xoff, 'yoff': s.yoff, 'xres': s.res, 'yres': s.res, 'xsize': s.xsize, 'ysize': s.ysize}
        dv = [omaps.view_dsm(m, a, g) for m, a in zip(ms, afs)]
        per_view.append(dv)
        fused.append(omaps.fused_dsm(dv))
    return per_view, fused


@pytest.fixture(scope='module')
def small_case():
    from vissatsatellitestereo_gb300 import synth
    specs, maps, affines = synth.small_aoi_case()
    return specs, maps, affines, oracle_results(specs, maps, affines)


@pytest.mark.parametrize('rows_per_item,pad', [(8, 0), (1, 3), (64, 5), (3, 1)])
def test_batch_matches_oracle(small_case, rows_per_item, pad):
    specs, maps, affines, (ref_views, ref_fused) = small_case
    b = build_batch(specs, maps, affines, rows_per_item=rows_per_item, pad=pad)
    vd, fu, sc = b.new_view_dsm(), b.new_fused(), b.new_scratch()
    b.run(vd, sc)
    b.fuse(vd, fu, sc)
    torch.cuda.synchronize()
    v = 0
    for a in range(len(specs)):
        for k in range(len(maps[a])):
            assert same_bits(b.view_dsm(vd, v).cpu().numpy(), ref_views[a][k]), (a, k)
            v += 1
        assert same_bits(b.fused_dsm(fu, a).cpu().numpy(), ref_fused[a]), a
    b.close()


def test_per_view_runs_equal_the_batched_run(small_case):
    specs, maps, affines, _ = small_case
    b = build_batch(specs, maps, affines)
    sc = b.new_scratch()
    one, many = b.new_view_dsm(), b.new_view_dsm()
    b.run(many, sc)
    for v in range(b.n_views):
        b.run(one, sc, views=(v, v + 1), bin_blocks_per_sm=1)
    torch.cuda.synchronize()
    assert same_bits(one.cpu().numpy(), many.cpu().numpy())


def test_points_on_cell_boundaries():
    """Pixels placed exactly on grid lines (gsd = resolution, aligned origin) exercise the
    threshold correction of the binning."""
    from vissatsatellitestereo_gb300 import synth
    s = synth.AoiSpec(0, 400000.0, 5000000.0, 0.5, 40, 30, 1, 0, 1)
    H, W = 64, 84
    # pixel j at easting xoff + 0.5 (j - 4) and row i at northing yoff - 0.5 (i - 4): every
    # coordinate sits on a grid line, and the first four rows/columns fall before the grid
    ce = s.xoff + 0.25 * (W - 1) - 2.0
    cn = s.yoff - 0.25 * (H - 1) + 2.0
    aff = synth.map_affine(ce, cn, 0.5, 0.0)
    rng = np.random.default_rng(5)
    m = rng.normal(5.0, 1.0, (H, W)).astype(np.float32)
    b = build_batch([s], [[m]], [[aff]])
    vd, fu, sc = b.new_view_dsm(), b.new_fused(), b.new_scratch()
    b.run(vd, sc)
    torch.cuda.synchronize()
    g = {'xoff': s.xoff, 'yoff': s.yoff, 'xres': s.res, 'yres': s.res, 'xsize': s.xsize, 'ysize': s.ysize}
    assert same_bits(b.view_dsm(vd, 0).cpu().numpy(), omaps.view_dsm(m, aff, g))


def test_plan_rejects_unsupported_grids_and_views():
    from vissatsatellitestereo_gb300 import _lib, synth
    from vissatsatellitestereo_gb300.batch import AoiBatch, AoiGrid, MapAffine, MapView
    m = torch.zeros((8, 8), dtype=torch.float32, device='cuda')
    aff = MapAffine(**synth.map_affine(400010.0, 5000010.0, 0.5, 0.0))
    with pytest.raises(_lib.VsError):       # grid crossing 2^19 m of easting
        AoiBatch([AoiGrid(524280.0, 5000020.0, 0.5, 0.5, 100, 40)], [[MapView(m, 8, 8, aff)]])
    with pytest.raises(_lib.VsError):       # negative origin
        AoiBatch([AoiGrid(-400000.0, 5000020.0, 0.5, 0.5, 40, 40)], [[MapView(m, 8, 8, aff)]])
    big = MapAffine(e0=1 << 60, n0=aff.n0, ej=aff.ej, ei=aff.ei, nj=aff.nj, ni=aff.ni)
    with pytest.raises(_lib.VsError):       # coordinates beyond the exact range
        AoiBatch([AoiGrid(400000.0, 5000020.0, 0.5, 0.5, 40, 40)], [[MapView(m, 8, 8, big)]])
    with pytest.raises(ValueError):
        AoiBatch([AoiGrid(400000.0, 5000020.0, 0.5, 0.5, 40, 40)], [[MapView(m.double(), 8, 8, aff)]])


def test_map_points_kernel_matches_oracle(small_case):
    """vs_map_points (the plain per-view path's point list) against oracle/maps.map_points,
    bit-exact, on padded strides; its points through proj_to_grid + blur give the oracle's
    per-view DSM."""
    from vissatsatellitestereo_gb300.batch import map_points
    from vissatsatellitestereo_gb300.proj_to_grid import median_blur3x3, proj_to_grid
    specs, maps, affines, (ref_views, _) = small_case
    for a, s in enumerate(specs):
        for k, (m, aff) in enumerate(zip(maps[a], affines[a])):
            H, W = m.shape
            store = np.full((H, W + 3), 5.0, dtype=np.float32)
            store[:, :W] = m
            pts = map_points(torch.from_numpy(store).cuda(), aff, width=W, height=H)
            assert same_bits(pts.cpu().numpy(), omaps.map_points(m, aff))
            d = median_blur3x3(proj_to_grid(pts, s.xoff, s.yoff, s.res, s.res, s.xsize, s.ysize))
            assert same_bits(d.cpu().numpy() if isinstance(d, torch.Tensor) else d, ref_views[a][k])
