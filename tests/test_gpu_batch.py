"""Batched form over many AOIs (height maps -> per-view DSMs -> fused DSMs) against the
oracle restatement of aggregate_2p5d_util.py:75-98 + produce_dsm.py:46-58 +
aggregate_2p5d.py:65-81, through the C ABI.  Bit-exact (NaN payloads aside)."""
import numpy as np
import pytest
import torch

from conftest import same_bits
from oracle import maps as omaps

pytestmark = pytest.mark.gpu


def build_batch(specs, maps, affines, tile=64, pad=0):
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
    return AoiBatch(grids, views, tile=tile)


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


@pytest.mark.parametrize('tile,pad,blocks', [(64, 0, 4), (32, 3, 4), (64, 5, 1), (32, 1, 8)])
def test_batch_matches_oracle(small_case, tile, pad, blocks):
    specs, maps, affines, (ref_views, ref_fused) = small_case
    b = build_batch(specs, maps, affines, tile=tile, pad=pad)
    vd, fu, sc = b.new_view_dsm(), b.new_fused(), b.new_scratch()
    b.run(vd, blocks_per_sm=blocks)
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
    one, many = b.new_view_dsm(), b.new_view_dsm()
    b.run(many)
    for v in range(b.n_views):
        b.run(one, views=(v, v + 1), blocks_per_sm=1)
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
    vd = b.new_view_dsm()
    b.run(vd)
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


def _geometry_cases():
    """Views whose pixel boxes stress the tile kernel: large rotations, a mirrored map,
    pixels much larger and much smaller than cells, a map half off the grid, one far away
    and a singular (rank-one) map; grids spanning several tiles."""
    from vissatsatellitestereo_gb300 import synth
    rng = np.random.default_rng(11)
    cases = []

    def heights(H, W):
        m = (rng.normal(0.0, 0.3, (H, W)) + rng.choice([0.0, 10.0, 25.0], (H, W), p=[0.6, 0.3, 0.1]))
        m = m.astype(np.float32)
        m[rng.random((H, W)) < 0.15] = np.nan
        zeros = rng.random((H, W)) < 0.02
        m[zeros] = np.where(rng.random(zeros.sum()) < 0.5, np.float32(0.0), np.float32(-0.0))
        return m

    s = synth.AoiSpec(0, 354052.25, 6182702.5, 0.5, 150, 130, 1, 0, 1)
    ce, cn = s.xoff + 37.5, s.yoff - 32.5
    cases.append(('rotated', s, heights(200, 180), synth.map_affine(ce, cn, 0.4, 0.7)))
    mir = synth.map_affine(ce + 3.0, cn - 2.0, 0.45, 2.5)
    mir['ej'], mir['nj'] = -mir['ej'], -mir['nj']
    cases.append(('mirrored', s, heights(170, 190), mir))
    cases.append(('sparse', s, heights(60, 70), synth.map_affine(ce, cn, 1.7, 0.2)))
    cases.append(('half_off_grid', s, heights(150, 160), synth.map_affine(s.xoff + 5.0, cn, 0.45, -0.1)))
    cases.append(('far_away', s, heights(40, 40), synth.map_affine(ce + 5000.0, cn, 0.5, 0.0)))
    sing = synth.map_affine(ce, cn, 0.4, 0.0)
    sing['ei'], sing['ni'] = sing['ej'], sing['nj']
    cases.append(('singular', s, heights(90, 90), sing))
    d = synth.AoiSpec(0, 300001.0, 4300123.75, 1.0, 70, 66, 1, 0, 1)
    cases.append(('dense', d, heights(700, 640), synth.map_affine(d.xoff + 33.0, d.yoff - 31.0, 0.1, 0.3)))
    return cases


@pytest.mark.parametrize('tile', [32, 64])
def test_tile_pixel_boxes_cover_every_geometry(tile):
    """Each view's DSM equals the oracle bit for bit: every pixel that reaches a tile (and
    its halo) lies inside the tile's pixel box, whatever the map's rotation, mirroring,
    scale or rank."""
    cases = _geometry_cases()
    specs = [c[1] for c in cases]
    b = build_batch(specs, [[c[2]] for c in cases], [[c[3]] for c in cases], tile=tile, pad=1)
    vd = b.new_view_dsm()
    b.run(vd)
    torch.cuda.synchronize()
    for v, (name, s, m, aff) in enumerate(cases):
        g = {'xoff': s.xoff, 'yoff': s.yoff, 'xres': s.res, 'yres': s.res, 'xsize': s.xsize, 'ysize': s.ysize}
        assert same_bits(b.view_dsm(vd, v).cpu().numpy(), omaps.view_dsm(m, aff, g)), name
    b.close()
