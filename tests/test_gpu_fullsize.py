"""Parity at the benchmark's full sizes: against the oracle where it finishes in seconds
(one full 4096^2 view through proj_to_grid + blur; a 96-row band of the 50-view fusion),
and through size-independent properties where it cannot:

* rasterisation of 50 views x 4096^2 points onto 2000 x 2000 at 0.3 m: the overlapped
  two-stream schedule and the serial one are bit-identical, and a view rasterised alone
  equals the same view inside the 50-view call;
* fusion of the 50 DSMs: identical from the [H][W][V] and [V][H][W] layouts, and the
  fused value of every cell lies within its views' range;
* camera fit of 50 views x 200x200x20 points: the double-float projection path and the
  FP64 one give cameras that reproject within 1e-3 px of each other;
* precision form at 16 M points x 50 cameras: BF16X6 within 1e-3 px of the FP64 exact
  projection on a sample;
* batched multi-AOI form (20 AOIs of the 200-AOI set): batched and per-view launches give
  bit-identical fused DSMs;
* depth maps -> DSMs (2 views x 4096^2 onto 2000 x 2000 at 0.3 m): the fused path and the
  points path give bit-identical DSMs, and one full view's 14 M points lie within 1e-6 m of
  the oracle's numpy chain (a few seconds on the host).
"""
import numpy as np
import pytest
import torch

from conftest import same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def aoi50():
    from vissatsatellitestereo_gb300 import synth
    scene, views = synth.aoi50_raster_case()
    dev = torch.device('cuda')
    n = views[0].height * views[0].width
    pts = torch.empty((len(views) * n, 3), dtype=torch.float64, device=dev)
    for v, spec in enumerate(views):
        pts[v * n:(v + 1) * n] = synth.view_points_torch(scene, spec, dev)
    offsets = torch.arange(0, len(views) + 1, dtype=torch.int64, device=dev) * n
    g = scene.grid
    args = (g.xoff, g.yoff, g.xres, g.yres, g.xsize, g.ysize)
    yield pts, offsets, args, n
    del pts
    torch.cuda.empty_cache()


def test_full_size_raster_schedules_and_batch_independence(aoi50):
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    pts, offsets, args, n = aoi50
    serial = dsm_from_points(pts, offsets, *args)
    over = dsm_from_points(pts, offsets, *args, epilogue_stream=torch.cuda.Stream())
    pipe = dsm_from_points(pts, offsets, *args, pipelined=True)
    torch.cuda.synchronize()
    assert torch.equal(serial.view(torch.int32), over.view(torch.int32))
    assert torch.equal(serial.view(torch.int32), pipe.view(torch.int32))
    for v in (0, 17, 49):
        alone = dsm_from_points(pts[v * n:(v + 1) * n], torch.tensor([0, n]), *args)
        assert torch.equal(alone[0].view(torch.int32), serial[v].view(torch.int32)), v
    finite = torch.isfinite(serial)
    assert finite.float().mean() > 0.9                      # the views cover the grid
    assert float(serial[finite].min()) > -5.0 and float(serial[finite].max()) < 85.0


def test_full_size_view_matches_oracle(aoi50):
    """One full 4096^2 view (16.8 M points) against the oracle's proj_to_grid + blur, bit-exact."""
    from oracle import blur, raster
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    pts, offsets, args, n = aoi50
    v = 17
    got = dsm_from_points(pts[v * n:(v + 1) * n], torch.tensor([0, n]), *args)[0].cpu().numpy()
    host = pts[v * n:(v + 1) * n].cpu().numpy()
    ref = blur.median_blur3x3(raster.proj_to_grid(host, *args).astype(np.float32))
    assert same_bits(got, ref)


def test_full_size_fusion_band_matches_oracle(aoi50):
    """A 96-row band of the 50-view fusion against the reference's numpy calls, bit-exact,
    unblurred and blurred (the band's blur is compared away from its cut edges)."""
    from oracle import blur, fuse
    from vissatsatellitestereo_gb300.aggregate_2p5d import fuse_dsms
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    pts, offsets, args, n = aoi50
    dsms = dsm_from_points(pts, offsets, *args)
    plain = fuse_dsms(dsms, median_blur=False, layout='vhw').cpu().numpy()
    blurred = fuse_dsms(dsms, median_blur=True, layout='vhw').cpu().numpy()
    r0, r1 = 952, 1048
    band = dsms[:, r0:r1].permute(1, 2, 0).contiguous().cpu().numpy()
    ref = fuse.fuse_numpy(band)
    assert same_bits(plain[r0:r1], ref)
    assert same_bits(blurred[r0 + 1:r1 - 1], blur.median_blur3x3(ref)[1:-1])


def test_full_size_fusion_layouts_and_range(aoi50):
    from vissatsatellitestereo_gb300.aggregate_2p5d import fuse_dsms
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points
    pts, offsets, args, n = aoi50
    dsms = dsm_from_points(pts, offsets, *args)
    vhw = fuse_dsms(dsms, median_blur=False, layout='vhw')
    hwv = fuse_dsms(dsms.permute(1, 2, 0).contiguous(), median_blur=False, layout='hwv')
    torch.cuda.synchronize()
    assert torch.equal(vhw.view(torch.int32), hwv.view(torch.int32))
    lo = torch.nan_to_num(dsms, nan=float('inf')).amin(0)
    hi = torch.nan_to_num(dsms, nan=float('-inf')).amax(0)
    ok = torch.isfinite(vhw)
    assert bool(((vhw[ok] >= lo[ok]) & (vhw[ok] <= hi[ok])).all())


def test_full_size_camera_fit_fast_vs_exact():
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.camera_approx import approx_perspective_enu, params_to_krt
    metas = [synth.make_rpc_meta(synth.BASE_SEED + 1000 + v, 4096, 4096) for v in range(50)]
    grids = [synth.rpc_sample_grid_torch(m, 200, 20, 'cuda') for m in metas]
    st = {k: torch.stack([g[k] for g in grids]) for k in ('lat', 'lon', 'alt', 'x', 'y', 'z')}
    args = (st['lat'], st['lon'], st['alt'], st['x'], st['y'], st['z'])
    pf, ef, sf = approx_perspective_enu(metas, *args, mode='fast', shared_points=False)
    pe, ee, se = approx_perspective_enu(metas, *args, mode='exact', shared_points=False)
    assert bool((sf == 0).all()) and bool((se == 0).all())
    pf, pe = pf.cpu().numpy(), pe.cpu().numpy()
    idx = np.arange(0, 800000, 997)
    for v in range(0, 50, 7):
        X = np.stack([st[k][v, idx].cpu().numpy() for k in ('x', 'y', 'z')])
        P = []
        for p in (pf[v], pe[v]):
            K, R, t = params_to_krt(p)
            h = K @ (R @ X + t)
            P.append(h[:2] / h[2])
        assert np.max(np.hypot(*(P[0] - P[1]))) < 1e-3, v


def test_full_size_precision_form_bf16x6():
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.rpc_model import project_cameras, project_cube
    metas = [synth.make_rpc_meta(synth.BASE_SEED + 1000 + v, 4096, 4096) for v in range(50)]
    n = 16 << 20
    gen = torch.Generator(device='cuda').manual_seed(5)
    xyz = torch.rand((3, n), generator=gen, device='cuda') * 2 - 1
    out = project_cube(metas, xyz, 'bf16x6')
    s = xyz[:, ::4099].double()
    la = torch.stack([s[0] * m['rpc']['latScale'] + m['rpc']['latOff'] for m in metas])
    lo = torch.stack([s[1] * m['rpc']['lonScale'] + m['rpc']['lonOff'] for m in metas])
    al = torch.stack([s[2] * m['rpc']['altScale'] + m['rpc']['altOff'] for m in metas])
    col, row = project_cameras(metas, la, lo, al, mode='exact', shared=False)
    err = torch.maximum((out[:, 0, ::4099].double() - col).abs().max(), (out[:, 1, ::4099].double() - row).abs().max())
    assert float(err) <= 1e-3
    del out


def test_batched_form_batched_equals_per_view_launches():
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.engine import AoiSetEngine
    specs = synth.make_aoi_set(200)[:20]
    pool = synth.height_map_pool(8, max(s.image for s in specs), device='cuda')
    eng = AoiSetEngine(specs, pool, [synth.aoi_view_affines(s) for s in specs], budget_bytes=24 << 30)
    eng.step('batched')
    batched = eng.fused.clone()
    eng.step('per_view')
    torch.cuda.synchronize()
    assert same_bits(batched.cpu().numpy(), eng.fused.cpu().numpy())
    eng.step('graph')
    torch.cuda.synchronize()
    assert same_bits(batched.cpu().numpy(), eng.fused.cpu().numpy())
    eng.close()


def test_full_size_depth_fused_equals_points_and_oracle():
    from oracle import geo
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.aggregate_2p5d_util import depth_map_to_points, dsm_from_depth_maps
    from vissatsatellitestereo_gb300.produce_dsm import dsm_from_points

    def utm(la, lo, z, s):
        e, n = geo.geodetic_to_utm(np.array([la]), np.array([lo]), z, s)
        return float(e[0]), float(n[0])

    case = synth.make_depth_case(synth.BASE_SEED + 3000, 2, 4096, 4096, utm, aoi_m=600.0, n_boxes=300)
    aoi = case.aoi
    grid = (aoi['ul_easting'], aoi['ul_northing'], 0.3, 0.3, 2000, 2000)
    depths = [synth.depth_map_torch(case, v, 'cuda') for v in range(2)]
    fused = dsm_from_depth_maps(depths, list(case.inv_proj), aoi, grid)
    pts = [depth_map_to_points(d, case.inv_proj[v], aoi) for v, d in enumerate(depths)]
    offs = torch.tensor(np.cumsum([0] + [p.shape[0] for p in pts]), dtype=torch.int64)
    two_step = dsm_from_points(torch.cat(pts), offs, *grid)
    torch.cuda.synchronize()
    assert same_bits(fused.cpu().numpy(), two_step.cpu().numpy())
    assert float(torch.isfinite(fused).float().mean()) > 0.8     # corners of the rotated UTM grid stay empty
    lat0 = (aoi['lat_min'] + aoi['lat_max']) / 2
    lon0 = (aoi['lon_min'] + aoi['lon_max']) / 2
    ref, _, _ = geo.depth_to_points(depths[0].cpu().numpy(), case.inv_proj[0], lat0, lon0, aoi['alt_min'])
    ours = pts[0].cpu().numpy()
    assert ours.shape == ref.shape and np.abs(ours - ref).max() < 1e-6
