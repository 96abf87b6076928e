"""Generate the golden vectors of the geometry path from the reference's own code.

Run once in a container where the reference checkout is present:

    python tests/golden/make_golden.py --ref <reference checkout> [--sections ...]

(or with the checkout in $VISSAT_REFERENCE).

It imports the reference modules that import cleanly (``lib/rpc_model.py``,
``lib/solve_perspective.py``, ``lib/check_error.py``, ``lib/gen_grid.py``,
``lib/solve_affine.py``) and executes
the reference's source for the two routines whose modules do not import:

* ``lib/proj_to_grid.py`` -- needs ``numpy_groupies`` (absent) and ``np.int`` (removed
  from numpy).  The module source is executed with ``np.int`` aliased to ``np.int64``
  and a stand-in ``numpy_groupies`` module whose ``aggregate(func='nanmax')`` restates
  numpy_groupies 0.9.9's numba implementation (see ``oracle/raster.py``).  Binning and
  the hole-fill loop are therefore the reference's own lines.
* ``aggregate_2p5d_util.py`` -- imports cv2 through produce_dsm.  The depth map -> ENU
  block of ``convert_depth_map_worker`` is cut out and executed as is (its geodesy calls
  pymap3d/pyproj, absent, and stays with the oracle's restatement).
* ``aggregate_2p5d.py`` -- needs cv2/GDAL/imageio.  The fusion block (from
  ``cnt = len(all_dsm)`` to the ``np.nanmean`` line) is cut out of ``run_fuse`` and
  executed as is.

Inputs come from the seeded synthetic generators, so the fixtures are reproducible.
The reference is never imported at test time: tests read the ``.npz`` files only.
"""
import argparse
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.dont_write_bytecode = True   # never write __pycache__ into the reference tree

from vissatsatellitestereo_gb300 import synth  # noqa: E402


def _fake_numpy_groupies():
    mod = types.ModuleType('numpy_groupies')

    def aggregate(group_idx, a, func='sum', size=None, fill_value=0, **kw):
        assert func == 'nanmax'
        size = int(group_idx.max()) + 1 if size is None else size
        out = np.full(size, fill_value, dtype=np.float64)
        seen = np.zeros(size, dtype=bool)
        for g, v in zip(group_idx.tolist(), a.tolist()):   # numba kernel, sequential
            if v != v:
                continue
            if not seen[g]:
                out[g] = v
                seen[g] = True
            elif out[g] < v:
                out[g] = v
        return out

    mod.aggregate = aggregate
    return mod


def load_proj_to_grid(ref):
    src = open(os.path.join(ref, 'lib', 'proj_to_grid.py')).read()
    sys.modules['numpy_groupies'] = _fake_numpy_groupies()
    had_int = hasattr(np, 'int')
    np.int = np.int64
    ns = {}
    exec(compile(src, os.path.join(ref, 'lib', 'proj_to_grid.py'), 'exec'), ns)
    return ns['proj_to_grid'], had_int


def fusion_block(ref):
    lines = open(os.path.join(ref, 'aggregate_2p5d.py')).read().splitlines()
    start = next(i for i, l in enumerate(lines) if l.strip().startswith('cnt = len(all_dsm)'))
    end = next(i for i, l in enumerate(lines) if 'np.nanmean(all_dsm, axis=2)' in l)
    body = '\n'.join(l[4:] for l in lines[start:end + 1])
    return compile(body, os.path.join(ref, 'aggregate_2p5d.py'), 'exec')


def inverse_and_affine(ref, seed):
    """(e) RPCModel.inverse_projection on 1-D inputs (the shape its np.vstack(...).T
    expects) and (f) solve_affine on lat/lon/alt grids, as approx_affine_latlonalt calls it."""
    from lib.rpc_model import RPCModel
    from lib.solve_affine import solve_affine
    inv = {}
    for i, size in enumerate((2048, 4096, 8192)):
        meta = synth.make_rpc_meta(seed + 600 + i, size, size)
        r = meta['rpc']
        rng = np.random.default_rng(seed + 610 + i)
        n = 400
        col = rng.uniform(0, size, n)
        row = rng.uniform(0, size, n)
        alt = r['altOff'] + r['altScale'] * rng.uniform(-1, 1, n)
        lon, lat, _ = RPCModel(meta).inverse_projection(col, row, alt)
        lon_n, lat_n, alt_n = RPCModel(meta).inverse_projection(col, row, alt, return_normalized=True)
        inv[f'cam{i}'] = dict(meta=np.array(repr(meta)), col=col, row=row, alt=alt, lon=lon, lat=lat,
                              lon_n=lon_n, lat_n=lat_n, alt_n=alt_n)
    np.savez_compressed(os.path.join(HERE, 'rpc_inverse.npz'),
                        **{f'{k}_{f}': v[f] for k, v in inv.items() for f in v})
    aff = {}
    for i, size in enumerate((2048, 4096)):
        meta = synth.make_rpc_meta(seed + 700 + i, size, size)
        g = synth.rpc_sample_grid(meta, 25, 6)
        col, row = RPCModel(meta).projection(g.lat, g.lon, g.alt)
        keep = (col >= 0) & (row >= 0) & (col < size) & (row < size)
        P = solve_affine(g.lat, g.lon, g.alt, col, row, keep)
        aff[f'cam{i}'] = dict(meta=np.array(repr(meta)), lat=g.lat, lon=g.lon, alt=g.alt, col=col, row=row,
                              keep=keep, P=P)
    np.savez_compressed(os.path.join(HERE, 'affine_fit.npz'),
                        **{f'{k}_{f}': v[f] for k, v in aff.items() for f in v})


def ply_files(ref, seed):
    """(g) lib/ply_np_converter.np2ply binary outputs (its text mode raises with the vendored
    plyfile): float32 without colour, float32 with colour and comments, float64."""
    from lib.ply_np_converter import np2ply
    rng = np.random.default_rng(seed + 800)
    v = rng.normal(0.0, 100.0, (37, 3)) + np.array([354052.0, 6182702.0, 50.0])
    c = rng.integers(0, 256, (37, 3)).astype(np.uint8)
    np.savez_compressed(os.path.join(HERE, 'ply_inputs.npz'), vertex=v, color=c)
    np2ply(v, os.path.join(HERE, 'ply_f32.ply'))
    np2ply(v, os.path.join(HERE, 'ply_f32_color.ply'), color=c, comments=['VisSat point cloud', 'utm 17N'])
    np2ply(v, os.path.join(HERE, 'ply_f64.ply'), use_double=True)


def depth_block(ref):
    """The depth map -> ENU lines of aggregate_2p5d_util.convert_depth_map_worker (from the
    depth <= 0 replacement to ``points = tmp[:, valid_mask].T``), cut out of the function
    (its module imports cv2 through produce_dsm) and compiled as they are."""
    lines = open(os.path.join(ref, 'aggregate_2p5d_util.py')).read().splitlines()
    start = next(i for i, l in enumerate(lines) if 'depth_map[depth_map <= 0.0] = np.nan' in l)
    end = next(i for i, l in enumerate(lines) if l.strip().startswith('points = tmp[:, valid_mask].T'))
    body = '\n'.join(l[4:] for l in lines[start:end + 1])
    return compile(body, os.path.join(ref, 'aggregate_2p5d_util.py'), 'exec')


def _colmap_bytes(arr):
    """A COLMAP dense array file: "width&height&channels&" then float32 column-major
    (width, height, channels), written here from the format's description."""
    a = arr if arr.ndim == 3 else arr[:, :, None]
    h, w, c = a.shape
    body = np.asfortranarray(np.transpose(a, (1, 0, 2)).astype('<f4')).tobytes(order='F')
    return f'{w}&{h}&{c}&'.encode() + body


def depth_files(ref, seed):
    """(h) colmap/read_dense.read_array on a depth map (1 channel) and a normal map (3
    channels); the depth -> ENU block of convert_depth_map_worker on two synthetic views."""
    from colmap.read_dense import read_array
    sys.path.insert(0, REPO)
    from oracle import geo
    rng = np.random.default_rng(seed + 900)
    depth = rng.uniform(-1.0, 2.0, (23, 37)).astype(np.float32)
    normal = rng.normal(0.0, 1.0, (23, 37, 3)).astype(np.float32)
    out = {}
    for name, arr in (('depth', depth), ('normal', normal)):
        path = os.path.join(HERE, f'colmap_{name}.bin')
        with open(path, 'wb') as f:
            f.write(_colmap_bytes(arr))
        out[f'{name}_written'] = arr
        out[f'{name}_read'] = read_array(path)
    np.savez_compressed(os.path.join(HERE, 'colmap_arrays.npz'), **out)

    def utm(la, lo, z, s):
        e, n = geo.geodetic_to_utm(np.array([la]), np.array([lo]), z, s)
        return float(e[0]), float(n[0])

    case = synth.make_depth_case(seed + 950, 2, 40, 56, utm, aoi_m=60.0, n_boxes=8)
    block = depth_block(ref)
    res = {'aoi': np.array(repr(case.aoi))}
    for v in range(2):
        depth_map = synth.depth_map_torch(case, v).numpy()
        depth_map[3, 5] = np.nan
        depth_map[4, 7] = np.inf
        ns = {'np': np, 'depth_map': depth_map.copy(), 'inv_proj_mats': {'img': case.inv_proj[v]},
              'img_name': 'img'}
        exec(block, ns)
        res[f'v{v}_depth'] = depth_map
        res[f'v{v}_inv_proj'] = case.inv_proj[v]
        res[f'v{v}_points4'] = ns['points']
        res[f'v{v}_valid'] = ns['valid_mask']
        res[f'v{v}_height_map'] = ns['height_map']
    np.savez_compressed(os.path.join(HERE, 'depth_enu.npz'), **res)


from fit_cases import fit_cases  # noqa: E402


def fit_at_size(RPCModel, solve_perspective, check_perspective_error):
    """Reference fits and error statistics at the benchmarked grid sizes.  The grids are not
    stored (the tests regenerate them with ``synth.rpc_sample_grid``); a strided sample of
    each grid is, so a test can tell that its regenerated grid is the one fitted here."""
    out = {}
    for name, metas, n_xy, n_z, _ in fit_cases():
        g = synth.rpc_sample_grid(metas[0], n_xy, n_z)
        out[f'{name}_probe'] = np.hstack((g.lat, g.lon, g.alt, g.x, g.y, g.z))[::997]
        for c, meta in enumerate(metas):
            col, row = RPCModel(meta).projection(g.lat, g.lon, g.alt)
            w, h = meta['width'], meta['height']
            keep = np.logical_and(np.logical_and(col >= 0, row >= 0), np.logical_and(col < w, row < h))
            K, R, t = solve_perspective(g.x, g.y, g.z, col, row, keep)
            err = check_perspective_error(g.x, g.y, g.z, col, row, K, R, t, keep)
            key = f'{name}_cam{c}'
            out[f'{key}_meta'] = np.array(repr(meta))
            out[f'{key}_K'], out[f'{key}_R'], out[f'{key}_t'] = K, R, t
            out[f'{key}_err'] = np.array(err, dtype=np.float64)
            out[f'{key}_kept'] = np.array(int(keep.sum()))
            print(name, c, 'kept', int(keep.sum()), 'of', keep.size, 'err', np.array(err))
    np.savez_compressed(os.path.join(HERE, 'perspective_fit_fullsize.npz'), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('VISSAT_REFERENCE'),
                    help='checkout of the reference (default: $VISSAT_REFERENCE)')
    ap.add_argument('--sections', default='all',
                    help="'all' or a comma list of: base, inverse, formats, depth, fitsize")
    args = ap.parse_args()
    if not args.ref:
        ap.error('give the reference checkout with --ref or $VISSAT_REFERENCE')
    ref = os.path.abspath(args.ref)
    sys.path.insert(0, ref)
    from lib.rpc_model import RPCModel
    from lib.solve_perspective import solve_perspective
    from lib.check_error import check_perspective_error
    from lib.gen_grid import gen_grid

    seed = synth.BASE_SEED
    sections = {'base', 'inverse', 'formats', 'depth', 'fitsize'} if args.sections == 'all' \
        else set(args.sections.split(','))
    if 'fitsize' in sections:
        fit_at_size(RPCModel, solve_perspective, check_perspective_error)
    if 'depth' in sections:
        depth_files(ref, seed)
    if 'inverse' in sections:
        inverse_and_affine(ref, seed)
    if 'formats' in sections:
        ply_files(ref, seed)
    if 'base' not in sections:
        print('golden vectors written to', HERE)
        return

    # (a) RPC projection: three cameras, grid points plus ragged extras (NaN, far away)
    rpc_cases = {}
    for i, size in enumerate((2048, 4096, 8192)):
        meta = synth.make_rpc_meta(seed + 100 + i, size, size)
        r = meta['rpc']
        lat_p = r['latOff'] + r['latScale'] * np.linspace(1.1, -1.1, 15)
        lon_p = r['lonOff'] + r['lonScale'] * np.linspace(-1.1, 1.1, 15)
        alt_p = r['altOff'] + r['altScale'] * np.linspace(-1.0, 1.0, 5)
        lat, lon, alt = gen_grid(lat_p, lon_p, alt_p)
        xs_lat, xs_lon, xs_alt = synth.grid_points(lat_p, lon_p, alt_p)
        assert np.array_equal(lat, xs_lat) and np.array_equal(lon, xs_lon) and np.array_equal(alt, xs_alt)
        extra = np.array([[np.nan, r['lonOff'], r['altOff']],
                          [r['latOff'], np.nan, r['altOff']],
                          [r['latOff'], r['lonOff'], np.inf],
                          [r['latOff'] + 3.0, r['lonOff'] - 3.0, 9000.0]])
        lat = np.vstack((lat, extra[:, 0:1]))
        lon = np.vstack((lon, extra[:, 1:2]))
        alt = np.vstack((alt, extra[:, 2:3]))
        with np.errstate(all='ignore'):
            col, row = RPCModel(meta).projection(lat, lon, alt)
        rpc_cases[f'cam{i}'] = dict(meta=meta, lat=lat, lon=lon, alt=alt, col=col, row=row)
    np.savez_compressed(os.path.join(HERE, 'rpc_projection.npz'),
                        **{f'{k}_{f}': (v[f] if f != 'meta' else np.array(repr(v[f])))
                           for k, v in rpc_cases.items() for f in v})

    # (b) perspective fit: two cameras, 25x25x6 grids, in-image keep masks
    fit = {}
    for i, size in enumerate((2048, 4096)):
        meta = synth.make_rpc_meta(seed + 200 + i, size, size)
        g = synth.rpc_sample_grid(meta, 25, 6)
        col, row = RPCModel(meta).projection(g.lat, g.lon, g.alt)
        keep = (col >= 0) & (row >= 0) & (col < size) & (row < size)
        K, R, t = solve_perspective(g.x, g.y, g.z, col, row, keep)
        err = check_perspective_error(g.x, g.y, g.z, col, row, K, R, t, keep)
        fit[f'cam{i}'] = dict(meta=np.array(repr(meta)), lat=g.lat, lon=g.lon, alt=g.alt,
                              x=g.x, y=g.y, z=g.z, col=col, row=row, keep=keep,
                              K=K, R=R, t=t, err=np.array(err, dtype=np.float64))
    np.savez_compressed(os.path.join(HERE, 'perspective_fit.npz'),
                        **{f'{k}_{f}': v[f] for k, v in fit.items() for f in v})

    # (c) rasterisation: 96x96 height map onto a 50x50 grid at 0.5 m (holes, NaNs,
    # points off the grid), plus the special values the binning must handle
    proj_to_grid, had_int = load_proj_to_grid(ref)
    grid = synth.DsmGrid(synth.EXPLORER_UL_EASTING, synth.EXPLORER_UL_NORTHING, 0.5, 0.5, 50, 50)
    scene = synth.make_scene(seed + 300, grid, 12, 5.0, 60.0)
    view = synth.ViewSpec(96, 96, 0.27, theta=0.05, shift_e=1.0, shift_n=-1.0, nan_frac=0.35,
                          seed=seed + 301)
    pts = synth.view_points(scene, view)
    special = np.array([[np.nan, grid.yoff - 3.0, 7.0],
                        [grid.xoff + 3.0, np.nan, 7.0],
                        [np.inf, grid.yoff - 3.0, 7.0],
                        [grid.xoff + 3.0, -np.inf, 7.0],
                        [grid.xoff + 1e30, grid.yoff - 3.0, 7.0],
                        [grid.xoff - 1e-9, grid.yoff - 3.0, 7.0],       # just west of the grid
                        [grid.xoff + 0.0, grid.yoff - 0.0, 11.0],       # exactly on the UL corner
                        [grid.xoff + 24.99999999, grid.yoff - 24.99999999, 8.0],
                        [grid.xoff + 25.0, grid.yoff - 25.0, -np.inf],  # last cell, -inf only
                        [grid.xoff + 10.2, grid.yoff - 10.2, -0.0],     # zero-sign ties
                        [grid.xoff + 10.3, grid.yoff - 10.3, 0.0],
                        [grid.xoff + 12.2, grid.yoff - 12.2, 0.0],
                        [grid.xoff + 12.3, grid.yoff - 12.3, -0.0]])
    pts = np.vstack((pts, special))
    with np.errstate(all='ignore'):
        dsm = proj_to_grid(pts, grid.xoff, grid.yoff, grid.xres, grid.yres, grid.xsize, grid.ysize,
                           propagate=True)
    if not had_int:
        del np.int
    np.savez_compressed(os.path.join(HERE, 'proj_to_grid.npz'), points=pts, dsm=dsm,
                        grid=np.array([grid.xoff, grid.yoff, grid.xres, grid.yres,
                                       grid.xsize, grid.ysize], dtype=np.float64))

    # (d) fusion: 32x32 cells, V in {9, 50}, random NaN patterns, run through the
    # reference's own block of aggregate_2p5d.run_fuse
    code = fusion_block(ref)
    fused = {}
    rng = np.random.default_rng(seed + 400)
    for V in (9, 50):
        base = rng.normal(20.0, 8.0, (32, 32, 1)).astype(np.float32)
        stack = (base + rng.normal(0.0, 0.5, (32, 32, V))).astype(np.float32)
        outl = rng.random(stack.shape) < 0.1
        stack[outl] += rng.normal(0.0, 30.0, outl.sum()).astype(np.float32)
        stack[rng.random(stack.shape) < rng.uniform(0.05, 0.9, (32, 32, 1))] = np.nan
        stack[0, 0, :] = np.float32(-0.0)
        stack[0, 1, :] = np.nan
        stack[0, 2, :3] = np.float32(5.0)
        stack[0, 2, 3:] = np.nan
        ns = {'np': np, 'all_dsm': [stack[:, :, v:v + 1].copy() for v in range(V)]}
        import warnings
        with warnings.catch_warnings(), np.errstate(all='ignore'):
            warnings.simplefilter('ignore')
            exec(code, ns)
        fused[f'v{V}_stack'] = stack
        fused[f'v{V}_fused'] = ns['all_dsm_mean_no_outliers']
    np.savez_compressed(os.path.join(HERE, 'fusion.npz'), **fused)
    print('golden vectors written to', HERE)


if __name__ == '__main__':
    main()
