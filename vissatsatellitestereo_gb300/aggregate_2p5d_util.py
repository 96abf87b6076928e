"""Depth maps -> UTM points -> per-view DSMs on the GPU: the numeric core of the reference's
``aggregate_2p5d_util.convert_depth_map_worker`` (``aggregate_2p5d_util.py:75-98``) feeding
``produce_dsm_from_points`` (``produce_dsm.py:46-58``).

``depth_map_to_points`` returns the reference's ``points`` array: for every pixel whose
depth is > 0 and whose homogeneous z is not NaN, in row-major pixel order, the UTM
(easting, northing, altitude) of inv_proj @ [col, row, 1, depth] after the homogeneous
divide, ENU -> geodetic about the AOI origin, and geodetic -> UTM in the zone and hemisphere
of the first point.  ``dsm_from_depth_maps`` bins those points straight into per-view DSMs
without materialising them (same bits as ``depth_map_to_points`` + ``dsm_from_points``).

File reading (``colmap/read_dense.read_array``, ``inv_proj_mats.txt``) is in ``io_formats``;
the visualisation the reference also writes (``plot_height_map``) is out of scope.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._dev import VsError, as_device, is_cuda_tensor, require_cuda, stream_handle, workspace
from .coordinate_system import aoi_enu_box, aoi_origin, enu_to_geodetic, load_aoi, plan_for, utm_zone
from .produce_dsm import E_RESOLUTION, N_RESOLUTION, dsm_from_points, grid_size

MODES = {'exact': _lib.VS_GEO_EXACT, 'fast': _lib.VS_GEO_FAST}


def _matrix(inv_proj_mat):
    m = np.ascontiguousarray(np.asarray(inv_proj_mat, dtype=np.float64).reshape(4, 4))
    if not np.all(np.isfinite(m)):
        raise ValueError('inverse projection matrix must be finite')
    return m


def first_point_zone(depth, inv_proj_mat, lat0, lon0, alt0):
    """(zone, south) of the first valid pixel, as ``latlon_to_eastnorh`` takes them from
    ``lat[0, 0], lon[0, 0]``; None when the map has no valid pixel.  A pixel with a finite
    positive depth is valid unless its homogeneous w is zero."""
    m = torch.from_numpy(_matrix(inv_proj_mat)).cuda()
    flat = depth.reshape(-1)
    ok = (flat > 0) & torch.isfinite(flat)
    W = depth.shape[1]
    start = 0
    while True:
        tail = ok[start:]
        if tail.numel() == 0 or not bool(tail.any()):
            return None
        i = start + int(torch.argmax(tail.to(torch.uint8)))
        r, c = divmod(i, W)
        vec = torch.stack([torch.tensor(float(c), dtype=torch.float64, device='cuda'),
                           torch.tensor(float(r), dtype=torch.float64, device='cuda'),
                           torch.ones((), dtype=torch.float64, device='cuda'), flat[i].double()])
        tmp = m @ vec
        if float(tmp[3]) != 0.0:
            enu = tmp[:3] / tmp[3]
            lat, lon, _ = enu_to_geodetic(enu[0:1], enu[1:2], enu[2:3], lat0, lon0, alt0)
            la, lo = float(lat[0]), float(lon[0])
            return utm_zone(la, lo), la < 0
        start = i + 1


def _plan(depth, inv_proj_mat, aoi, zone, south, box):
    lat0, lon0, alt0 = aoi_origin(aoi)
    if zone is None:
        zs = first_point_zone(depth, inv_proj_mat, lat0, lon0, alt0)
        if zs is None:
            return None
        zone, south = zs
    if isinstance(box, str) and box == 'aoi':
        box = aoi_enu_box(aoi)
    return plan_for(lat0, lon0, alt0, zone, bool(south), box)


def depth_map_to_points(depth_map, inv_proj_mat, aoi, mode='fast', zone=None, south=None, box='aoi'):
    """(N, 3) float64 UTM points (easting, northing, altitude) of a depth map.

    depth_map: (H, W) float32 (``read_array`` layout); inv_proj_mat: the view's 4x4 matrix;
    aoi: the AOI dict or the work_dir holding aoi.json (origin = its centre and lowest
    altitude).  zone / south: UTM zone and hemisphere; None takes them from the first point
    like the reference.  box: the ENU box of the fast path ('aoi': the AOI's extent with a
    margin; None: FP64 everywhere).  Returns a device tensor for a device input, else numpy.
    Raises AssertionError when the points lie in both hemispheres (the reference asserts)."""
    require_cuda()
    aoi = load_aoi(aoi)
    depth = as_device(depth_map, torch.float32)
    if depth.dim() != 2:
        raise ValueError('depth map must be 2-D (height, width)')
    H, W = depth.shape
    plan = _plan(depth, inv_proj_mat, aoi, zone, south, box)
    if plan is None:
        pts = torch.empty((0, 3), dtype=torch.float64, device='cuda')
        return pts if is_cuda_tensor(depth_map) else pts.cpu().numpy()
    m = _matrix(inv_proj_mat)
    points = torch.empty((H * W, 3), dtype=torch.float64, device='cuda')
    count = torch.zeros(1, dtype=torch.int64, device='cuda')
    flags = torch.zeros(1, dtype=torch.int32, device='cuda')
    wp, wb = workspace(_lib.lib().vs_depth_to_points_workspace_size(H, W))
    _lib.call('vs_depth_to_points', depth.data_ptr(), H, W, m.ctypes.data_as(ctypes.c_void_p), plan.handle,
              MODES[mode], points.data_ptr(), count.data_ptr(), flags.data_ptr(), wp, wb, stream_handle())
    n, fl = (int(v) for v in torch.cat([count, flags.to(torch.int64)]).cpu())
    assert not (fl & _lib.VS_GEO_FLAG_HEMISPHERE), 'points lie in both hemispheres'
    pts = points[:n]
    return pts if is_cuda_tensor(depth_map) else pts.cpu().numpy()


def aoi_grid(aoi, e_resolution=E_RESOLUTION, n_resolution=N_RESOLUTION):
    """(xoff, yoff, xres, yres, xsize, ysize) of ``produce_dsm_from_points`` for an AOI."""
    aoi = load_aoi(aoi)
    xsize, ysize = grid_size(aoi['width'], aoi['height'], e_resolution, n_resolution)
    return aoi['ul_easting'], aoi['ul_northing'], e_resolution, n_resolution, xsize, ysize


def dsm_from_depth_maps(depth_maps, inv_proj_mats, aoi, grid=None, mode='fast', zones=None, box='aoi', out=None):
    """Per-view DSMs (V, ysize, xsize) float32 of depth maps, as ``produce_dsm_from_points``
    makes them from ``depth_map_to_points``: nanmax rasterisation, hole fill, float32, 3x3
    median blur.  grid: (xoff, yoff, xres, yres, xsize, ysize), default the AOI's 0.5 m grid.
    zones: per-view (zone, south), default each view's first point.  Views sharing a frame
    go through one fused launch per view; a grid the fused binning cannot take (not inside
    its origins' binades) goes through the points."""
    require_cuda()
    aoi = load_aoi(aoi)
    depths = [as_device(d, torch.float32) for d in depth_maps]
    mats = [_matrix(m) for m in inv_proj_mats]
    if len(depths) != len(mats) or not depths:
        raise ValueError('need one inverse projection matrix per depth map')
    xoff, yoff, xres, yres, xsize, ysize = grid if grid is not None else aoi_grid(aoi)
    xsize, ysize = int(xsize), int(ysize)
    V = len(depths)
    if out is None:
        out = torch.empty((V, ysize, xsize), dtype=torch.float32, device='cuda')
    groups = {}
    for v, d in enumerate(depths):
        key = zones[v] if zones is not None else None
        plan = _plan(d, mats[v], aoi, *(key if key is not None else (None, None)), box)
        if plan is None:                     # no valid pixel: an all-NaN DSM
            out[v].fill_(float('nan'))
            continue
        groups.setdefault(id(plan), (plan, []))[1].append(v)
    for plan, views in groups.values():
        ptrs = (ctypes.c_void_p * len(views))(*[depths[v].data_ptr() for v in views])
        hs = (ctypes.c_int64 * len(views))(*[depths[v].shape[0] for v in views])
        ws_ = (ctypes.c_int64 * len(views))(*[depths[v].shape[1] for v in views])
        ms = np.ascontiguousarray(np.stack([mats[v] for v in views]))
        contiguous = views == list(range(views[0], views[0] + len(views)))
        dst = out[views[0]:views[0] + len(views)] if contiguous else torch.empty(
            (len(views), ysize, xsize), dtype=torch.float32, device='cuda')
        flags = torch.zeros(1, dtype=torch.int32, device='cuda')
        wp, wb = workspace(_lib.lib().vs_dsm_from_depth_maps_workspace_size(xsize, ysize))
        try:
            _lib.call('vs_dsm_from_depth_maps', ptrs, hs, ws_, len(views), ms.ctypes.data_as(ctypes.c_void_p),
                      plan.handle, MODES[mode], float(xoff), float(yoff), float(xres), float(yres), xsize, ysize,
                      dst.data_ptr(), flags.data_ptr(), wp, wb, stream_handle())
        except VsError as e:
            if e.status != _lib.VS_ERR_ARG or 'binades' not in str(e):
                raise
            pts = [depth_map_to_points(depths[v], mats[v], aoi, mode, plan.zone, plan.south, box) for v in views]
            offs = torch.tensor(np.cumsum([0] + [p.shape[0] for p in pts]), dtype=torch.int64, device='cuda')
            dsm_from_points(torch.cat(pts), offs, xoff, yoff, xres, yres, xsize, ysize, out=dst)
        assert not (int(flags.item()) & _lib.VS_GEO_FLAG_HEMISPHERE), 'points lie in both hemispheres'
        if not contiguous:
            out[views] = dst
    return out
