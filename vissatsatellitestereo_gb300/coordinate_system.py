"""ENU <-> geodetic <-> UTM on the GPU: drop-ins for the reference's ``coordinate_system.py``
(``local_to_global``, ``:41-50``) and ``lib/latlon_utm_converter.py`` (``latlon_to_eastnorh``,
``:38-52``), plus the frame plan shared with the depth map -> points path.

The reference calls pymap3d 1.7.15 (``enu2geodetic``), utm 0.4.2 (zone of the first point)
and pyproj 2.4.0 (UTM projection).  The library restates their published algorithms in
FP64 on the device (ENU -> ECEF rotation, You 2000 for ECEF -> geodetic, Krueger's series to
n^6 for transverse Mercator); see ``include/vissat_gb300.h``.

The ENU origin of an AOI is its centre latitude/longitude and lowest altitude
(``coordinate_system.py:44-47``).
"""
import ctypes
import json
import math
import os

import numpy as np
import torch

from . import _lib
from ._dev import as_device, is_cuda_tensor, require_cuda, stream_handle

EARTH_RADIUS_M = 6378137.0


def load_aoi(aoi):
    """The AOI dict: given as a dict, or read from ``<work_dir>/aoi.json`` like the reference."""
    if isinstance(aoi, dict):
        return aoi
    with open(os.path.join(aoi, 'aoi.json')) as fp:
        return json.load(fp)


def aoi_origin(aoi):
    aoi = load_aoi(aoi)
    lat0 = (aoi['lat_min'] + aoi['lat_max']) / 2.0
    lon0 = (aoi['lon_min'] + aoi['lon_max']) / 2.0
    return lat0, lon0, aoi['alt_min']


def aoi_enu_box(aoi, margin=1.0, pad_m=500.0, pad_up_m=200.0):
    """ENU box of the fast path for an AOI: its latitude/longitude extent at the origin's
    scale, doubled (`margin`) and padded by `pad_m` -- satellite views cropped to an AOI
    reach well beyond it, and the polynomial stays within its validated bound over a few
    km -- with altitudes alt_min .. alt_max padded by `pad_up_m` and the Earth-curvature
    drop across the box.  Points outside take the FP64 chain."""
    aoi = load_aoi(aoi)
    lat0, lon0, alt0 = aoi_origin(aoi)
    rad = math.pi / 180.0
    he = 0.5 * (aoi['lon_max'] - aoi['lon_min']) * rad * EARTH_RADIUS_M * math.cos(lat0 * rad)
    hn = 0.5 * (aoi['lat_max'] - aoi['lat_min']) * rad * EARTH_RADIUS_M
    he = he * (1.0 + margin) + pad_m
    hn = hn * (1.0 + margin) + pad_m
    drop = (he * he + hn * hn) / (2.0 * EARTH_RADIUS_M)
    lo = (-he, -hn, -pad_up_m - drop)
    hi = (he, hn, aoi['alt_max'] - alt0 + pad_up_m)
    return lo, hi


def utm_zone(lat, lon):
    """utm 0.4.2 ``latlon_to_zone_number``: 6-degree zones with the Norway and Svalbard
    exceptions."""
    if 56 <= lat < 64 and 3 <= lon < 12:
        return 32
    if 72 <= lat <= 84 and lon >= 0:
        if lon < 9:
            return 31
        if lon < 21:
            return 33
        if lon < 33:
            return 35
        if lon < 42:
            return 37
    return int((lon + 180) / 6) + 1


class GeoPlan:
    """A frame (ENU origin, UTM zone and hemisphere) with its validated fast-path box, on the
    current device.  Creating one synchronises the current stream."""

    def __init__(self, lat0, lon0, alt0, zone, south, box_lo=None, box_hi=None):
        require_cuda()
        lib = _lib.lib()
        nbytes = lib.vs_geo_plan_device_bytes()
        self.buffer = torch.empty(int(nbytes), dtype=torch.uint8, device='cuda')
        lo = tuple(box_lo) if box_lo is not None else (0.0, 0.0, 0.0)
        hi = tuple(box_hi) if box_hi is not None else (0.0, 0.0, 0.0)
        frame = _lib.VsGeoFrame(float(lat0), float(lon0), float(alt0), int(zone), int(bool(south)),
                                (ctypes.c_double * 3)(*lo), (ctypes.c_double * 3)(*hi))
        handle = ctypes.c_void_p()
        _lib.call('vs_geo_plan_create', ctypes.byref(frame), self.buffer.data_ptr(), nbytes, ctypes.byref(handle),
                  stream_handle())
        self.handle = handle
        self.zone, self.south = int(zone), bool(south)
        self.origin = (float(lat0), float(lon0), float(alt0))
        err = ctypes.c_double()
        en = ctypes.c_int32()
        _lib.call('vs_geo_plan_query', handle, ctypes.byref(err), ctypes.byref(en))
        self.max_err_m = err.value
        self.fast_enabled = bool(en.value)

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h:
            _lib.lib().vs_geo_plan_destroy(h)
            self.handle = None


_plans = {}


def plan_for(lat0, lon0, alt0, zone, south, box=None):
    """Cached GeoPlan per (device, frame, box)."""
    key = (torch.cuda.current_device(), float(lat0), float(lon0), float(alt0), int(zone), bool(south),
           None if box is None else (tuple(box[0]), tuple(box[1])))
    p = _plans.get(key)
    if p is None:
        p = GeoPlan(lat0, lon0, alt0, zone, south, *(box if box is not None else (None, None)))
        _plans[key] = p
    return p


def _out_like(ref, t):
    return t if is_cuda_tensor(ref) else t.cpu().numpy()


def enu_to_geodetic(e, n, u, lat0, lon0, alt0):
    """pymap3d ``enu2geodetic`` (FP64 on the device): ENU metres -> lat, lon (degrees), alt."""
    require_cuda()
    shape = np.shape(e) if not isinstance(e, torch.Tensor) else tuple(e.shape)
    enu = torch.stack([as_device(x, torch.float64).reshape(-1) for x in (e, n, u)], dim=1).contiguous()
    count = enu.shape[0]
    plan = plan_for(lat0, lon0, alt0, 1, False)        # the zone does not enter this conversion
    out = torch.empty((3, count), dtype=torch.float64, device='cuda')
    _lib.call('vs_enu_to_geodetic', plan.handle, enu.data_ptr(), count, 3, out[0].data_ptr(), out[1].data_ptr(),
              out[2].data_ptr(), stream_handle())
    return tuple(_out_like(e, out[i].reshape(shape)) for i in range(3))


def local_to_global(aoi, xx, yy, zz):
    """``coordinate_system.local_to_global``: ENU about the AOI origin -> lat, lon, alt."""
    return enu_to_geodetic(xx, yy, zz, *aoi_origin(aoi))


def latlon_to_eastnorh(lat, lon):
    """``lib/latlon_utm_converter.latlon_to_eastnorh``: every point projected in the zone of
    the first point; AssertionError when the points are not all in one hemisphere."""
    require_cuda()
    shape = np.shape(lat) if not isinstance(lat, torch.Tensor) else tuple(lat.shape)
    la = as_device(lat, torch.float64).reshape(-1)
    lo = as_device(lon, torch.float64).reshape(-1)
    first_lat, first_lon = (float(v) for v in torch.stack([la[0], lo[0]]).cpu())
    south = first_lat < 0
    plan = plan_for(0.0, 0.0, 0.0, utm_zone(first_lat, first_lon), south)
    out = torch.empty((2, la.numel()), dtype=torch.float64, device='cuda')
    flags = torch.zeros(1, dtype=torch.int32, device='cuda')
    _lib.call('vs_geodetic_to_utm', plan.handle, la.data_ptr(), lo.data_ptr(), la.numel(), out[0].data_ptr(),
              out[1].data_ptr(), flags.data_ptr(), stream_handle())
    assert not (int(flags.item()) & _lib.VS_GEO_FLAG_HEMISPHERE), 'points lie in both hemispheres'
    return _out_like(lat, out[0].reshape(shape)), _out_like(lat, out[1].reshape(shape))
