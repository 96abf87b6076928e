"""Batched ``produce_dsm_from_points`` (produce_dsm.py:46-58): every view's point cloud
rasterised onto one DSM grid (proj_to_grid) and median-blurred in float32, in one call."""
import ctypes

import numpy as np
import torch

from . import _lib
from ._dev import as_device, ptr, require_cuda, stream_handle, workspace

E_RESOLUTION = 0.5   # produce_dsm.py:41-42
N_RESOLUTION = 0.5


def grid_size(aoi_width, aoi_height, e_resolution=E_RESOLUTION, n_resolution=N_RESOLUTION):
    """(e_size, n_size) as produce_dsm.py:54-55 derives them."""
    return int(aoi_width / e_resolution) + 1, int(aoi_height / n_resolution) + 1


def dsm_from_points(points, offsets, xoff, yoff, xresolution, yresolution, xsize, ysize, out=None,
                    epilogue_stream=None, bin_events=None):
    """points: (total, 3) float64 (device tensor or array); offsets: (V+1,) int64 view
    boundaries.  Returns (V, ysize, xsize) float32 device tensor.

    ``epilogue_stream`` (a torch.cuda.Stream): run each view's decode / hole fill / blur
    there, overlapped with the binning of the next view on the current stream (the
    current stream still covers all the work when the call returns).  ``bin_events`` (with
    ``epilogue_stream``): a list of 2V timing-enabled torch.cuda.Events recorded around
    each view's binning launch on the current stream.

    Points in host memory (a CPU tensor or a numpy array; pinned memory overlaps best) are
    not copied up front: the library copies view by view into a ring of device staging
    buffers on a second stream while the earlier views are binned (the offsets are read on
    the host)."""
    require_cuda()
    if not (isinstance(points, torch.Tensor) and points.is_cuda) and epilogue_stream is None and bin_events is None:
        return _dsm_from_host_points(points, offsets, xoff, yoff, xresolution, yresolution, xsize, ysize, out)
    pts = as_device(points, torch.float64)
    offs = as_device(offsets, torch.int64)
    V = offs.numel() - 1
    xsize, ysize = int(xsize), int(ysize)
    if out is None:
        out = torch.empty((V, ysize, xsize), dtype=torch.float32, device='cuda')
    args = (ptr(pts), ptr(offs), V, float(xoff), float(yoff), float(xresolution), float(yresolution), xsize, ysize,
            ptr(out))
    if epilogue_stream is None:
        wp, wb = workspace(_lib.lib().vs_dsm_from_points_workspace_size(V, xsize, ysize))
        _lib.call('vs_dsm_from_points', *args, wp, wb, stream_handle())
    else:
        wp, wb = workspace(_lib.lib().vs_dsm_from_points_overlap_workspace_size(V, xsize, ysize))
        evs = None
        if bin_events is not None:
            if len(bin_events) != 2 * V:
                raise ValueError('bin_events needs 2 events per view')
            for e in bin_events:        # the event handle exists once the event was recorded
                if not e.cuda_event:
                    e.record()
            evs = (ctypes.c_void_p * (2 * V))(*[e.cuda_event for e in bin_events])
        _lib.call('vs_dsm_from_points_overlap', *args, wp, wb, stream_handle(), epilogue_stream.cuda_stream, evs)
    return out


_copy_streams = {}
HOST_RING = 3


def _dsm_from_host_points(points, offsets, xoff, yoff, xresolution, yresolution, xsize, ysize, out):
    pts = points if isinstance(points, torch.Tensor) else torch.from_numpy(np.asarray(points))
    if pts.dtype != torch.float64 or not pts.is_contiguous():
        pts = pts.to(torch.float64).contiguous()
    offs = offsets.cpu().numpy() if isinstance(offsets, torch.Tensor) else np.asarray(offsets)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    V = offs.size - 1
    xsize, ysize = int(xsize), int(ysize)
    if out is None:
        out = torch.empty((V, ysize, xsize), dtype=torch.float32, device='cuda')
    dev = torch.cuda.current_device()
    cs = _copy_streams.get(dev)
    if cs is None:
        cs = _copy_streams[dev] = torch.cuda.Stream()
    max_view = int(np.max(np.diff(offs))) if V > 0 else 0
    lib = _lib.lib()
    wp, wb = workspace(lib.vs_dsm_from_points_host_workspace_size(max_view, HOST_RING, xsize, ysize))
    _lib.call('vs_dsm_from_points_host', pts.data_ptr() if pts.numel() else None,
              offs.ctypes.data_as(ctypes.c_void_p), V, float(xoff), float(yoff), float(xresolution),
              float(yresolution), xsize, ysize, out.data_ptr(), HOST_RING, wp, wb, stream_handle(), cs.cuda_stream)
    if pts is not points and not pts.is_pinned():
        torch.cuda.current_stream().synchronize()       # a converted temporary: keep it until copied
    return out
