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
                    epilogue_stream=None, bin_events=None, pipelined=False, launch_events=None):
    """points: (total, 3) float64 (device tensor or array); offsets: (V+1,) int64 view
    boundaries.  Returns (V, ysize, xsize) float32 device tensor.

    ``pipelined``: V + 1 launches on the current stream, each binning one view while its
    other CTAs run the previous view's decode / hole fill / blur (same results);
    ``launch_events`` (with ``pipelined``): 2(V + 1) timing-enabled torch.cuda.Events
    recorded around each launch.

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
    if pipelined and (epilogue_stream is not None or bin_events is not None):
        raise ValueError('pipelined runs on the current stream only (no epilogue_stream, no bin_events)')
    if launch_events is not None and not pipelined:
        raise ValueError('launch_events needs pipelined=True')
    if not (isinstance(points, torch.Tensor) and points.is_cuda) and epilogue_stream is None and bin_events is None \
            and not pipelined:
        return _dsm_from_host_points(points, offsets, xoff, yoff, xresolution, yresolution, xsize, ysize, out)
    pts = as_device(points, torch.float64)
    offs = as_device(offsets, torch.int64)
    V = offs.numel() - 1
    xsize, ysize = int(xsize), int(ysize)
    if out is None:
        out = torch.empty((V, ysize, xsize), dtype=torch.float32, device='cuda')
    args = (ptr(pts), ptr(offs), V, float(xoff), float(yoff), float(xresolution), float(yresolution), xsize, ysize,
            ptr(out))
    if pipelined:
        wp, wb = workspace(_lib.lib().vs_dsm_from_points_pipelined_workspace_size(V, xsize, ysize))
        _lib.call('vs_dsm_from_points_pipelined', *args, wp, wb, stream_handle(),
                  _event_array(launch_events, 2 * (V + 1)))
    elif epilogue_stream is None:
        wp, wb = workspace(_lib.lib().vs_dsm_from_points_workspace_size(V, xsize, ysize))
        _lib.call('vs_dsm_from_points', *args, wp, wb, stream_handle())
    else:
        wp, wb = workspace(_lib.lib().vs_dsm_from_points_overlap_workspace_size(V, xsize, ysize))
        _lib.call('vs_dsm_from_points_overlap', *args, wp, wb, stream_handle(), epilogue_stream.cuda_stream,
                  _event_array(bin_events, 2 * V))
    return out


def _event_array(events, count):
    """ctypes array of the cudaEvent_t handles of torch.cuda.Events (None stays None)."""
    if events is None:
        return None
    if len(events) != count:
        raise ValueError(f'expected {count} events, got {len(events)}')
    for e in events:            # the event handle exists once the event was recorded
        if not e.cuda_event:
            e.record()
    return (ctypes.c_void_p * count)(*[e.cuda_event for e in events])


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
