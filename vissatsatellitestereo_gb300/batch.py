"""Batched form over many AOIs: per-view FP32 height maps -> per-view DSMs -> fused DSMs.

The reference produces one AOI at a time: per view, the depth map's pixels become UTM
points (aggregate_2p5d_util.py:75-98), ``produce_dsm_from_points`` rasterises them
(produce_dsm.py:46-58: proj_to_grid + the float32 3x3 median blur), and ``run_fuse``
fuses the AOI's views (aggregate_2p5d.py:65-81).  ``AoiBatch`` plans many AOIs at once:
the rasterisation of all their views is one persistent launch over tiles of their DSMs,
each binned and finished in shared memory (``run``), and the fusion follows per AOI
(``fuse``).  A view's points are its
height-map pixels placed by a fixed-point affine pixel -> UTM map (``MapAffine``), whose
coordinates are exact doubles, so every DSM is bit-identical to materialising the FP64
point list and running the per-view reference path.
"""
import ctypes
import math
from dataclasses import dataclass

import torch

from . import _lib
from ._dev import require_cuda, stream_handle

FRAC_BITS = 28


class VsAoi(ctypes.Structure):
    _fields_ = [('xoff', ctypes.c_double), ('yoff', ctypes.c_double), ('xres', ctypes.c_double),
                ('yres', ctypes.c_double), ('xsize', ctypes.c_int64), ('ysize', ctypes.c_int64),
                ('first_view', ctypes.c_int32), ('n_views', ctypes.c_int32)]


class VsMapView(ctypes.Structure):
    _fields_ = [('heights', ctypes.c_void_p), ('row_stride', ctypes.c_int64), ('width', ctypes.c_int32),
                ('height', ctypes.c_int32), ('aoi', ctypes.c_int32), ('reserved', ctypes.c_int32),
                ('e0', ctypes.c_int64), ('n0', ctypes.c_int64), ('ej', ctypes.c_int32), ('ei', ctypes.c_int32),
                ('nj', ctypes.c_int32), ('ni', ctypes.c_int32), ('dsm', ctypes.c_void_p)]


@dataclass
class MapAffine:
    """Pixel (i, j) of a W x H map -> easting (e0 + ej(2j+1-W) + ei(2i+1-H)) 2^-28 and
    northing (n0 + nj(2j+1-W) + ni(2i+1-H)) 2^-28 metres (integers)."""
    e0: int
    n0: int
    ej: int
    ei: int
    nj: int
    ni: int

    @staticmethod
    def rotated(ce, cn, gsd, theta):
        """The synthetic view geometry: pixel centres on a grid of spacing ``gsd`` rotated
        by ``theta`` about the image centre (ce, cn), rows running south."""
        s = float(1 << FRAC_BITS)
        c, sn = math.cos(theta), math.sin(theta)
        return MapAffine(e0=int(round(ce * s)), n0=int(round(cn * s)), ej=int(round(gsd * c / 2 * s)),
                         ei=int(round(-gsd * sn / 2 * s)), nj=int(round(-gsd * sn / 2 * s)),
                         ni=int(round(-gsd * c / 2 * s)))


@dataclass
class AoiGrid:
    xoff: float
    yoff: float
    xres: float
    yres: float
    xsize: int
    ysize: int


@dataclass
class MapView:
    heights: torch.Tensor      # CUDA float32, (H, stride) storage; the view uses [:height, :width]
    width: int
    height: int
    affine: MapAffine
    dsm: torch.Tensor = None   # optional CUDA float32 (ysize, xsize) output of this view's DSM


class AoiBatch:
    """A plan over ``grids`` (one per AOI) and ``views`` (a list per AOI of ``MapView``).

    ``run()`` rasterises all views (or a range) into the per-view DSM buffer;
    ``fuse()`` fuses each AOI's views into the fused buffer.  ``view_dsm(v)`` and
    ``fused_dsm(a)`` return the (H, W) slices."""

    def __init__(self, grids, views, tile=64):
        require_cuda()
        self.grids = list(grids)
        self.views = [list(vs) for vs in views]
        if len(self.grids) != len(self.views):
            raise ValueError('one view list per AOI grid')
        self.tile = int(tile)
        if self.tile not in (32, 64):
            raise ValueError('tile must be 32 or 64')
        n_aois = len(self.grids)
        flat = [(a, v) for a, vs in enumerate(self.views) for v in vs]
        self.n_views = len(flat)
        self.aoi_arr = (VsAoi * n_aois)()
        first = 0
        for a, (g, vs) in enumerate(zip(self.grids, self.views)):
            self.aoi_arr[a] = VsAoi(g.xoff, g.yoff, g.xres, g.yres, g.xsize, g.ysize, first, len(vs))
            first += len(vs)
        self.view_arr = (VsMapView * self.n_views)()
        self._keep = []
        for i, (a, v) in enumerate(flat):
            h = v.heights
            if not (h.is_cuda and h.dtype == torch.float32 and h.dim() == 2 and h.stride(1) == 1):
                raise ValueError('heights must be a 2-D CUDA float32 tensor with unit column stride')
            if h.shape[0] < v.height or h.shape[1] < v.width:
                raise ValueError('heights smaller than the view')
            self._keep.append(h)
            out = 0
            if v.dsm is not None:
                g = self.grids[a]
                if not (v.dsm.is_cuda and v.dsm.dtype == torch.float32 and v.dsm.is_contiguous() and
                        v.dsm.numel() == g.xsize * g.ysize):
                    raise ValueError('dsm must be a contiguous CUDA float32 tensor of the AOI grid size')
                self._keep.append(v.dsm)
                out = v.dsm.data_ptr()
            m = v.affine
            self.view_arr[i] = VsMapView(h.data_ptr(), h.stride(0), v.width, v.height, a, 0, m.e0, m.n0, m.ej, m.ei,
                                         m.nj, m.ni, out or None)
        lib = _lib.lib()
        nbytes = lib.vs_aoi_batch_plan_workspace_size(self.aoi_arr, n_aois, self.n_views)
        self._plan_ws = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device='cuda')
        self._plan = ctypes.c_void_p()
        _lib.call('vs_aoi_batch_plan', self.aoi_arr, n_aois, self.view_arr, self.n_views, self.tile,
                  self._plan_ws.data_ptr(), self._plan_ws.numel(), ctypes.byref(self._plan), stream_handle())
        vc, fc, sb = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_size_t()
        _lib.call('vs_aoi_batch_query', self._plan, ctypes.byref(vc), ctypes.byref(fc), ctypes.byref(sb))
        self.view_cells, self.fused_cells, self.scratch_bytes = vc.value, fc.value, sb.value
        self.view_off = [0]
        self.fused_off = [0]
        for a, (g, vs) in enumerate(zip(self.grids, self.views)):
            for _ in vs:
                self.view_off.append(self.view_off[-1] + g.xsize * g.ysize)
            self.fused_off.append(self.fused_off[-1] + g.xsize * g.ysize)
        self.first_view = [self.aoi_arr[a].first_view for a in range(n_aois)]
        self.view_aoi = [a for a, _ in flat]
        self.pixels = sum(v.width * v.height for _, v in flat)

    def close(self):
        if self._plan:
            _lib.lib().vs_aoi_batch_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def new_view_dsm(self):
        return torch.empty(self.view_cells, dtype=torch.float32, device='cuda')

    def new_fused(self):
        return torch.empty(self.fused_cells, dtype=torch.float32, device='cuda')

    def new_scratch(self):
        return torch.empty(self.scratch_bytes, dtype=torch.uint8, device='cuda')

    def run(self, view_dsm, views=None, blocks_per_sm=4):
        """Rasterise views[0]..views[1]-1 (all by default) into ``view_dsm`` (views with
        their own ``dsm`` output write there; ``view_dsm`` may then be None)."""
        v0, v1 = (0, self.n_views) if views is None else views
        _lib.call('vs_aoi_batch_run', self._plan, v0, v1, int(blocks_per_sm),
                  None if view_dsm is None else view_dsm.data_ptr(), stream_handle())
        return view_dsm

    def fuse(self, view_dsm, fused, scratch, aois=None, median_blur=True):
        a0, a1 = (0, len(self.grids)) if aois is None else aois
        _lib.call('vs_aoi_batch_fuse', self._plan, a0, a1, view_dsm.data_ptr(), fused.data_ptr(),
                  int(bool(median_blur)), scratch.data_ptr(), scratch.numel(), stream_handle())
        return fused

    def view_dsm(self, buf, v):
        g = self.grids[self.view_aoi[v]]
        return buf[self.view_off[v]:self.view_off[v + 1]].view(g.ysize, g.xsize)

    def fused_dsm(self, buf, a):
        g = self.grids[a]
        return buf[self.fused_off[a]:self.fused_off[a + 1]].view(g.ysize, g.xsize)


def map_points(heights, affine, width=None, height=None, out=None):
    """FP64 point list (H*W, 3) [easting, northing, height] of one height-map view in pixel
    order (``vs_map_points``): the per-view points the plain per-view path rasterises.
    ``heights``: CUDA float32 (rows, stride) with unit column stride; ``affine``: MapAffine
    or its dict; the view is heights[:height, :width]."""
    require_cuda()
    if not (heights.is_cuda and heights.dtype == torch.float32 and heights.dim() == 2 and heights.stride(1) == 1):
        raise ValueError('heights must be a 2-D CUDA float32 tensor with unit column stride')
    height = heights.shape[0] if height is None else int(height)
    width = heights.shape[1] if width is None else int(width)
    m = affine if isinstance(affine, MapAffine) else MapAffine(**affine)
    n = width * height
    if out is None:
        out = torch.empty((n, 3), dtype=torch.float64, device='cuda')
    elif out.shape != (n, 3) or out.dtype != torch.float64 or not out.is_contiguous():
        raise ValueError('out must be a contiguous (H*W, 3) float64 CUDA tensor')
    _lib.call('vs_map_points', heights.data_ptr(), heights.stride(0), width, height, m.e0, m.n0, m.ej, m.ei, m.nj,
              m.ni, out.data_ptr(), stream_handle())
    return out


def upload_map(heights, width=None, height=None, out=None):
    """The (height, width) window of a height map held in host memory (CPU float32, 2-D,
    unit column stride; pinned for the copy to be asynchronous) as a contiguous CUDA
    tensor, copied on the current stream (``vs_map_upload``)."""
    require_cuda()
    if heights.is_cuda or heights.dtype != torch.float32 or heights.dim() != 2 or heights.stride(1) != 1:
        raise ValueError('heights must be a 2-D CPU float32 tensor with unit column stride')
    height = heights.shape[0] if height is None else int(height)
    width = heights.shape[1] if width is None else int(width)
    if height > heights.shape[0] or width > heights.shape[1]:
        raise ValueError('window larger than the map')
    if out is None:
        out = torch.empty((height, width), dtype=torch.float32, device='cuda')
    elif not (out.is_cuda and out.dtype == torch.float32 and out.shape == (height, width) and out.is_contiguous()):
        raise ValueError('out must be a contiguous (height, width) float32 CUDA tensor')
    _lib.call('vs_map_upload', heights.data_ptr(), heights.stride(0), width, height, out.data_ptr(), width,
              stream_handle())
    return out
