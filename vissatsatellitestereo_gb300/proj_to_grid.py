"""Drop-in ``proj_to_grid`` (lib/proj_to_grid.py:41-81) on the GPU, bit-identical to the
reference: FP64 binning, per-cell nanmax, non-propagating 3x3 median hole fill."""
import numpy as np
import torch

from . import _lib
from ._dev import as_device, is_cuda_tensor, ptr, require_cuda, stream_handle, workspace


def proj_to_grid(points, xoff, yoff, xresolution, yresolution, xsize, ysize, propagate=False):
    """(ysize, xsize) float64 DSM; `propagate` is accepted and ignored, as in the reference."""
    require_cuda()
    on_device = is_cuda_tensor(points)
    pts = as_device(points, torch.float64)
    if pts.dim() != 2 or pts.shape[1] < 3:
        raise ValueError('points must be (N, 3)')
    if pts.shape[1] != 3:
        pts = pts[:, :3].contiguous()
    xsize, ysize = int(xsize), int(ysize)
    dsm = torch.empty((ysize, xsize), dtype=torch.float64, device=pts.device)
    wp, wb = workspace(_lib.lib().vs_proj_to_grid_workspace_size(xsize, ysize))
    _lib.call('vs_proj_to_grid', ptr(pts), pts.shape[0], float(xoff), float(yoff), float(xresolution),
              float(yresolution), xsize, ysize, ptr(dsm), wp, wb, stream_handle())
    return dsm if on_device else dsm.cpu().numpy()


def median_blur3x3(img):
    """cv2.medianBlur(img.astype(np.float32), 3) with replicated borders (NaN sorts last).
    img: (H, W) or (B, H, W), numpy or CUDA tensor, float32 or float64."""
    require_cuda()
    on_device = is_cuda_tensor(img)
    src = img if on_device else torch.from_numpy(np.ascontiguousarray(img)).cuda()
    src = src.contiguous()
    if src.dtype not in (torch.float32, torch.float64):
        src = src.to(torch.float64)
    shape = src.shape
    h, w = shape[-2], shape[-1]
    b = int(np.prod(shape[:-2])) if len(shape) > 2 else 1
    out = torch.empty(shape, dtype=torch.float32, device=src.device)
    fn = 'vs_median_blur3x3_f32' if src.dtype == torch.float32 else 'vs_median_blur3x3_f64'
    _lib.call(fn, ptr(src), ptr(out), h, w, b, stream_handle())
    return out if on_device else out.cpu().numpy()
