"""Drop-in ``solve_affine`` (lib/solve_affine.py:37-72) and the batched affine camera
approximation of ``CameraApprox.approx_affine_latlonalt`` (camera_approx.py:112-137)."""
import numpy as np
import torch

from . import _lib
from ._dev import as_device, is_cuda_tensor, ptr, require_cuda, stream_handle, workspace


def solve_affine_batch(xx, yy, zz, col, row, keep_mask=None, shared_points=False):
    """P (V, 2, 4) and status (V,) for V views: col/row (V, N); xx/yy/zz (V, N), or (N,)
    with shared_points; keep_mask (V, N) or None.  Device tensors in, device tensors out."""
    require_cuda()
    c, r = as_device(col, torch.float64), as_device(row, torch.float64)
    V, n = c.shape
    x, y, z = (as_device(a, torch.float64) for a in (xx, yy, zz))
    k = None if keep_mask is None else as_device(keep_mask, torch.uint8)
    P = torch.empty((V, 2, 4), dtype=torch.float64, device='cuda')
    status = torch.empty((V,), dtype=torch.int32, device='cuda')
    wp, wb = workspace(_lib.lib().vs_affine_fit_workspace_size(V, n))
    _lib.call('vs_affine_fit', ptr(x), ptr(y), ptr(z), 0 if shared_points else n, ptr(c), ptr(r), ptr(k), V, n,
              ptr(P), ptr(status), wp, wb, stream_handle())
    return P, status


def solve_affine(xx, yy, zz, col, row, keep_mask=None):
    """The reference's signature: arrays of equal size, optional boolean keep mask; returns
    P as a (2, 4) float64 array.  Raises AssertionError on a size mismatch (as the
    reference) and ValueError when fewer than 4 points are kept or the system is singular."""
    sizes = [np.size(a) for a in (xx, yy, zz, col, row)]
    assert all(s == sizes[0] for s in sizes)
    on_device = any(is_cuda_tensor(a) for a in (xx, yy, zz, col, row))
    flat = [torch.as_tensor(a).reshape(1, -1) if isinstance(a, torch.Tensor) else np.asarray(a, np.float64).reshape(1, -1)
            for a in (xx, yy, zz, col, row)]
    k = None
    if keep_mask is not None:
        k = keep_mask.reshape(1, -1) if isinstance(keep_mask, torch.Tensor) else np.asarray(keep_mask).reshape(1, -1)
    P, status = solve_affine_batch(*flat, keep_mask=k)
    if int(status[0].item()) != 0:
        raise ValueError('solve_affine: fewer than 4 kept points or a singular system')
    return P[0] if on_device else P[0].cpu().numpy()


def approx_affine_latlonalt(meta_dicts, lat, lon, alt, shared_points=True):
    """Per-view [width, height, P (8)] (V, 10) and status (V,) as device tensors: each RPC
    camera projects the lat/lon/alt grid ((N,) shared or (V, N)), keeps the in-image points
    and fits the affine camera in (lat, lon, alt)."""
    require_cuda()
    cams = meta_dicts if isinstance(meta_dicts, torch.Tensor) else torch.from_numpy(_lib.camera_array(meta_dicts))
    cams = cams.to(device='cuda', dtype=torch.float64).contiguous()
    V = cams.shape[0]
    la, lo, al = (as_device(a, torch.float64) for a in (lat, lon, alt))
    n = la.shape[-1]
    params = torch.empty((V, 10), dtype=torch.float64, device='cuda')
    status = torch.empty((V,), dtype=torch.int32, device='cuda')
    wp, wb = workspace(_lib.lib().vs_camera_approx_affine_workspace_size(V, n))
    _lib.call('vs_camera_approx_affine', ptr(cams), V, ptr(la), ptr(lo), ptr(al), n, 0 if shared_points else n,
              ptr(params), ptr(status), wp, wb, stream_handle())
    return params, status
