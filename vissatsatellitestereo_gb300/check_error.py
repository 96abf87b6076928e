"""Drop-in ``check_perspective_error`` (lib/check_error.py:37-121) on the GPU: mean,
median and max pixel reprojection error and metric inverse-projection error of a
perspective camera K[R|t] over the kept points."""
import numpy as np
import torch

from . import _lib
from ._dev import as_device, ptr, require_cuda, stream_handle, workspace


def perspective_error_batch(xx, yy, zz, col, row, K, R, t, keep_mask=None, shared_points=True):
    """(V, 6) float64 device tensor of error statistics for V views."""
    require_cuda()
    c = as_device(col, torch.float64)
    r = as_device(row, torch.float64)
    V = c.shape[0] if c.dim() > 1 else 1
    n = c.shape[-1]
    x, y, z = (as_device(a, torch.float64) for a in (xx, yy, zz))
    keep = None if keep_mask is None else as_device(keep_mask, torch.uint8)
    Kd, Rd, td = (as_device(a, torch.float64) for a in (K, R, t))
    err = torch.empty((V, _lib.VS_ERROR_STATS), dtype=torch.float64, device='cuda')
    wp, wb = workspace(_lib.lib().vs_perspective_error_workspace_size(V, n))
    _lib.call('vs_perspective_error', ptr(x), ptr(y), ptr(z), 0 if shared_points else n, ptr(c), ptr(r), ptr(keep),
              V, n, ptr(Kd), ptr(Rd), ptr(td), ptr(err), wp, wb, stream_handle())
    return err


def check_perspective_error(xx, yy, zz, col, row, r, q, t, keep_mask):
    flat = lambda a: np.asarray(a, dtype=np.float64).reshape(-1)
    keep = None if keep_mask is None else np.asarray(keep_mask).reshape(1, -1)
    err = perspective_error_batch(flat(xx), flat(yy), flat(zz), flat(col).reshape(1, -1), flat(row).reshape(1, -1),
                                  np.asarray(r, dtype=np.float64).reshape(1, 3, 3),
                                  np.asarray(q, dtype=np.float64).reshape(1, 3, 3),
                                  np.asarray(t, dtype=np.float64).reshape(1, 3, 1), keep)
    return tuple(float(v) for v in err[0].cpu().numpy())
