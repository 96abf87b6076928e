"""Drop-in ``solve_perspective`` (lib/solve_perspective.py:82-126) on the GPU.

Same signature, same results to rounding: (K, R, t) with K upper triangular, positive
diagonal, K[2,2] = 1, det R = +1, as the reference's ``factorize`` (:38-79) leaves them.
Raises AssertionError where the reference's assertions would fire (size mismatch,
failed factorisation check).  The batched form fits many views in one launch.
"""
import numpy as np
import torch

from . import _lib
from ._dev import as_device, ptr, require_cuda, stream_handle, workspace


def _flat(a):
    return a.reshape(-1) if isinstance(a, torch.Tensor) else np.asarray(a, dtype=np.float64).reshape(-1)


def solve_perspective_batch(xx, yy, zz, col, row, keep_mask=None, shared_points=True):
    """Fit V cameras.  xx/yy/zz: (N,) shared points (shared_points=True) or (V, N);
    col/row: (V, N); keep_mask: (V, N) bool or None.  Returns device tensors
    K (V,3,3), R (V,3,3), t (V,3,1), status (V,) int32."""
    require_cuda()
    c = as_device(col, torch.float64)
    r = as_device(row, torch.float64)
    V = c.shape[0] if c.dim() > 1 else 1
    n = c.shape[-1]
    x, y, z = (as_device(a, torch.float64) for a in (xx, yy, zz))
    stride = 0 if shared_points else n
    keep = None if keep_mask is None else as_device(keep_mask, torch.uint8)
    K = torch.empty((V, 3, 3), dtype=torch.float64, device='cuda')
    R = torch.empty((V, 3, 3), dtype=torch.float64, device='cuda')
    t = torch.empty((V, 3, 1), dtype=torch.float64, device='cuda')
    status = torch.empty((V,), dtype=torch.int32, device='cuda')
    need = _lib.lib().vs_dlt_fit_workspace_size(V, n)
    wp, wb = workspace(need)
    _lib.call('vs_dlt_fit', ptr(x), ptr(y), ptr(z), stride, ptr(c), ptr(r), ptr(keep), V, n, ptr(K), ptr(R), ptr(t),
              ptr(status), wp, wb, stream_handle())
    return K, R, t, status


def solve_perspective(xx, yy, zz, col, row, keep_mask=None):
    sizes = [np.size(a) if not isinstance(a, torch.Tensor) else a.numel() for a in (xx, yy, zz, col, row)]
    assert all(s == sizes[0] for s in sizes)
    keep = None if keep_mask is None else _flat(keep_mask).reshape(1, -1)
    K, R, t, status = solve_perspective_batch(_flat(xx), _flat(yy), _flat(zz), _flat(col).reshape(1, -1),
                                              _flat(row).reshape(1, -1), keep)
    st = int(status[0].item())
    assert st == _lib.VS_OK, f'perspective factorisation failed (status {st})'
    return K[0].cpu().numpy(), R[0].cpu().numpy(), t[0].cpu().numpy()
