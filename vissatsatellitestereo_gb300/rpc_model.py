"""Drop-in ``RPCModel`` (lib/rpc_model.py:131-168) backed by the sm_103a projection kernel.

``RPCModel(meta_dict).projection(lat, lon, alt) -> (col, row)`` keeps the reference's
signature and semantics: arrays of any broadcastable shape, float64 results of the
broadcast shape, NaN propagated, nothing raised for out-of-image points.  numpy inputs
are copied to the GPU and back; CUDA tensors stay on the device (results are tensors).

``mode='exact'`` (default) evaluates in FP64 in the reference's operation order and is
bit-identical to it; ``mode='fast'`` uses the compensated FP32 form (< 1e-4 px).
"""
import numpy as np
import torch

from . import _lib
from ._dev import as_device, is_cuda_tensor, ptr, require_cuda, stream_handle

MODES = {'exact': _lib.VS_PROJ_EXACT, 'fast': _lib.VS_PROJ_FAST}


class RPCModel(object):
    def __init__(self, meta_dict, mode='exact'):
        rpc = meta_dict['rpc']
        self.rowOff, self.rowScale = rpc['rowOff'], rpc['rowScale']
        self.colOff, self.colScale = rpc['colOff'], rpc['colScale']
        self.latOff, self.latScale = rpc['latOff'], rpc['latScale']
        self.lonOff, self.lonScale = rpc['lonOff'], rpc['lonScale']
        self.altOff, self.altScale = rpc['altOff'], rpc['altScale']
        self.rowNum, self.rowDen = rpc['rowNum'], rpc['rowDen']
        self.colNum, self.colDen = rpc['colNum'], rpc['colDen']
        self.width = meta_dict['width']
        self.height = meta_dict['height']
        if mode not in MODES:
            raise ValueError(f'mode must be one of {sorted(MODES)}')
        self.mode = mode
        self._host = _lib.camera_array([meta_dict])
        self._dev = {}

    def _camera(self):
        dev = torch.cuda.current_device()
        if dev not in self._dev:
            self._dev[dev] = torch.from_numpy(self._host).cuda()
        return self._dev[dev]

    def projection(self, lat, lon, alt):
        require_cuda()
        on_device = any(is_cuda_tensor(a) for a in (lat, lon, alt))
        if on_device:
            shape = torch.broadcast_shapes(*(torch.as_tensor(a).shape if not isinstance(a, torch.Tensor) else a.shape
                                             for a in (lat, lon, alt)))
            la, lo, al = (torch.as_tensor(a, dtype=torch.float64, device='cuda').expand(shape).contiguous()
                          for a in (lat, lon, alt))
        else:
            la_np, lo_np, al_np = np.broadcast_arrays(np.asarray(lat, dtype=np.float64),
                                                      np.asarray(lon, dtype=np.float64),
                                                      np.asarray(alt, dtype=np.float64))
            shape = la_np.shape
            la, lo, al = (as_device(a, torch.float64) for a in (la_np, lo_np, al_np))
        n = la.numel()
        col = torch.empty(shape, dtype=torch.float64, device=la.device)
        row = torch.empty(shape, dtype=torch.float64, device=la.device)
        if n:
            _lib.call('vs_rpc_project', ptr(self._camera()), 1, ptr(la), ptr(lo), ptr(al), n, 0, ptr(col), ptr(row),
                      None, MODES[self.mode], stream_handle())
        if on_device:
            return col, row
        return col.cpu().numpy(), row.cpu().numpy()


def project_cameras(meta_dicts, lat, lon, alt, mode='fast', shared=True, keep=False):
    """Batched projection: C cameras over one shared point set (shared=True, arrays of N)
    or one point set per camera (arrays of C x N).  Device tensors in, device tensors out:
    (col, row[, keep]) of shape (C, N)."""
    require_cuda()
    cams = torch.from_numpy(_lib.camera_array(meta_dicts)).cuda()
    C = cams.shape[0]
    la, lo, al = (as_device(a, torch.float64) for a in (lat, lon, alt))
    n = la.shape[-1]
    stride = 0 if shared else n
    col = torch.empty((C, n), dtype=torch.float64, device='cuda')
    row = torch.empty((C, n), dtype=torch.float64, device='cuda')
    kp = torch.empty((C, n), dtype=torch.uint8, device='cuda') if keep else None
    if n:
        _lib.call('vs_rpc_project', ptr(cams), C, ptr(la), ptr(lo), ptr(al), n, stride, ptr(col), ptr(row), ptr(kp),
                  MODES[mode], stream_handle())
    return (col, row, kp) if keep else (col, row)
