"""Drop-in ``RPCModel`` (lib/rpc_model.py:131-168) backed by the sm_103a projection kernel.

``RPCModel(meta_dict).projection(lat, lon, alt) -> (col, row)`` keeps the reference's
signature and semantics: arrays of any broadcastable shape, float64 results of the
broadcast shape, NaN propagated, nothing raised for out-of-image points.  numpy inputs
are copied to the GPU and back; CUDA tensors stay on the device (results are tensors).

``mode='exact'`` (default) evaluates in FP64 in the reference's operation order and is
bit-identical to it; ``mode='fast'`` uses the compensated FP32 form (< 1e-4 px).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._dev import as_device, is_cuda_tensor, ptr, require_cuda, stream_handle, workspace

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

    def inverse_projection(self, col, row, alt, return_normalized=False):
        """(lon, lat, alt) of image points at the given altitudes (lib/rpc_model.py:170-249),
        bit-identical to the reference on 1-D inputs.  Arrays of one shape (the reference
        needs 1-D; any shape works here, point by point).  With return_normalized the
        normalised (lon, lat, alt) come back."""
        require_cuda()
        on_device = any(is_cuda_tensor(a) for a in (col, row, alt))
        shape = tuple(torch.as_tensor(col).shape) if not isinstance(col, torch.Tensor) else tuple(col.shape)
        c, r, a = (as_device(v, torch.float64).reshape(-1) for v in (col, row, alt))
        n = c.numel()
        lon = torch.empty(n, dtype=torch.float64, device='cuda')
        lat = torch.empty(n, dtype=torch.float64, device='cuda')
        alt_out = torch.empty(n, dtype=torch.float64, device='cuda')
        its = (ctypes.c_int32 * 1)()
        if n:
            wp, wb = workspace(_lib.lib().vs_rpc_inverse_project_workspace_size(1, n))
            _lib.call('vs_rpc_inverse_project', ptr(self._camera()), 1, ptr(c), ptr(r), ptr(a), n, 0,
                      int(bool(return_normalized)), ptr(lon), ptr(lat), ptr(alt_out), 1000, its, wp, wb,
                      stream_handle())
        self.last_iterations = int(its[0])
        outs = [t.reshape(shape) for t in (lon, lat, alt_out)]
        if not return_normalized and not on_device:
            outs[2] = alt
        if on_device:
            return tuple(outs)
        return tuple(o if isinstance(o, np.ndarray) or not isinstance(o, torch.Tensor) else o.cpu().numpy()
                     for o in outs)


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


CUBE_VARIANTS = {'fp32': _lib.VS_CUBE_FP32, 'bf16x3': _lib.VS_CUBE_BF16X3, 'tf32x3': _lib.VS_CUBE_TF32X3,
                 'bf16x6': _lib.VS_CUBE_BF16X6, 'bf16x3_tc': _lib.VS_CUBE_BF16X3_TC,
                 'bf16x3_lin': _lib.VS_CUBE_BF16X3_LIN, 'bf16x3_lin_tc': _lib.VS_CUBE_BF16X3_LIN_TC}
TC_VARIANTS = ('bf16x3_tc', 'bf16x3_lin_tc')


def project_cube(meta_dicts, xyz, variant='tf32x3', out=None, check=True):
    """Precision form of ``RPCModel.projection`` for C cameras over one point set already in
    the normalised frame (the monomial x coefficient contraction of lib/rpc_model.py:40-79,
    denormalised as in :164-168).

    xyz: (3, N) float32 (normalised latitude, longitude, altitude), numpy or CUDA tensor.
    Returns a CUDA float32 tensor (C, 2, N): col plane then row plane per camera.
    ``variant``: 'fp32' (CUDA cores), 'bf16x3', 'tf32x3', 'bf16x6' (tensor-core split forms),
    'bf16x3_tc' (BF16X3 on tcgen05), 'bf16x3_lin' (BF16X3 for the higher-order terms, the
    constant and linear terms in FP32), 'bf16x3_lin_tc' (the same with the contraction on
    tcgen05).
    ``out``: optional preallocated (C, 2, N) float32 CUDA tensor.
    ``check``: for the tcgen05 variants, read the kernel's device-side status back (synchronises the
    stream) and raise ``VsError`` (VS_ERR_TIMEOUT) if a CTA gave up waiting for the tensor
    cores; with ``check=False`` the caller reads it later with ``project_cube_status``.
    """
    require_cuda()
    if variant not in CUBE_VARIANTS:
        raise ValueError(f'variant must be one of {sorted(CUBE_VARIANTS)}')
    cams = meta_dicts if isinstance(meta_dicts, torch.Tensor) else torch.from_numpy(_lib.camera_array(meta_dicts))
    cams = cams.to(device='cuda', dtype=torch.float64).contiguous()
    C = cams.shape[0]
    pts = as_device(xyz, torch.float32)
    if pts.dim() != 2 or pts.shape[0] != 3:
        raise ValueError(f'xyz must have shape (3, N), got {tuple(pts.shape)}')
    n = pts.shape[1]
    if out is None:
        out = torch.empty((C, 2, n), dtype=torch.float32, device='cuda')
    elif out.shape != (C, 2, n) or out.dtype != torch.float32 or not out.is_cuda or not out.is_contiguous():
        raise ValueError('out must be a contiguous CUDA float32 tensor of shape (C, 2, N)')
    ws_bytes = _lib.lib().vs_rpc_project_cube_workspace_size(C)
    ws_ptr, ws_len = workspace(ws_bytes)
    _lib.call('vs_rpc_project_cube', ptr(cams), C, ptr(pts), n, ptr(out), CUBE_VARIANTS[variant], ws_ptr, ws_len,
              stream_handle())
    if check and variant in TC_VARIANTS and n > 0:
        project_cube_status(C, variant)
    return out


def project_cube_status(n_cams, variant):
    """Raise ``VsError`` if the last ``project_cube`` call of ``variant`` over ``n_cams``
    cameras on the current stream reported a device-side timeout (synchronises the stream)."""
    ws_ptr, _ = workspace(_lib.lib().vs_rpc_project_cube_workspace_size(n_cams))
    _lib.call('vs_rpc_project_cube_status', ws_ptr, n_cams, CUBE_VARIANTS[variant], stream_handle())


def inverse_project_cameras(meta_dicts, col, row, alt, shared=True, normalized=False, max_iter=1000):
    """Batched inverse projection: C cameras over one point set (shared, arrays of N) or one
    set per camera ((C, N) arrays).  Returns device tensors (lon, lat, alt) of shape (C, N)
    and the per-camera iteration counts."""
    require_cuda()
    cams = meta_dicts if isinstance(meta_dicts, torch.Tensor) else torch.from_numpy(_lib.camera_array(meta_dicts))
    cams = cams.to(device='cuda', dtype=torch.float64).contiguous()
    C = cams.shape[0]
    c, r, a = (as_device(v, torch.float64) for v in (col, row, alt))
    n = c.shape[-1]
    lon = torch.empty((C, n), dtype=torch.float64, device='cuda')
    lat = torch.empty((C, n), dtype=torch.float64, device='cuda')
    alt_out = torch.empty((C, n), dtype=torch.float64, device='cuda')
    its = (ctypes.c_int32 * C)()
    if n:
        wp, wb = workspace(_lib.lib().vs_rpc_inverse_project_workspace_size(C, n))
        _lib.call('vs_rpc_inverse_project', ptr(cams), C, ptr(c), ptr(r), ptr(a), n, 0 if shared else n,
                  int(bool(normalized)), ptr(lon), ptr(lat), ptr(alt_out), int(max_iter), its, wp, wb, stream_handle())
    return lon, lat, alt_out, [int(v) for v in its]
