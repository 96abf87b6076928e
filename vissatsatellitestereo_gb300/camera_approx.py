"""Batched ``CameraApprox.approx_perspective_enu`` (camera_approx.py:150-204).

The reference loops over views: project the lat/lon/alt grid with the view's RPC, keep
the in-image points, fit a perspective camera, convert R to a quaternion and measure the
fit error.  Here all views run in one call of the fused device pipeline.
"""
import numpy as np
import torch

from . import _lib
from ._dev import as_device, ptr, require_cuda, stream_handle, workspace
from .rpc_model import MODES


def approx_perspective_enu(meta_dicts, lat, lon, alt, xx, yy, zz, mode='fast', with_errors=True, shared_points=True):
    """Per-view camera parameters [w, h, fx, fy, cx, cy, s, qw, qx, qy, qz, tx, ty, tz]
    (V, 14), error statistics (V, 6) (or None) and status (V,) as device tensors.

    lat/lon/alt/xx/yy/zz: (N,) shared by all views (the reference's grid) or (V, N).
    ``meta_dicts`` may also be the (V, 92) float64 CUDA camera tensor of
    ``_lib.camera_array`` (no host-to-device copy per call)."""
    require_cuda()
    if isinstance(meta_dicts, torch.Tensor):
        cams = meta_dicts.to(device='cuda', dtype=torch.float64).contiguous()
    else:
        cams = torch.from_numpy(_lib.camera_array(meta_dicts)).cuda()
    V = cams.shape[0]
    la, lo, al, x, y, z = (as_device(a, torch.float64) for a in (lat, lon, alt, xx, yy, zz))
    n = la.shape[-1]
    stride = 0 if shared_points else n
    params = torch.empty((V, _lib.VS_CAMERA_PARAMS), dtype=torch.float64, device='cuda')
    err = torch.empty((V, _lib.VS_ERROR_STATS), dtype=torch.float64, device='cuda') if with_errors else None
    status = torch.empty((V,), dtype=torch.int32, device='cuda')
    wp, wb = workspace(_lib.lib().vs_camera_approx_workspace_size(V, n))
    _lib.call('vs_camera_approx_perspective', ptr(cams), V, ptr(la), ptr(lo), ptr(al), ptr(x), ptr(y), ptr(z), n,
              stride, MODES[mode], ptr(params), ptr(err), ptr(status), wp, wb, stream_handle())
    return params, err, status


def params_to_krt(params):
    """K, R, t (numpy) from one camera parameter vector."""
    p = np.asarray(params, dtype=np.float64)
    fx, fy, cx, cy, s = p[2:7]
    qw, qx, qy, qz = p[7:11]
    K = np.array([[fx, s, cx], [0, fy, cy], [0, 0, 1.0]])
    R = np.array([[1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)],
                  [2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)],
                  [2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)]])
    return K, R, p[11:14].reshape(3, 1)
