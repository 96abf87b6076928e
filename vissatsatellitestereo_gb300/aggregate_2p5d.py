"""Fusion of per-view DSMs, the inline block of ``run_fuse`` (aggregate_2p5d.py:65-81).

``fuse_dsms(all_dsm)`` takes the reference's stacked array ``all_dsm`` ((H, W, V)
float32, NaN = no measurement) and returns what the reference holds in
``all_dsm_mean_no_outliers`` after its median blur, bit-identical to the numpy
arithmetic.  Device tensors may also be given view-major ((V, H, W), layout='vhw').
"""
import numpy as np
import torch

from . import _lib
from ._dev import is_cuda_tensor, ptr, require_cuda, stream_handle, workspace

LAYOUTS = {'hwv': _lib.VS_LAYOUT_HWV, 'vhw': _lib.VS_LAYOUT_VHW}


def fuse_dsms(all_dsm, median_blur=True, layout='hwv', out=None):
    require_cuda()
    on_device = is_cuda_tensor(all_dsm)
    src = all_dsm if on_device else torch.from_numpy(np.ascontiguousarray(all_dsm, dtype=np.float32)).cuda()
    src = src.to(torch.float32).contiguous()
    if layout not in LAYOUTS:
        raise ValueError(f'layout must be one of {sorted(LAYOUTS)}')
    if layout == 'hwv':
        h, w, v = src.shape
    else:
        v, h, w = src.shape
    if out is None:
        out = torch.empty((h, w), dtype=torch.float32, device=src.device)
    wp, wb = workspace(_lib.lib().vs_fuse_dsms_workspace_size(h, w))
    _lib.call('vs_fuse_dsms', ptr(src), LAYOUTS[layout], v, h, w, ptr(out), int(bool(median_blur)), wp, wb,
              stream_handle())
    return out if on_device else out.cpu().numpy()
