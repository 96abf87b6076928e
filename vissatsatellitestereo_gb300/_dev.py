"""Device plumbing for the drop-in wrappers: torch owns device memory and streams."""
import numpy as np
import torch

from ._lib import VsError  # noqa: F401  (re-exported for callers)


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError('vissat-gb300 runs on a CUDA GPU (sm_103a); none is visible')


def stream_handle():
    return torch.cuda.current_stream().cuda_stream


def is_cuda_tensor(a):
    return isinstance(a, torch.Tensor) and a.is_cuda


def as_device(a, dtype):
    """A contiguous CUDA tensor of `dtype` holding `a` (numpy array, scalar or tensor)."""
    if isinstance(a, torch.Tensor):
        t = a if a.is_cuda else a.cuda()
        return t.to(dtype).contiguous()
    arr = np.ascontiguousarray(np.asarray(a), dtype=torch.empty((), dtype=dtype).numpy().dtype)
    return torch.from_numpy(arr).cuda(non_blocking=False)


def ptr(t):
    return None if t is None else t.data_ptr()


class Workspace:
    """Grow-only scratch buffer per device and stream (the library never allocates; calls
    on different streams may run concurrently, so they never share scratch)."""
    _bufs = {}

    @classmethod
    def get(cls, nbytes):
        dev = torch.cuda.current_device()
        key = (dev, torch.cuda.current_stream().cuda_stream)
        buf = cls._bufs.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=f'cuda:{dev}')
            cls._bufs[key] = buf
        return buf


def workspace(nbytes):
    buf = Workspace.get(nbytes)
    return buf.data_ptr(), buf.numel()
