"""vs_fuse_dsms_static: the fusion for callers that cannot allocate device memory.

Callers such as a stream-ordered pipeline that forbids allocation after start-up, or a
foreign host without a device allocator, get the same fusion without passing a workspace:
the blur's intermediate grid lives in a library-owned static device array.  This checks,
through the C ABI, that two calls in a row give exactly what vs_fuse_dsms with a caller
workspace gives (fusion is bit-exact), and that grids beyond the array are refused.  The
file is collected last so that a failure here comes after every other test has run.
"""
import numpy as np
import pytest
import torch

from conftest import same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def lib():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from vissatsatellitestereo_gb300.build import build
    build()
    from vissatsatellitestereo_gb300 import _lib
    return _lib


def _stack(seed, h, w, v):
    rng = np.random.default_rng(seed)
    a = rng.normal(30, 10, (v, h, w)).astype(np.float32)
    a[rng.random(a.shape) < 0.3] = np.nan
    return torch.tensor(a, device='cuda')


def test_static_fusion_matches_workspace_fusion(lib):
    L = lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    h, w, v = 300, 257, 13
    for call, seed in enumerate((1, 2)):          # two calls in a row, different inputs
        dsm = _stack(seed, h, w, v)
        ref = torch.empty((h, w), dtype=torch.float32, device='cuda')
        got = torch.full((h, w), -1.0, dtype=torch.float32, device='cuda')
        ws_bytes = L.vs_fuse_dsms_workspace_size(h, w)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device='cuda')
        st = L.vs_fuse_dsms(dsm.data_ptr(), lib.VS_LAYOUT_VHW, v, h, w, ref.data_ptr(), 1, ws.data_ptr(), ws_bytes,
                            stream)
        assert st == lib.VS_OK, L.vs_last_error()
        st = L.vs_fuse_dsms_static(dsm.data_ptr(), lib.VS_LAYOUT_VHW, v, h, w, got.data_ptr(), 1, stream)
        assert st == lib.VS_OK, L.vs_last_error()
        torch.cuda.synchronize()
        assert same_bits(got.cpu().numpy(), ref.cpu().numpy()), f'call {call}'


@pytest.mark.parametrize('h,w', [
    (2049, 2048),                                   # one row more than the 2048 x 2048 cells it holds
    (1 << 32, 1 << 32),                             # h * w wraps to 0 in 64-bit arithmetic
    (4, (1 << 62) + 1),                             # h * w wraps to 4 cells
])
def test_static_fusion_rejects_grids_beyond_its_array(lib, h, w):
    L = lib.lib()
    assert h * w > lib.VS_FUSE_STATIC_MAX_CELLS
    # real (small) device buffers: if the size check ever regressed, a launch would still
    # touch only memory this process owns rather than a wild address
    dsm = torch.zeros(3 * 16, dtype=torch.float32, device='cuda')
    out = torch.zeros(16, dtype=torch.float32, device='cuda')
    st = L.vs_fuse_dsms_static(dsm.data_ptr(), lib.VS_LAYOUT_VHW, 3, h, w, out.data_ptr(), 1, None)
    torch.cuda.synchronize()
    assert st == lib.VS_ERR_ARG
    assert b'exceeds the static scratch' in L.vs_last_error()
    assert torch.count_nonzero(out).item() == 0
