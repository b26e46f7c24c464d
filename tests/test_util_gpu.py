"""GPU checks of the library's utility entry points (ff_zero_f32)."""
import ctypes

import pytest
import torch

from gpu_util import need_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu():
    need_gpu()


def test_zero_f32_many_buffers_unaligned_and_tails():
    """11 buffers (two launches of at most 8), views starting off a 16-byte boundary, sizes that
    are not multiples of 4, an empty buffer; the memory around each view stays untouched."""
    from factor_fields_gb300 import _native as N
    base = torch.full((1 << 16,), 7.0, device="cuda")
    spans = [(0, 1), (1, 5), (7, 1000), (1003, 3), (2000, 4096), (6101, 0), (6200, 17), (7001, 33),
             (9000, 20000), (29003, 1), (30001, 30000)]
    views = [base[o:o + n] for o, n in spans]
    ptrs = (ctypes.c_void_p * len(views))(*[v.data_ptr() for v in views])
    counts = (ctypes.c_int64 * len(views))(*[v.numel() for v in views])
    N.call("ff_zero_f32", ptrs, counts, len(views), N.stream_ptr(), kernels=2)
    torch.cuda.synchronize()
    want = torch.full_like(base, 7.0)
    for o, n in spans:
        want[o:o + n] = 0.0
    assert torch.equal(base, want)
    with pytest.raises(N.NativeError):
        N.call("ff_zero_f32", ptrs, counts, -1, N.stream_ptr())
