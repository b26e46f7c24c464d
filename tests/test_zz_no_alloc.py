"""ff_scan_counts_noalloc: the ray-count scan for callers that cannot allocate device memory
(for example a host engine that owns every device buffer and hands the library only inputs
and outputs, or code that must not touch the device allocator). It keeps its partial sums in a
fixed scratch array inside the library instead of a caller workspace.

Checked through the C ABI against ff_scan_counts (the workspace variant) on two calls in a
row — the second call must not see the first call's leftovers in the shared scratch — and
at the size limit. The comparison is exact: offsets are integers. This file is collected
last so that a run stopping at the first failure has already run every other test."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _lib():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from factor_fields_gb300 import build
    from factor_fields_gb300 import _native as N
    build.build()
    return N.load()


def _scan_with_workspace(lib, counts, stream):
    n = counts.numel()
    out = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    wsb = lib.ff_scan_workspace_bytes(n)
    ws = torch.empty(max(wsb, 8), dtype=torch.uint8, device="cuda")
    rc = lib.ff_scan_counts(ctypes.c_void_p(counts.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                            ctypes.c_void_p(ws.data_ptr()), wsb, stream)
    assert rc == 0, lib.ff_last_error()
    return out


def _scan_no_alloc(lib, counts, stream):
    n = counts.numel()
    out = torch.full((n + 1,), -1, dtype=torch.int64, device="cuda")
    rc = lib.ff_scan_counts_noalloc(ctypes.c_void_p(counts.data_ptr()), n, ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == 0, lib.ff_last_error()
    return out


def test_no_alloc_scan_matches_workspace_scan_twice():
    lib = _lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    g = torch.Generator(device="cuda").manual_seed(0)
    # two different calls in a row: a large multi-block scan, then a smaller one
    for n, hi in ((1_000_003, 1025), (70_001, 7)):
        counts = torch.randint(0, hi, (n,), dtype=torch.int32, device="cuda", generator=g)
        ref = _scan_with_workspace(lib, counts, stream)
        got = _scan_no_alloc(lib, counts, stream)
        torch.cuda.synchronize()
        assert torch.equal(got, ref), n


def test_no_alloc_scan_leaves_device_memory_unchanged():
    """After a first call on the device (which may load the library's module and with it the
    scratch array), a call changes neither the free device memory nor torch's allocations."""
    lib = _lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = 300_001
    counts = torch.randint(0, 50, (n,), dtype=torch.int32, device="cuda")
    out = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    assert lib.ff_scan_counts_noalloc(ctypes.c_void_p(counts.data_ptr()), n, ctypes.c_void_p(out.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    counts.random_(0, 50)
    assert lib.ff_scan_counts_noalloc(ctypes.c_void_p(counts.data_ptr()), n, ctypes.c_void_p(out.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == alloc0
    ref = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    ref[1:] = torch.cumsum(counts.long(), 0)
    assert torch.equal(out, ref)


def test_no_alloc_scan_limits():
    lib = _lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    cap = lib.ff_scan_noalloc_max_counts()
    assert cap == 16_777_216
    # exactly at the limit: still served, and equal to the workspace scan
    counts = torch.ones(cap, dtype=torch.int32, device="cuda")
    assert torch.equal(_scan_no_alloc(lib, counts, stream), _scan_with_workspace(lib, counts, stream))
    # one past the limit: a clear error, nothing launched
    over = torch.ones(cap + 1, dtype=torch.int32, device="cuda")
    out = torch.empty(cap + 2, dtype=torch.int64, device="cuda")
    rc = lib.ff_scan_counts_noalloc(ctypes.c_void_p(over.data_ptr()), cap + 1, ctypes.c_void_p(out.data_ptr()),
                                    stream)
    assert rc == -5 and b"fixed scratch" in lib.ff_last_error()
    # the empty scan
    empty = torch.empty(0, dtype=torch.int32, device="cuda")
    assert torch.equal(_scan_no_alloc(lib, empty, stream).cpu(), torch.zeros(1, dtype=torch.int64))
