"""GPU: the allocation-free prefix sum (dv_exclusive_scan_static), called
through the C ABI, gives exactly the offsets of the allocating entry point
(dv_exclusive_scan) on two calls in a row.

It exists for callers that cannot allocate device memory themselves (an
embedding application whose allocator owns the GPU, a frame loop with a fixed
budget, work recorded into a CUDA graph): its scratch is a fixed 32 KiB array
inside the library, so it takes only inputs and outputs.  This file is
collected last so that a run stopping at the first failure has already run
every other test."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def allocating_scan(lib, counts):
    n = counts.numel()
    out = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    scratch = torch.empty(max(int(lib.dv_scan_scratch_bytes(n)), 8), dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    assert lib.dv_exclusive_scan(ctypes.c_void_p(counts.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                                 ctypes.c_void_p(scratch.data_ptr()), ctypes.c_void_p(st)) == 0
    return out


def static_scan(lib, counts):
    n = counts.numel()
    out = torch.full((n + 1,), -7, dtype=torch.int64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.dv_exclusive_scan_static(ctypes.c_void_p(counts.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                                      ctypes.c_void_p(st))
    assert rc == 0, rc
    return out


def test_static_scan_matches_allocating_scan_on_two_calls():
    from diver_gb300 import _native

    lib = _native.lib()
    g = torch.Generator(device="cuda").manual_seed(5)
    # a multi-tile call, then a smaller one that reuses the shared array
    first = torch.randint(0, 700, (3_000_001,), dtype=torch.int32, device="cuda", generator=g)
    second = torch.randint(0, 50, (4_097,), dtype=torch.int32, device="cuda", generator=g)
    a = static_scan(lib, first)
    b = static_scan(lib, second)
    torch.cuda.synchronize()
    assert torch.equal(a, allocating_scan(lib, first))
    assert torch.equal(b, allocating_scan(lib, second))


def test_static_scan_at_its_limit_and_when_empty():
    """n equal to the limit fills all 4096 tiles of the array; n = 0 writes
    only offsets[0] = 0."""
    from diver_gb300 import _native

    lib = _native.lib()
    limit = int(lib.dv_exclusive_scan_static_max())
    g = torch.Generator(device="cuda").manual_seed(9)
    full = torch.randint(0, 300, (limit,), dtype=torch.int32, device="cuda", generator=g)
    a = static_scan(lib, full)
    torch.cuda.synchronize()
    assert torch.equal(a, allocating_scan(lib, full))
    empty = torch.zeros(0, dtype=torch.int32, device="cuda")
    z = static_scan(lib, empty)
    torch.cuda.synchronize()
    assert z.tolist() == [0]


def test_static_scan_rejects_oversized_input():
    from diver_gb300 import _native

    lib = _native.lib()
    limit = int(lib.dv_exclusive_scan_static_max())
    assert limit == 4096 * 2048
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    # the size check comes before any launch or pointer use
    rc = lib.dv_exclusive_scan_static(ctypes.c_void_p(out.data_ptr()), limit + 1, ctypes.c_void_p(out.data_ptr()),
                                      None)
    assert rc == 5  # DV_ERR_OVERFLOW
