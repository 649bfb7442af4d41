"""The allocation-free exclusive scan, called through the C ABI.

abx_exclusive_scan_i32_noalloc serves callers that must not allocate device
memory (code running under a memory budget that another allocator owns, or
latency-critical loops that must avoid cudaMalloc/cudaFree and their
synchronisation); its scratch is a static array in the library's device
memory.  It must give exactly the offsets of abx_exclusive_scan_i32, also on
a second call that finds the scratch still holding the first call's sums.
This file is collected last so that a failure here never hides another test.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_noalloc_scan_matches_allocating_scan_on_consecutive_calls(ax):
    L = ax._lib.load()
    rng = np.random.default_rng(2718)
    # the first call fills most of the static scratch, the second (smaller)
    # call must not see any of it; the third uses the maximum size
    for n in (5_000_003, 1234, ax._lib.NOALLOC_SCAN_MAX_N):
        x = torch.from_numpy(rng.integers(0, 100, size=n).astype(np.int32)).cuda()
        want = torch.empty(n + 1, dtype=torch.int32, device="cuda")
        got = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
        ax._lib.check(L.abx_exclusive_scan_i32(_stream(), _p(x), n, _p(want)))
        ax._lib.check(L.abx_exclusive_scan_i32_noalloc(_stream(), _p(x), n, _p(got)))
        torch.cuda.synchronize()
        assert torch.equal(got, want), n
        assert int(got[-1]) == int(x.sum())


def test_noalloc_scan_in_place_twice(ax):
    L = ax._lib.load()
    x = torch.arange(100_000, dtype=torch.int32, device="cuda") % 13
    want = torch.empty(x.numel() + 1, dtype=torch.int32, device="cuda")
    ax._lib.check(L.abx_exclusive_scan_i32(_stream(), _p(x), x.numel(), _p(want)))
    for _ in range(2):
        buf = torch.empty(x.numel() + 1, dtype=torch.int32, device="cuda")
        buf[:-1] = x
        ax._lib.check(L.abx_exclusive_scan_i32_noalloc(_stream(), _p(buf), x.numel(), _p(buf)))
        torch.cuda.synchronize()
        assert torch.equal(buf, want)


def test_noalloc_scan_rejects_sizes_above_its_maximum(ax):
    L = ax._lib.load()
    n = ax._lib.NOALLOC_SCAN_MAX_N + 1
    x = torch.zeros(n, dtype=torch.int32, device="cuda")
    out = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    status = L.abx_exclusive_scan_i32_noalloc(_stream(), _p(x), n, _p(out))
    assert status == ax._lib.ERROR_INVALID_ARGUMENT
    assert b"exceeds the maximum" in L.abx_last_error()
    torch.cuda.synchronize()
    assert int(out.abs().sum()) == 0  # nothing was launched
