"""compareCompositionVectorsStatic: pair compare for callers that cannot
allocate device memory.

Such a caller might be a runtime that handed all device memory to fixed cache
slots when it started, or one whose device memory is owned by another
framework's allocator; either way it has no scratch buffer to pass.  The entry
point runs the same kernels as compareCompositionVectors on an array built into
the library.  These tests call both entry points through the C ABI on the same
inputs, twice in a row (the second call must not see the first call's leftover
scratch contents), and check that oversized inputs are refused.

This file is named to be collected last.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rocket_gb300 import _native

pytestmark = pytest.mark.gpu

STATIC_MAX_ENTRIES = 1 << 26


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _compare_both(L, lk, lv, rk, rv):
    st = torch.cuda.current_stream().cuda_stream
    dlk, dlv, drk, drv = _dev(lk), _dev(lv), _dev(rk), _dev(rv)
    out_ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    out_static = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    scratch = torch.empty(L.estimateScratchMemory(b"DNA", 3, max(len(lk), len(rk), 1)),
                          dtype=torch.uint8, device="cuda")
    _native.check(L.compareCompositionVectors(
        st, scratch.data_ptr(), scratch.numel(), dlk.data_ptr(), dlv.data_ptr(), len(lk),
        drk.data_ptr(), drv.data_ptr(), len(rk), out_ref.data_ptr()))
    _native.check(L.compareCompositionVectorsStatic(
        st, dlk.data_ptr(), dlv.data_ptr(), len(lk), drk.data_ptr(), drv.data_ptr(), len(rk),
        out_static.data_ptr()))
    return float(out_ref.item()), float(out_static.item())


def test_static_scratch_matches_caller_scratch_on_consecutive_calls():
    L = _native.load()
    cases = [O.bindings_compare_case(1, 100000, 0.5), O.bindings_compare_case(2, 30000, 1.0)]
    for lk, lv, rk, rv, _ in cases:  # two calls in a row
        ref, static = _compare_both(L, lk, lv, rk, rv)
        assert abs(ref - static) <= 1e-12 * max(1.0, abs(ref))
        exact = O.compare_fp64(lk.view(np.uint32), lv, rk.view(np.uint32), rv)
        assert abs(static - exact) <= 1e-12 * max(1.0, abs(exact))


def test_static_scratch_refuses_inputs_over_the_limit():
    L = _native.load()
    st = torch.cuda.current_stream().cuda_stream
    # refused on the host before any kernel runs, so no buffers are needed
    half = STATIC_MAX_ENTRIES // 2
    rc = L.compareCompositionVectorsStatic(st, 0, 0, half, 0, 0, half + 1, 0)
    assert rc == 1  # cudaErrorInvalidValue
