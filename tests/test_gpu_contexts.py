"""The drop-in entry points in contexts the caller creates and destroys.

Rocket creates its own CUDA context per device worker (cuCtxCreate,
CudaContext.java:45) and destroys it again (:124); BindingsTest does so once per
test.  State the library looks up once -- the built-in scratch array's device
address, the compare kernel's shared-memory limit -- belongs to one context, so
two contexts created and destroyed one after the other must each work.  Buffers
are allocated with the driver API inside each context, as JCuda does; the
context is current on the calling thread, as CudaContext.with makes it.

Also: the compare kernels' bounded waits, driven into their timeout path with
the test hook (every CTA's first wait gives up at once, after its copies were
issued): the call returns cudaErrorLaunchTimeout, the status word is set, and the
context stays usable.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from rocket_gb300 import _native

pytestmark = pytest.mark.gpu


class Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.check(self.cu.cuInit(0))

    @staticmethod
    def check(rc):
        assert rc == 0, f"CUDA driver error {rc}"

    def create_context(self, ordinal=0):
        dev = ctypes.c_int(0)
        self.check(self.cu.cuDeviceGet(ctypes.byref(dev), ordinal))
        ctx = ctypes.c_void_p(0)
        self.check(self.cu.cuCtxCreate_v2(ctypes.byref(ctx), 0, dev))
        return ctx

    def current(self):
        ctx = ctypes.c_void_p(0)
        self.check(self.cu.cuCtxGetCurrent(ctypes.byref(ctx)))
        return ctx

    def set_current(self, ctx):
        self.check(self.cu.cuCtxSetCurrent(ctx))

    def destroy(self, ctx):
        self.check(self.cu.cuCtxDestroy_v2(ctx))

    def upload(self, a):
        a = np.ascontiguousarray(a)
        p = ctypes.c_uint64(0)
        self.check(self.cu.cuMemAlloc_v2(ctypes.byref(p), ctypes.c_size_t(max(a.nbytes, 8))))
        if a.nbytes:
            self.check(self.cu.cuMemcpyHtoD_v2(p, a.ctypes.data_as(ctypes.c_void_p),
                                               ctypes.c_size_t(a.nbytes)))
        return p.value

    def alloc(self, nbytes):
        p = ctypes.c_uint64(0)
        self.check(self.cu.cuMemAlloc_v2(ctypes.byref(p), ctypes.c_size_t(max(nbytes, 8))))
        return p.value

    def read_double(self, ptr):
        out = np.zeros(1, np.float64)
        self.check(self.cu.cuMemcpyDtoH_v2(out.ctypes.data_as(ctypes.c_void_p),
                                           ctypes.c_uint64(ptr), ctypes.c_size_t(8)))
        return float(out[0])

    def free(self, ptr):
        self.check(self.cu.cuMemFree_v2(ctypes.c_uint64(ptr)))


def test_compare_in_two_created_and_destroyed_contexts():
    L = _native.load()
    torch.cuda.synchronize()
    drv = Driver()
    saved = drv.current()
    cases = [O.bindings_compare_case(3, 100000, 0.5), O.bindings_compare_case(4, 20000, 1.0)]
    try:
        for lk, lv, rk, rv, _ in cases:
            exact = O.compare_fp64(lk.view(np.uint32), lv, rk.view(np.uint32), rv)
            ctx = drv.create_context()  # current on this thread from here
            bufs = []
            try:
                dlk, dlv, drk, drv_ = (drv.upload(x) for x in (lk, lv, rk, rv))
                nscr = int(L.estimateScratchMemory(b"DNA", 3, max(len(lk), len(rk))))
                scratch = drv.alloc(nscr)
                out = drv.alloc(8)
                bufs = [dlk, dlv, drk, drv_, scratch, out]
                # stream 0: the legacy default stream of this context
                assert L.compareCompositionVectors(0, scratch, nscr, dlk, dlv, len(lk), drk, drv_,
                                                   len(rk), out) == 0
                c = drv.read_double(out)
                assert abs(c - exact) <= 1e-12 * max(1.0, abs(exact))
                assert L.compareCompositionVectorsStatic(0, dlk, dlv, len(lk), drk, drv_, len(rk),
                                                         out) == 0
                c2 = drv.read_double(out)
                assert abs(c2 - exact) <= 1e-12 * max(1.0, abs(exact))
            finally:
                for b in bufs:
                    drv.free(b)
                drv.destroy(ctx)
    finally:
        drv.set_current(saved)
    # torch's context still works after the others are gone
    x = torch.ones(4, device="cuda")
    assert float(x.sum().item()) == 4.0


def test_bounded_wait_timeout_path():
    """The first wait of every CTA gives up at once: status bit 1, return code
    cudaErrorLaunchTimeout, every issued copy drained before the CTA exits; the
    next call (default limit) is exact again."""
    L = _native.load()
    lk, lv, rk, rv, _ = O.bindings_compare_case(5, 100000, 0.5)  # about 40 tiles
    exact = O.compare_fp64(lk.view(np.uint32), lv, rk.view(np.uint32), rv)
    t = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (lk, lv, rk, rv)]
    nscr = int(L.estimateScratchMemory(b"DNA", 3, max(len(lk), len(rk))))
    scratch = torch.zeros(nscr, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    args = (st, scratch.data_ptr(), nscr, t[0].data_ptr(), t[1].data_ptr(), len(lk),
            t[2].data_ptr(), t[3].data_ptr(), len(rk), out.data_ptr())
    L.phyloCompareTestWaitLimit(0)
    try:
        rc = L.compareCompositionVectors(*args)
        status = int(scratch[4:8].cpu().numpy().view(np.uint32)[0])
        rc_static = L.compareCompositionVectorsStatic(st, *args[3:])
    finally:
        L.phyloCompareTestWaitLimit(0xFFFFFFFF)
    assert rc == 702  # cudaErrorLaunchTimeout
    assert status & 1  # DEV_WAIT_TIMEOUT
    assert rc_static == 702
    # the context is intact and the default limit is back
    assert L.compareCompositionVectors(*args) == 0
    assert abs(float(out.item()) - exact) <= 1e-12 * max(1.0, abs(exact))
    assert int(scratch[4:8].cpu().numpy().view(np.uint32)[0]) == 0
