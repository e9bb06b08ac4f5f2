"""ctypes view of libphylogenetics.so.

The library is built in-tree (``rocket_gb300/libphylogenetics.so``).  There is
no fallback: if the library is missing or fails to load, every entry point
raises, so no CPU path can silently stand in for the device code.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

c_long = ctypes.c_long
c_int = ctypes.c_int
c_uint = ctypes.c_uint
c_ptr = ctypes.c_size_t  # uintptr_t
c_char_p = ctypes.c_char_p


class NativeLibraryError(RuntimeError):
    pass


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Loads the library; raises NativeLibraryError if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if build_if_missing:
                _build.build()
            else:
                raise NativeLibraryError(
                    f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                    "(the CUDA library is required; there is no CPU fallback)")
        L = ctypes.CDLL(path)
        _declare(L)
        _lib = L
        return L


def _declare(L: ctypes.CDLL) -> None:
    # drop-in boundary (Bindings.java:17-45)
    L.estimateScratchMemory.argtypes = [c_char_p, c_int, c_int]
    L.estimateScratchMemory.restype = c_long
    L.buildCompositionVector.argtypes = [c_ptr, c_ptr, c_long, c_char_p, c_int, c_ptr, c_long,
                                         c_ptr, c_ptr, c_ptr, c_int]
    L.buildCompositionVector.restype = c_int
    L.compareCompositionVectors.argtypes = [c_ptr, c_ptr, c_long, c_ptr, c_ptr, c_int, c_ptr,
                                            c_ptr, c_int, c_ptr]
    L.compareCompositionVectors.restype = c_int
    L.compareCompositionVectorsStatic.argtypes = [c_ptr, c_ptr, c_ptr, c_int, c_ptr, c_ptr, c_int,
                                                  c_ptr]
    L.compareCompositionVectorsStatic.restype = c_int
    L.phyloCompareTestWaitLimit.argtypes = [c_uint]
    L.phyloCompareTestWaitLimit.restype = None
    # batched construction
    L.phyloBuildBatchScratch.argtypes = [c_char_p, c_int, c_int, c_long]
    L.phyloBuildBatchScratch.restype = c_long
    L.phyloBuildBatchPlan.argtypes = [c_ptr, c_ptr, c_long, c_char_p, c_int, c_int, c_ptr, c_ptr,
                                      c_long, c_ptr, c_ptr]
    L.phyloBuildBatchPlan.restype = c_int
    L.phyloBuildBatchPlanAsync.argtypes = [c_ptr, c_ptr, c_long, c_char_p, c_int, c_int, c_ptr,
                                           c_ptr, c_long, c_ptr]
    L.phyloBuildBatchPlanAsync.restype = c_int
    L.phyloBuildBatchSummaryBytes.argtypes = [c_int]
    L.phyloBuildBatchSummaryBytes.restype = c_long
    L.phyloBuildBatchEmit.argtypes = [c_ptr, c_ptr, c_long, c_char_p, c_int, c_int, c_long, c_ptr,
                                      c_ptr, c_ptr, c_long, c_ptr]
    L.phyloBuildBatchEmit.restype = c_int
    L.phyloBuildBatchNorms.argtypes = [c_ptr, c_ptr, c_long, c_char_p, c_int, c_int, c_long, c_ptr]
    L.phyloBuildBatchNorms.restype = c_int
    L.phyloBuildBatchCounts.argtypes = [c_ptr, c_ptr, c_long, c_char_p, c_int, c_int, c_long,
                                        c_int, c_ptr, c_ptr, c_ptr]
    L.phyloBuildBatchCounts.restype = c_int
    L.phyloBuildLaunchesPerBatch.argtypes = []
    L.phyloBuildLaunchesPerBatch.restype = c_int
    # pair engine
    L.phyloWindowIndex.argtypes = [c_ptr, c_ptr, c_ptr, c_int, c_int, c_uint, c_long, c_ptr]
    L.phyloWindowIndex.restype = c_int
    L.phyloPairsPrepare.argtypes = [c_int, c_int, c_int, ctypes.POINTER(c_int)]
    L.phyloPairsPrepare.restype = c_int
    L.phyloPairsSmemBytes.argtypes = [c_int, c_int, c_int]
    L.phyloPairsSmemBytes.restype = c_int
    L.phyloPairsThreads.argtypes = [c_int, c_int, c_int]
    L.phyloPairsThreads.restype = c_int
    L.phyloPairsLaunch.argtypes = [c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                                   c_uint, c_int, c_ptr, c_ptr, c_ptr, c_int, c_ptr, c_ptr, c_int,
                                   c_ptr, c_int, c_int, c_int]
    L.phyloPairsLaunch.restype = c_int
    L.phyloPairsReduce.argtypes = [c_ptr, c_ptr, c_ptr, c_int, c_int, c_int, c_int, c_ptr, c_ptr,
                                   c_ptr, c_long, c_int, c_int]
    L.phyloPairsReduce.restype = c_int
    L.phyloSelfDot.argtypes = [c_ptr, c_ptr, c_ptr, c_int, c_long, c_ptr, c_ptr, c_long]
    L.phyloSelfDot.restype = c_int
    L.phyloSelfDotPartBytes.argtypes = [c_int, c_long]
    L.phyloSelfDotPartBytes.restype = c_long
    L.phyloComparePairAsync.argtypes = [c_ptr, c_ptr, c_long, c_ptr, c_ptr, c_int, c_ptr, c_ptr,
                                        c_int, c_ptr]
    L.phyloComparePairAsync.restype = c_int
    L.phyloKeyRankScratch.argtypes = [c_long]
    L.phyloKeyRankScratch.restype = c_long
    L.phyloKeyRankBitmapBytes.argtypes = [c_long]
    L.phyloKeyRankBitmapBytes.restype = c_long
    L.phyloKeyRanks.argtypes = [c_ptr, c_ptr, c_long, c_long, c_ptr, c_ptr, c_int, c_long, c_ptr,
                                c_ptr, c_ptr]
    L.phyloKeyRanks.restype = c_int
    L.phyloKeyRankIndex.argtypes = [c_ptr, c_ptr, c_long, c_long, c_ptr, c_ptr, c_int, c_long,
                                    c_long, c_ptr, c_int, c_uint, c_ptr, c_ptr]
    L.phyloKeyRankIndex.restype = c_int
    L.phyloCompareTileElements.argtypes = []
    L.phyloCompareTileElements.restype = c_int
    L.phyloComparePairsManyScratch.argtypes = [c_int, c_long]
    L.phyloComparePairsManyScratch.restype = c_long
    L.phyloComparePairsMany.argtypes = [c_ptr, c_ptr, c_long] + [c_ptr] * 10 + [c_int, c_long, c_ptr]
    L.phyloComparePairsMany.restype = c_int
    # key-major (postings) pair engine
    L.phyloPostingsSmemBytes.argtypes = [c_int, c_int]
    L.phyloPostingsSmemBytes.restype = c_long
    L.phyloPostingsCapacity.argtypes = [c_int, c_int]
    L.phyloPostingsCapacity.restype = c_long
    L.phyloPostingsThreads.argtypes = [c_int]
    L.phyloPostingsThreads.restype = c_int
    L.phyloPostingsPrepare.argtypes = [c_int, c_int, ctypes.POINTER(c_int)]
    L.phyloPostingsPrepare.restype = c_int
    L.phyloPostingsLaunch.argtypes = [c_ptr] * 9 + [c_uint, c_int] + [c_ptr] * 3 + [c_int] + \
        [c_ptr] * 4 + [c_int, c_int]
    L.phyloPostingsLaunch.restype = c_int
    L.phyloPostingsReduce.argtypes = [c_ptr, c_ptr, c_ptr, c_int, c_int, c_ptr, c_ptr, c_ptr,
                                      c_long, c_int, c_int]
    L.phyloPostingsReduce.restype = c_int


# Every symbol that include/phylogenetics.h declares.
EXPORTED = [
    "estimateScratchMemory", "buildCompositionVector", "compareCompositionVectors",
    "compareCompositionVectorsStatic", "phyloCompareTestWaitLimit", "phyloBuildBatchScratch", "phyloBuildBatchPlan", "phyloBuildBatchPlanAsync",
    "phyloBuildBatchSummaryBytes", "phyloBuildBatchEmit", "phyloBuildBatchNorms",
    "phyloBuildBatchCounts", "phyloBuildLaunchesPerBatch", "phyloWindowIndex",
    "phyloPairsPrepare", "phyloPairsSmemBytes", "phyloPairsThreads", "phyloPairsLaunch",
    "phyloPairsReduce",
    "phyloSelfDot", "phyloSelfDotPartBytes", "phyloKeyRankScratch", "phyloKeyRankBitmapBytes",
    "phyloKeyRanks", "phyloKeyRankIndex",
    "phyloCompareTileElements", "phyloComparePairsManyScratch",
    "phyloComparePairsMany", "phyloComparePairAsync",
    "phyloPostingsSmemBytes", "phyloPostingsCapacity", "phyloPostingsThreads",
    "phyloPostingsPrepare", "phyloPostingsLaunch", "phyloPostingsReduce",
]


CUDA_ERROR_NAMES = {0: "cudaSuccess", 1: "cudaErrorInvalidValue", 2: "cudaErrorMemoryAllocation",
                    702: "cudaErrorLaunchTimeout", 999: "cudaErrorUnknown"}


class CudaException(RuntimeError):
    """Mirror of jcuda.CudaException raised by CompositionVectorKernels on a
    nonzero status (CompositionVectorKernels.java:60-62, 84-86)."""

    def __init__(self, code: int):
        self.code = code
        super().__init__(CUDA_ERROR_NAMES.get(code, f"cudaError({code})"))


def check(code: int) -> None:
    if code != 0:
        raise CudaException(code)
