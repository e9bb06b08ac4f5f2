"""Mirror of CompositionVectorKernels (phylogenetics_analysis/kernels/
CompositionVectorKernels.java:32-89): owns one stream and one scratch buffer
per context and calls the C ABI.  Device memory is held in torch tensors
(``torch`` is used for allocation and streams only).

The reference class also carries the Java CPU path (buildCPU/compareCPU,
(:91-222); it is not part of the device product and is restated, as a test
oracle, under ``oracle/``.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native
from .bindings import Bindings

KEY_SIZE = 4
VALUE_SIZE = 4


def ptr(t: torch.Tensor) -> int:
    return int(t.data_ptr())


class CompositionVectorKernels:
    def __init__(self, alphabet: str, k: int, max_vector_size: int, max_input_size: int = 0,
                 device=None):
        if k < 3 or k > 25:  # CompositionVectorKernels.java:33
            raise ValueError(f"k should be in the range 3-25, not {k}")
        self.k = k
        self.alphabet = alphabet
        self.device = torch.device(device if device is not None else "cuda")
        self.stream = torch.cuda.Stream(device=self.device)
        self.max_vector_size = int(max_vector_size)
        scratch_size = Bindings.INSTANCE.estimateScratchMemory(alphabet, k, self.max_vector_size)
        self.scratch = torch.empty(max(scratch_size, 1), dtype=torch.uint8, device=self.device)
        self._size = np.zeros(1, np.int32)

    @property
    def stream_handle(self) -> int:
        return int(self.stream.cuda_stream)

    def build_vector_gpu(self, d_input: torch.Tensor, d_keys: torch.Tensor,
                         d_values: torch.Tensor, input_len: int = None) -> int:
        """buildVectorGPU (:45-66): returns the vector size."""
        n = d_input.numel() if input_len is None else int(input_len)
        # work queued on other streams that produced the input must be visible
        self.stream.wait_stream(torch.cuda.current_stream(self.device))
        err = Bindings.INSTANCE.buildCompositionVector(
            self.stream_handle, ptr(self.scratch), self.scratch.numel(), self.alphabet, self.k,
            ptr(d_input), n, ptr(d_keys), ptr(d_values), self._size, self.max_vector_size)
        if err != 0:
            raise _native.CudaException(err)
        self.stream.synchronize()
        return int(self._size[0])

    def compare_vectors_gpu(self, left_keys: torch.Tensor, left_values: torch.Tensor,
                            left_size: int, right_keys: torch.Tensor, right_values: torch.Tensor,
                            right_size: int, result: torch.Tensor) -> None:
        """compareVectorsGPU (:68-89): writes C (double) into ``result``."""
        self.stream.wait_stream(torch.cuda.current_stream(self.device))
        err = Bindings.INSTANCE.compareCompositionVectors(
            self.stream_handle, ptr(self.scratch), self.scratch.numel(), ptr(left_keys),
            ptr(left_values), int(left_size), ptr(right_keys), ptr(right_values), int(right_size),
            ptr(result))
        if err != 0:
            raise _native.CudaException(err)
        self.stream.synchronize()

    def cleanup(self) -> None:
        self.scratch = None
