"""Mirror of SequenceAnalysisContext, Rocket's plug-in for this application
(phylogenetics_analysis/SequenceAnalysisContext.java:19-143), implementing the
ApplicationContext contract (rocket/scheduler/ApplicationContext.java:11-99).

Buffers are torch uint8 tensors standing in for Rocket's CudaMem slices.  A
preprocessed item occupies ``[keys(n) | values(n)]`` of its cache slot, exactly
as the reference lays it out, so correlate_gpu works on slot slices of
8 * n bytes.
"""
from __future__ import annotations

import struct

import torch

from . import fasta
from .kernels import KEY_SIZE, VALUE_SIZE, CompositionVectorKernels


class SequenceAnalysisContext:
    def __init__(self, alphabet: str, k: int, max_vector_size: int, max_input_size: int,
                 device=None):
        while max_vector_size % 32 != 0:  # :30
            max_vector_size += 1
        self.kernel = CompositionVectorKernels(alphabet, k, max_vector_size, max_input_size, device)
        self.max_vector_size = max_vector_size
        self.max_input_size = max_input_size
        self.device = self.kernel.device

    # sizes (:38-50)
    def get_max_file_size(self) -> int:
        return self.max_input_size

    def get_max_input_size(self) -> int:
        return self.max_vector_size * (KEY_SIZE + VALUE_SIZE)

    def get_max_output_size(self) -> int:
        return 8

    # host side (:60-76)
    def parse_files(self, key, inputs, output: bytearray = None) -> bytes:
        """Returns the parsed residue stream (and fills ``output`` if given)."""
        data = fasta.parse_file_bytes(bytes(inputs[0]), str(key))
        if output is not None:
            output[:len(data)] = data
        return data

    # device side (:79-104)
    def preprocess_input_gpu(self, key, input_buf: torch.Tensor, output_buf: torch.Tensor,
                             input_len: int = None) -> int:
        m = self.max_vector_size
        keys = output_buf[:m * KEY_SIZE].view(torch.int32)
        values = output_buf[m * KEY_SIZE:m * (KEY_SIZE + VALUE_SIZE)].view(torch.float32)
        size = self.kernel.build_vector_gpu(input_buf, keys, values, input_len)
        # move the values right after the keys; chunks never overlap (:92-100).
        offset = 0
        with torch.cuda.stream(self.kernel.stream):
            while offset < size:
                chunk = min(size - offset, m - size)
                if chunk <= 0:  # size == max: values already follow the keys
                    break
                src = output_buf[(m + offset) * KEY_SIZE:(m + offset + chunk) * KEY_SIZE]
                dst = output_buf[(size + offset) * KEY_SIZE:(size + offset + chunk) * KEY_SIZE]
                dst.copy_(src)
                offset += chunk
        self.kernel.stream.synchronize()
        return size * (KEY_SIZE + VALUE_SIZE)

    @staticmethod
    def _split(slot: torch.Tensor):
        n = slot.numel() // (KEY_SIZE + VALUE_SIZE)
        keys = slot[:n * KEY_SIZE]
        values = slot[n * KEY_SIZE:n * (KEY_SIZE + VALUE_SIZE)]
        return n, keys, values

    def correlate_gpu(self, left_key, left: torch.Tensor, right_key, right: torch.Tensor,
                      output: torch.Tensor) -> int:
        """(:107-131) writes C (double) to output[:8]."""
        nl, lk, lv = self._split(left)
        nr, rk, rv = self._split(right)
        self.kernel.compare_vectors_gpu(lk, lv, nl, rk, rv, nr, output)
        return 8

    def postprocess_output(self, left_key, right_key, output: bytes) -> float:
        """(:134-136) the raw cosine C; distance() gives D = (1 - C) / 2."""
        return struct.unpack("<d", bytes(output[:8]))[0]

    @staticmethod
    def distance(c: float) -> float:
        return (1.0 - c) / 2.0

    def destroy(self) -> None:
        self.kernel.cleanup()
