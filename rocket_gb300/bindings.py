"""Python mirror of the reference's JNA interface (Bindings.java:14-46).

``Bindings.INSTANCE`` exposes the three drop-in entry points with the Java
binding's argument order and meaning: device pointers and the stream are
plain integers (JNA ``Pointer``), ``vector_size_ptr`` is a host int array
(JNA ``int[]``), and each call returns the CUDA status code.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native


class _Bindings:
    def __init__(self):
        self._L = None

    @property
    def L(self):
        if self._L is None:
            self._L = _native.load()
        return self._L

    def estimateScratchMemory(self, alphabet: str, k: int, max_vector_size: int) -> int:
        return int(self.L.estimateScratchMemory(alphabet.encode(), k, max_vector_size))

    def buildCompositionVector(self, stream: int, d_temp_storage_ptr: int, temp_storage_size: int,
                               alphabet: str, k: int, d_string_ptr: int, string_len: int,
                               d_vector_keys_ptr: int, d_vector_values_ptr: int,
                               vector_size_ptr: np.ndarray, max_vector_size: int) -> int:
        assert vector_size_ptr.dtype == np.int32 and vector_size_ptr.size >= 1
        return int(self.L.buildCompositionVector(
            stream, d_temp_storage_ptr, temp_storage_size, alphabet.encode(), k, d_string_ptr,
            string_len, d_vector_keys_ptr, d_vector_values_ptr,
            vector_size_ptr.ctypes.data_as(ctypes.c_void_p).value, max_vector_size))

    def compareCompositionVectors(self, stream: int, d_temp_storage_ptr: int,
                                  temp_storage_size: int, d_left_keys_ptr: int,
                                  d_left_values_ptr: int, left_size: int, d_right_keys_ptr: int,
                                  d_right_values_ptr: int, right_size: int,
                                  d_output_ptr: int) -> int:
        return int(self.L.compareCompositionVectors(
            stream, d_temp_storage_ptr, temp_storage_size, d_left_keys_ptr, d_left_values_ptr,
            left_size, d_right_keys_ptr, d_right_values_ptr, right_size, d_output_ptr))


class Bindings:
    INSTANCE = _Bindings()
