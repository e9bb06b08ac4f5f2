"""ctypes binding of the reference's own library (phylogenetics/src/main/cpp/native.cu
compiled unmodified into oracle/_ref/libphylogenetics_ref.so by ``make -C oracle ref``).

Test infrastructure: the parity tests drive it beside this project's library on
the same device buffers, with the calling convention of the reference's JNA
interface (Bindings.java:15-45).  The reference defines compareCompositionVectors
as returning ``double`` (native.cu:755), so its status arrives as a double here.
"""
from __future__ import annotations

import ctypes
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.path.join(ROOT, "oracle", "_ref", "src", "native.cu")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libphylogenetics_ref.so")

_lib = None


def staged() -> bool:
    """True where the reference's CUDA file was staged (it travels with the tree)."""
    return os.path.exists(REF_SRC)


def load() -> ctypes.CDLL:
    """The reference library; raises if its source was staged but it did not build."""
    global _lib
    if _lib is None:
        if not os.path.exists(REF_LIB):
            raise FileNotFoundError(
                f"{REF_LIB} is missing although {REF_SRC} is staged: the reference build failed")
        L = ctypes.CDLL(REF_LIB)
        vp, c_int, c_long, u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_uint32
        L.estimateScratchMemory.argtypes = [ctypes.c_char_p, c_int, c_int]
        L.estimateScratchMemory.restype = c_long
        L.buildCompositionVector.argtypes = [vp, vp, c_long, ctypes.c_char_p, c_int, vp, c_long,
                                             vp, vp, vp, c_int]
        L.buildCompositionVector.restype = c_int
        L.compareCompositionVectors.argtypes = [vp, vp, c_long, vp, vp, u32, vp, vp, u32, vp]
        L.compareCompositionVectors.restype = ctypes.c_double
        _lib = L
    return _lib


def scratch_bytes(alphabet: str, k: int, max_vector_size: int) -> int:
    return int(load().estimateScratchMemory(alphabet.encode(), k, int(max_vector_size)))


def build(stream: int, scratch, alphabet: str, k: int, d_string, string_len: int, d_keys,
          d_values, size_out, max_vector_size: int) -> int:
    """buildCompositionVector (native.cu:718-752); size_out: numpy int32[1]."""
    return int(load().buildCompositionVector(
        stream, scratch.data_ptr(), scratch.numel(), alphabet.encode(), k, d_string.data_ptr(),
        int(string_len), d_keys.data_ptr(), d_values.data_ptr(), size_out.ctypes.data,
        int(max_vector_size)))


def compare(stream: int, scratch, lk, lv, nl: int, rk, rv, nr: int, d_out) -> int:
    """compareCompositionVectors (native.cu:755-780); the status comes back as a double."""
    r = load().compareCompositionVectors(stream, scratch.data_ptr(), scratch.numel(),
                                         lk.data_ptr(), lv.data_ptr(), int(nl), rk.data_ptr(),
                                         rv.data_ptr(), int(nr), d_out.data_ptr())
    return int(r)


def compare_block_race(nl: int, nr: int, items_per_block: int = 256) -> bool:
    """Sizes at which the reference's compare may race with itself: it carves
    ceil((nl + nr) / 256) range slots but writes one more (native.cu:660-675), and
    when that count is a multiple of 32 the extra slot is the first partial sum,
    which block 0 writes while the last block reads it (native.cu:564-565, 639-641)."""
    nb = -(-(nl + nr) // items_per_block)
    return nb % 32 == 0
