"""CPU oracle for the composition-vector path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline /
reference arm import this module, always as the checker (or the timed CPU
baseline), never as the product path.  The product (``rocket_gb300``) never
imports it.

The C core (``phylo_oracle.c``) restates

* the GPU key rule of ``phylogenetics/src/main/cpp/native.cu`` (counting
  :220-256, totals :317-345, Markov alpha :350-400 with the reference's double
  operation order and the float-bits != 0 selection :402-458);
* the Java CPU path ``CompositionVectorKernels.buildCPU/compareCPU``
  (``src/main/java/nl/esciencecenter/phylogenetics_analysis/kernels/
  CompositionVectorKernels.java:91-222``);
* ``java.util.Random`` and the input generators of ``BindingsTest.java``.

This module adds what is easier to state exactly in Python: the norm as the
exact, correctly rounded sum of the float squares (``math.fsum``), the
normalised values ``float(alpha / sqrt(norm))`` (native.cu:415-468) and an
FP64 sparse cosine whose products are exact and whose sum is exact
(``math.fsum``).

Parity status: unpinned against reference OUTPUTS (the reference's CPU path is
Java and no JVM exists here; its GPU path cannot run here, and its sources are
not carried to the GPU host).  Pinned by hand-derived known answers and by the
reference tests' own input procedures (tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from typing import Dict, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libphylo_oracle.so")
_lib = None

ALPHABETS = {"protein": 0, "DNA": 1}
NSYM = {"protein": 21, "DNA": 4}
LETTERS = {"protein": "ACDEFGHIKLMNPQRSTVWYX", "DNA": "ACGT"}


def build() -> str:
    """Compile the oracle library (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        i32p = ctypes.POINTER(ctypes.c_int32)
        i64p = ctypes.POINTER(ctypes.c_int64)
        f32p = ctypes.POINTER(ctypes.c_float)
        c_i64, c_u64, c_int = ctypes.c_int64, ctypes.c_uint64, ctypes.c_int
        L.oracle_cv_slots.argtypes = [c_int, c_int, u8p, c_u64, u32p, u32p, u32p, u32p, u32p, u32p,
                                      c_i64, u32p]
        L.oracle_cv_slots.restype = c_i64
        L.oracle_cv_candidates.argtypes = [c_int, c_int, u8p, c_u64, u32p, u32p, u32p, u32p, u32p,
                                           u32p, c_i64, u32p, i64p]
        L.oracle_cv_candidates.restype = c_i64
        L.oracle_count_tables.argtypes = [c_int, c_int, u8p, c_u64, u32p, u32p, u32p]
        L.oracle_count_tables.restype = c_int
        L.java_build_cpu.argtypes = [c_int, c_int, u8p, c_u64, u32p, f32p, c_i64]
        L.java_build_cpu.restype = c_i64
        L.java_compare_cpu.argtypes = [i32p, f32p, c_i64, i32p, f32p, c_i64]
        L.java_compare_cpu.restype = ctypes.c_double
        L.oracle_compare_fp64.argtypes = [u32p, f32p, c_i64, u32p, f32p, c_i64]
        L.oracle_compare_fp64.restype = ctypes.c_double
        L.java_build_many.argtypes = [c_int, c_int, c_int, ctypes.POINTER(u8p),
                                      ctypes.POINTER(c_u64), ctypes.POINTER(u32p),
                                      ctypes.POINTER(f32p), i64p, i64p, c_int]
        L.java_build_many.restype = c_i64
        L.java_compare_pairs.argtypes = [c_int, i32p, i32p, ctypes.POINTER(i32p),
                                         ctypes.POINTER(f32p), i64p, ctypes.POINTER(ctypes.c_double),
                                         c_int]
        L.java_compare_pairs.restype = None
        L.oracle_max_threads.restype = c_int
        L.jrandom_ints.argtypes = [c_i64, c_int, ctypes.c_int32, i32p]
        L.jrandom_floats.argtypes = [c_i64, c_int, f32p]
        L.bindings_generate_input.argtypes = [c_i64, c_i64, c_int, u8p, c_i64]
        L.bindings_generate_input.restype = c_i64
        L.bindings_compare_case.argtypes = [c_i64, ctypes.c_int32, ctypes.c_double, i32p, f32p,
                                            i32p, f32p, i32p]
        L.bindings_compare_case.restype = c_int
        _lib = L
    return _lib


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def _as_bytes(seq) -> np.ndarray:
    if isinstance(seq, np.ndarray):
        return np.ascontiguousarray(seq, dtype=np.uint8)
    if isinstance(seq, str):
        seq = seq.encode("ascii")
    return np.frombuffer(bytes(seq), dtype=np.uint8).copy()


# --------------------------------------------------------------------------
# native.cu rule
# --------------------------------------------------------------------------

def cv_native(seq, k: int, alphabet: str = "protein", formulation: str = "candidates",
              with_values: bool = True) -> Dict[str, np.ndarray]:
    """Composition vector by the reference GPU rule (native.cu:258-477).

    Returns keys (uint32, ascending), alpha (float32; the float whose bits the
    reference stores, native.cu:399), the per-key counts full/prefix/suffix/
    middle, the totals n0/n1/n2, ``norm`` (exact sum of float squares) and
    ``values`` = float(alpha / sqrt(norm)).
    """
    s = _as_bytes(seq)
    a = ALPHABETS[alphabet]
    L = lib()
    cap = max(16, 21 * max(len(s), 1) + 64)
    keys = np.empty(cap, np.uint32)
    bits = np.empty(cap, np.uint32)
    c0, c1p, c1s, c2m = (np.empty(cap, np.uint32) for _ in range(4))
    tot = np.zeros(3, np.uint32)
    ncand = ctypes.c_int64(0)
    args = (a, k, _ptr(s, ctypes.c_uint8), len(s), _ptr(keys, ctypes.c_uint32),
            _ptr(bits, ctypes.c_uint32), _ptr(c0, ctypes.c_uint32), _ptr(c1p, ctypes.c_uint32),
            _ptr(c1s, ctypes.c_uint32), _ptr(c2m, ctypes.c_uint32), cap, _ptr(tot, ctypes.c_uint32))
    if formulation == "slots":
        n = L.oracle_cv_slots(*args)
        ncand.value = -1
    else:
        n = L.oracle_cv_candidates(*args, ctypes.byref(ncand))
    if n < 0:
        raise ValueError(f"oracle_cv failed ({n}) for k={k} alphabet={alphabet}")
    assert n <= cap
    out = dict(keys=keys[:n].copy(), alpha=bits[:n].copy().view(np.float32),
               c0=c0[:n].copy(), c1p=c1p[:n].copy(), c1s=c1s[:n].copy(), c2m=c2m[:n].copy(),
               n0=int(tot[0]), n1=int(tot[1]), n2=int(tot[2]), candidates=int(ncand.value))
    if with_values:
        out["norm"], out["values"] = normalise(out["alpha"])
    return out


def exact_sum_of_floats(x: np.ndarray) -> float:
    """The correctly rounded double of the exact sum of float32 values.

    Every finite float32 is m * 2^(e - 150) with an integer significand m < 2^24
    and biased exponent e (1 for subnormals).  The significands are summed per
    exponent in two 12-bit halves -- each half-sum stays below 2^53 for up to
    2^41 values, so the float64 bin counts are exact -- and the 2 x 256 exact
    partial sums are added by math.fsum, which rounds once."""
    x = np.ascontiguousarray(x, np.float32)
    if len(x) == 0:
        return 0.0
    if not np.all(np.isfinite(x)):
        return float(np.sum(x.astype(np.float64)))  # inf / nan propagate
    b = x.view(np.uint32)
    terms = []
    negative = b >> 31
    for sign, part in ((1.0, b), (-1.0, None)):
        if part is None:
            if not negative.any():
                break
            part = b[negative.astype(bool)]
        elif negative.any():
            part = b[~negative.astype(bool)]
        e = (part >> 23) & 0xFF          # biased exponent (sign bit cleared)
        m = part & 0x7FFFFF
        m = m | ((e > 0).astype(np.uint32) << 23)  # the implicit bit of normal numbers
        e = np.maximum(e, 1)
        lo = np.bincount(e, weights=m & 0xFFF, minlength=256)
        hi = np.bincount(e, weights=m >> 12, minlength=256)
        for k in np.flatnonzero(lo):
            terms.append(sign * math.ldexp(lo[k], int(k) - 150))
        for k in np.flatnonzero(hi):
            terms.append(sign * math.ldexp(hi[k], int(k) - 138))
    return math.fsum(terms)


def normalise(alpha: np.ndarray):
    """norm = exact sum of float(f*f) (native.cu:415-428, summed exactly);
    values = float(double(f) / sqrt(norm)) (native.cu:460-468)."""
    f = np.asarray(alpha, np.float32)
    sq = f * f  # float product, as the reference's lambda
    norm = exact_sum_of_floats(sq)
    with np.errstate(invalid="ignore", divide="ignore"):
        values = (f.astype(np.float64) / math.sqrt(norm)).astype(np.float32) if len(f) else \
            np.zeros(0, np.float32)
    return norm, values


def digest(keys: np.ndarray, values: np.ndarray):
    """(size, key digest, value digest): order-sensitive 64-bit sums over a vector,
    sum (key_i + 1)(2 i + 1) and sum (bits(value_i) + 7)(i + 3), wrapping mod 2^64."""
    k = np.asarray(keys, np.uint32).astype(np.uint64)
    v = np.asarray(values, np.float32).view(np.uint32).astype(np.uint64)
    i = np.arange(len(k), dtype=np.uint64)
    with np.errstate(over="ignore"):
        hk = int(np.sum((k + np.uint64(1)) * (np.uint64(2) * i + np.uint64(1)), dtype=np.uint64))
        hv = int(np.sum((v + np.uint64(7)) * (i + np.uint64(3)), dtype=np.uint64))
    return len(k), hk, hv


def cv_native_digest(args):
    """digest() of cv_native(seq, k) -- for a worker pool (no large arrays back)."""
    seq, k = args
    r = cv_native(seq, k)
    return digest(r["keys"], r["values"])


def count_tables(seq, k: int, alphabet: str = "protein"):
    """Dense (K-1)- and (K-2)-mer count tables and totals (native.cu:220-345)."""
    s = _as_bytes(seq)
    A = NSYM[alphabet]
    k1 = np.zeros(A ** (k - 1), np.uint32)
    k2 = np.zeros(A ** (k - 2), np.uint32)
    tot = np.zeros(3, np.uint32)
    rc = lib().oracle_count_tables(ALPHABETS[alphabet], k, _ptr(s, ctypes.c_uint8), len(s),
                                   _ptr(k1, ctypes.c_uint32), _ptr(k2, ctypes.c_uint32),
                                   _ptr(tot, ctypes.c_uint32))
    if rc:
        raise ValueError(rc)
    return k1, k2, (int(tot[0]), int(tot[1]), int(tot[2]))


# --------------------------------------------------------------------------
# compare
# --------------------------------------------------------------------------

def compare_fp64(lk, lv, rk, rv) -> float:
    """C = sum over shared keys of a*b: exact products, exact sum."""
    lk = np.asarray(lk, np.uint32)
    rk = np.asarray(rk, np.uint32)
    _, il, ir = np.intersect1d(lk, rk, assume_unique=True, return_indices=True)
    prod = np.asarray(lv, np.float32)[il].astype(np.float64) * \
        np.asarray(rv, np.float32)[ir].astype(np.float64)
    return math.fsum(prod.tolist())


def distance(c: float) -> float:
    """D = (1 - C) / 2."""
    return (1.0 - c) / 2.0


def java_compare(lk, lv, rk, rv) -> float:
    """CompositionVectorKernels.compareCPU (:147-168)."""
    lk = np.ascontiguousarray(lk, np.int32)
    rk = np.ascontiguousarray(rk, np.int32)
    lv = np.ascontiguousarray(lv, np.float32)
    rv = np.ascontiguousarray(rv, np.float32)
    return lib().java_compare_cpu(_ptr(lk, ctypes.c_int32), _ptr(lv, ctypes.c_float), len(lk),
                                  _ptr(rk, ctypes.c_int32), _ptr(rv, ctypes.c_float), len(rk))


def java_build(seq, k: int, alphabet: str = "protein"):
    """CompositionVectorKernels.buildCPU (:91-145)."""
    s = _as_bytes(seq)
    cap = max(16, (NSYM[alphabet] ** 2) * max(len(s), 1) + 64)
    cap = min(cap, NSYM[alphabet] ** k + 16)
    keys = np.empty(cap, np.uint32)
    vals = np.empty(cap, np.float32)
    n = lib().java_build_cpu(ALPHABETS[alphabet], k, _ptr(s, ctypes.c_uint8), len(s),
                             _ptr(keys, ctypes.c_uint32), _ptr(vals, ctypes.c_float), cap)
    if n < 0:
        raise ValueError(n)
    return keys[:n].copy(), vals[:n].copy()


def java_build_many(seqs: Sequence[np.ndarray], k: int, alphabet: str = "protein",
                    caps: Sequence[int] = None, threads: int = 0):
    """buildCPU over many proteomes, OpenMP over proteomes (CPU baseline)."""
    L = lib()
    n = len(seqs)
    seqs = [_as_bytes(s) for s in seqs]
    if caps is None:
        caps = [min(NSYM[alphabet] ** k, 21 * len(s) + 64) for s in seqs]
    keys = [np.empty(c, np.uint32) for c in caps]
    vals = [np.empty(c, np.float32) for c in caps]
    P8 = ctypes.POINTER(ctypes.c_uint8)
    P32 = ctypes.POINTER(ctypes.c_uint32)
    PF = ctypes.POINTER(ctypes.c_float)
    sp = (P8 * n)(*[_ptr(s, ctypes.c_uint8) for s in seqs])
    lens = (ctypes.c_uint64 * n)(*[len(s) for s in seqs])
    kp = (P32 * n)(*[_ptr(x, ctypes.c_uint32) for x in keys])
    vp = (PF * n)(*[_ptr(x, ctypes.c_float) for x in vals])
    capa = np.asarray(caps, np.int64)
    nnz = np.zeros(n, np.int64)
    L.java_build_many(ALPHABETS[alphabet], k, n, sp, lens, kp, vp, _ptr(capa, ctypes.c_int64),
                      _ptr(nnz, ctypes.c_int64), threads)
    return [(keys[i][:nnz[i]], vals[i][:nnz[i]]) for i in range(n)]


def java_compare_pairs(vectors, pairs, threads: int = 0) -> np.ndarray:
    """compareCPU over a list of (i, j) pairs, OpenMP over pairs (CPU baseline)."""
    L = lib()
    n = len(vectors)
    ks = [np.ascontiguousarray(v[0]).view(np.int32) for v in vectors]
    vs = [np.ascontiguousarray(v[1], np.float32) for v in vectors]
    PI = ctypes.POINTER(ctypes.c_int32)
    PF = ctypes.POINTER(ctypes.c_float)
    kp = (PI * n)(*[_ptr(x, ctypes.c_int32) for x in ks])
    vp = (PF * n)(*[_ptr(x, ctypes.c_float) for x in vs])
    sizes = np.asarray([len(x) for x in ks], np.int64)
    pairs = np.asarray(pairs, np.int32).reshape(-1, 2)
    pi = np.ascontiguousarray(pairs[:, 0])
    pj = np.ascontiguousarray(pairs[:, 1])
    out = np.zeros(len(pairs), np.float64)
    L.java_compare_pairs(len(pairs), _ptr(pi, ctypes.c_int32), _ptr(pj, ctypes.c_int32), kp, vp,
                         _ptr(sizes, ctypes.c_int64), _ptr(out, ctypes.c_double), threads)
    return out


def max_threads() -> int:
    return int(lib().oracle_max_threads())


# --------------------------------------------------------------------------
# java.util.Random and BindingsTest inputs
# --------------------------------------------------------------------------

class JavaRandom:
    """Pure-Python java.util.Random (48-bit LCG), used to cross-check the C clone."""

    MULT = 0x5DEECE66D
    MASK = (1 << 48) - 1

    def __init__(self, seed: int):
        self.seed = (seed ^ self.MULT) & self.MASK

    def next(self, bits: int) -> int:
        self.seed = (self.seed * self.MULT + 0xB) & self.MASK
        r = self.seed >> (48 - bits)
        if r & (1 << (bits - 1)) and bits == 32:
            r -= 1 << 32
        return r

    def next_int(self, bound: int = None) -> int:
        if bound is None:
            return self.next(32)
        if bound & -bound == bound:
            return (bound * self.next(31)) >> 31
        while True:
            bits = self.next(31)
            val = bits % bound
            if ((bits - val + (bound - 1)) & 0xFFFFFFFF) < 0x80000000:
                return val

    def next_float(self) -> float:
        return self.next(24) / float(1 << 24)


def jrandom_ints(seed: int, n: int, bound: int = 0) -> np.ndarray:
    out = np.zeros(n, np.int32)
    lib().jrandom_ints(seed, n, bound, _ptr(out, ctypes.c_int32))
    return out


def jrandom_floats(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float32)
    lib().jrandom_floats(seed, n, _ptr(out, ctypes.c_float))
    return out


def bindings_input(seed: int, n: int, alphabet: str = "protein") -> bytes:
    """BindingsTest.generateInput(seed, n, alphabet) (BindingsTest.java:29-46)."""
    cap = n + 1024
    out = np.zeros(cap, np.uint8)
    m = lib().bindings_generate_input(seed, n, ALPHABETS[alphabet], _ptr(out, ctypes.c_uint8), cap)
    if m < 0:
        raise ValueError("buffer too small")
    return out[:m].tobytes()


def bindings_compare_case(seed: int, n: int, overlap: float):
    """BindingsTest.testCompareVector input generation (BindingsTest.java:159-196).

    Returns (left_keys int32, left_values, right_keys int32, right_values, has_min_value).
    """
    lk = np.zeros(2 * n + 1, np.int32)
    rk = np.zeros(2 * n + 1, np.int32)
    lv = np.zeros(2 * n + 1, np.float32)
    rv = np.zeros(2 * n + 1, np.float32)
    sizes = np.zeros(2, np.int32)
    mv = lib().bindings_compare_case(seed, n, overlap, _ptr(lk, ctypes.c_int32),
                                     _ptr(lv, ctypes.c_float), _ptr(rk, ctypes.c_int32),
                                     _ptr(rv, ctypes.c_float), _ptr(sizes, ctypes.c_int32))
    ls, rs = int(sizes[0]), int(sizes[1])
    return lk[:ls].copy(), lv[:ls].copy(), rk[:rs].copy(), rv[:rs].copy(), bool(mv)
