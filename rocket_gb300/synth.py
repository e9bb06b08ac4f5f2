"""Seeded synthetic proteome workloads (no real proteome files are available).

Each workload is a set of proteomes related by a random binary tree (see
csrc/synth.c): 20-letter amino-acid background (table in synth.c, per mille:
A 83, R 55, N 41, D 55, C 14, Q 39, E 67, G 71, H 23, I 59, L 99, K 58, M 24,
F 39, P 47, S 65, T 53, W 11, Y 29, V 68), protein lengths lognormal with
median 300 and sigma 0.5, per-site substitutions on every branch, no indels.

Workloads (names describe what they are):

* ``cpu16``      16 proteomes x 1,500 proteins, seed 0, branch rate 0.05
* ``uniform256`` 256 proteomes x 1,500 proteins, seed 1, branch rate U(0.01, 0.2)
* ``uneven1024`` 1,024 proteomes, seed 2, protein counts lognormal (median 1,900,
                 sigma 0.9) clipped to [300, 12,000], branch rate U(0.01, 0.2)
* ``sweep512``   512 proteomes, seed 3, sizes as uneven1024 (run at K = 5, 6, 7)
* ``serve2048``  2,048 database proteomes + arriving queries, seed 4, sizes as
                 uneven1024
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import build as _build

_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.SYNTH_LIB):
            _build.build_synth()
        L = ctypes.CDLL(_build.SYNTH_LIB)
        i64p = ctypes.POINTER(ctypes.c_int64)
        L.synth_protein_lengths.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_double,
                                            ctypes.c_double, i64p]
        L.synth_lognormal_counts.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_double,
                                             ctypes.c_double, ctypes.c_int64, ctypes.c_int64, i64p]
        L.synth_proteomes.argtypes = [ctypes.c_uint64, ctypes.c_int, i64p, i64p, ctypes.c_int64,
                                      ctypes.c_double, ctypes.c_double,
                                      ctypes.POINTER(ctypes.c_uint8), i64p]
        L.synth_proteomes.restype = ctypes.c_int
        _lib = L
    return _lib


def _p64(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


@dataclass
class Proteomes:
    """Concatenated ReadFasta-format residue streams of n proteomes."""
    data: np.ndarray               # uint8, all proteomes back to back
    offsets: np.ndarray            # int64 [n + 1]
    protein_counts: np.ndarray     # int64 [n]
    name: str = ""
    meta: dict = field(default_factory=dict)

    def __len__(self):
        return len(self.offsets) - 1

    def get(self, i: int) -> bytes:
        return self.data[self.offsets[i]:self.offsets[i + 1]].tobytes()

    def lengths(self) -> np.ndarray:
        return np.diff(self.offsets)

    def subset(self, idx) -> "Proteomes":
        idx = np.asarray(idx, np.int64)
        parts = [self.data[self.offsets[i]:self.offsets[i + 1]] for i in idx]
        lens = np.array([len(p) for p in parts], np.int64)
        off = np.zeros(len(idx) + 1, np.int64)
        np.cumsum(lens, out=off[1:])
        data = np.concatenate(parts) if parts else np.zeros(0, np.uint8)
        return Proteomes(data, off, self.protein_counts[idx], self.name, dict(self.meta))


def generate(n: int, seed: int, counts, rate_lo: float, rate_hi: float,
             median_len: float = 300.0, sigma_len: float = 0.5, name: str = "") -> Proteomes:
    L = _load()
    counts = np.ascontiguousarray(counts, np.int64)
    assert len(counts) == n and n >= 1
    maxp = int(counts.max())
    plen = np.zeros(maxp, np.int64)
    L.synth_protein_lengths(seed, maxp, median_len, sigma_len, _p64(plen))
    cum = np.zeros(maxp + 1, np.int64)
    np.cumsum(plen, out=cum[1:])
    leaf_bytes = counts + cum[counts]
    off = np.zeros(n + 1, np.int64)
    np.cumsum(leaf_bytes, out=off[1:])
    data = np.zeros(int(off[-1]), np.uint8)
    rc = L.synth_proteomes(seed, n, _p64(counts), _p64(plen), maxp, rate_lo, rate_hi,
                           data.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _p64(off))
    if rc != 0:
        raise MemoryError("synth_proteomes failed")
    return Proteomes(data, off, counts, name,
                     dict(seed=seed, rate=(rate_lo, rate_hi), median_len=median_len,
                          sigma_len=sigma_len))


def uneven_counts(n: int, seed: int, median: float = 1900.0, sigma: float = 0.9,
                  lo: int = 300, hi: int = 12000) -> np.ndarray:
    out = np.zeros(n, np.int64)
    _load().synth_lognormal_counts(seed, n, median, sigma, lo, hi, _p64(out))
    return out


WORKLOADS = {
    "cpu16": dict(n=16, seed=0, uneven=False, proteins=1500, rate=(0.05, 0.05), k=6),
    "uniform256": dict(n=256, seed=1, uneven=False, proteins=1500, rate=(0.01, 0.2), k=6),
    "uneven1024": dict(n=1024, seed=2, uneven=True, rate=(0.01, 0.2), k=6),
    "sweep512": dict(n=512, seed=3, uneven=True, rate=(0.01, 0.2), k=6),
    "serve2048": dict(n=2048, seed=4, uneven=True, rate=(0.01, 0.2), k=6),
}


def workload(name: str, n: Optional[int] = None, scale: float = 1.0, extra: int = 0) -> Proteomes:
    """Generates a named workload.  ``n`` takes the first n proteomes' sizes
    (for smaller test cases of the same distribution); ``scale`` multiplies the
    protein counts; ``extra`` appends more leaves of the same tree (serving
    queries)."""
    w = WORKLOADS[name]
    total = (n if n is not None else w["n"]) + extra
    if w["uneven"]:
        counts = uneven_counts(total, w["seed"])
    else:
        counts = np.full(total, w["proteins"], np.int64)
    if scale != 1.0:
        counts = np.maximum(1, np.round(counts * scale)).astype(np.int64)
    return generate(total, w["seed"], counts, w["rate"][0], w["rate"][1], name=name)
