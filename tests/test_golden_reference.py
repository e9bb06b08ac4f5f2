"""The oracle against golden vectors of the reference's own library (CPU).

tests/golden/reference_vectors.npz holds what the reference's CUDA file
(phylogenetics/src/main/cpp/native.cu, compiled unmodified for the GB300) returned
through its C ABI for BindingsTest's build and compare inputs and for small edge
cases (made by tests/golden/make_reference_golden.py on a GB300).  The oracle's
restatement of the rule must give the same vector sizes and keys, values within 1
float ulp (the reference sums its norm in CUB's order, the oracle exactly), and C
within 1e-12 of the reference's compare.
"""
import importlib.util
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "reference_vectors.npz")


def _generator():
    spec = importlib.util.spec_from_file_location(
        "make_reference_golden", os.path.join(HERE, "golden", "make_reference_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def gold():
    if not os.path.exists(GOLD):
        pytest.skip("golden vectors not generated")
    g = np.load(GOLD)
    meta = g["meta"]
    starts = np.concatenate([[0], np.cumsum(meta[:, 4])])
    deltas = g["key_deltas"].astype(np.uint64)
    keys = []
    for a, b in zip(starts[:-1], starts[1:]):
        keys.append(np.cumsum(deltas[a:b]).astype(np.uint32))
    vals = [g["values"][a:b] for a, b in zip(starts[:-1], starts[1:])]
    return dict(meta=meta, keys=keys, vals=vals, cmp_meta=g["cmp_meta"], cmp_c=g["cmp_c"])


def _ulps(a, b):
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return int(np.max(np.abs(ia - ib))) if len(a) else 0


def test_builds_match_the_reference(gold):
    gen = _generator()
    meta = gold["meta"]
    assert len(meta) == len(gen.SWEEP) + len(gen.LITERALS)
    differ = 0
    empty = 0
    for row, keys, vals in zip(meta, gold["keys"], gold["vals"]):
        alpha, k, n, lit, size = (int(x) for x in row)
        alphabet = "protein" if alpha == 0 else "DNA"
        if lit >= 0:
            a2, k2, seq = gen.LITERALS[lit]
            assert (a2, k2) == (alphabet, k)
        else:
            seq = O.bindings_input(0, n, alphabet)
        r = O.cv_native(seq, k, alphabet)
        assert len(r["keys"]) == size, (alphabet, k, n, lit)
        assert np.array_equal(r["keys"], keys), (alphabet, k, n, lit)
        assert _ulps(r["values"].astype(np.float32), vals.astype(np.float32)) <= 1
        differ += int(np.count_nonzero(r["values"].view(np.uint32) != vals.view(np.uint32)))
        empty += size == 0
    assert empty >= 4  # the empty input, the short ones, the homopolymers
    total = int(meta[:, 4].sum())
    assert total > 40000 and differ <= total // 1000


def test_compares_match_the_reference(gold):
    assert len(gold["cmp_c"]) >= 40
    for (seed, n, ratio), c_ref in zip(gold["cmp_meta"], gold["cmp_c"]):
        lk, lv, rk, rv, _ = O.bindings_compare_case(int(seed), int(n), float(ratio))
        c = O.compare_fp64(lk.view(np.uint32), lv, rk.view(np.uint32), rv)
        assert abs(c - c_ref) <= 1e-12 * max(1.0, abs(c_ref)), (seed, n, ratio, c, c_ref)
