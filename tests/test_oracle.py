"""Pins the CPU oracle (oracle/) before it is trusted as the checker.

The reference's own tests hold no golden vectors (BindingsTest.java computes
its expectations at run time and its build test is disabled, :102), so the
oracle is pinned by:
  * java.util.Random outputs published in Java's documentation and widely
    reproduced, and agreement of the C clone with a pure-Python clone;
  * hand-derived known answers of the Markov rule of native.cu:350-400;
  * agreement of two independent formulations of the rule (every dense slot,
    as native.cu loops, versus candidate enumeration);
  * the relation to the Java CPU path (CompositionVectorKernels.java:91-222).
"""
import math

import numpy as np
import pytest

from oracle import oracle as O


# ---------------------------------------------------------------- java.util.Random

def test_java_random_known_values():
    # new Random(0).nextInt() x2 and new Random(42).nextInt(): published values
    assert list(O.jrandom_ints(0, 2)) == [-1155484576, -723955400]
    assert O.jrandom_ints(42, 1)[0] == -1170105035
    # new Random(0).nextFloat() == 0.73096776f
    assert abs(float(O.jrandom_floats(0, 1)[0]) - 0.73096776) < 1e-7


@pytest.mark.parametrize("seed", [0, 1, 7, 123456789, -5])
@pytest.mark.parametrize("bound", [0, 2, 21, 500, 1000, 7])
def test_java_random_c_matches_python(seed, bound):
    n = 2000
    c = O.jrandom_ints(seed, n, bound)
    r = O.JavaRandom(seed)
    py = [r.next_int(bound) if bound else r.next_int() for _ in range(n)]
    assert list(c) == py
    f = O.jrandom_floats(seed, 100)
    r = O.JavaRandom(seed)
    assert np.array_equal(f, np.array([r.next_float() for _ in range(100)], np.float32))


def test_bindings_generate_input_format():
    s = O.bindings_input(0, 5000)
    assert len(s) >= 5000
    # proteins are separated by the text "10" (StringBuilder.append((byte) '\n'))
    assert b"10" in s and b"\n" not in s
    letters = set(b"ACDEFGHIKLMNPQRSTVWYX10")
    assert set(s) <= letters
    d = O.bindings_input(3, 2000, "DNA")
    assert set(d) <= set(b"ACGT10")


@pytest.mark.parametrize("n", [10, 100, 1000, 10000])
@pytest.mark.parametrize("ratio", [0.0, 0.5, 1.0])
def test_bindings_compare_case(n, ratio):
    for seed in range(4):
        lk, lv, rk, rv, minval = O.bindings_compare_case(seed, n, ratio)
        assert not minval
        assert n <= len(lk) < 2 * n and n <= len(rk) < 2 * n
        assert np.all(np.diff(lk) > 0) and np.all(np.diff(rk) > 0)
        shared = len(np.intersect1d(lk, rk))
        assert shared == math.ceil(ratio * n)
        assert np.all((lv >= 0) & (lv < 1))


# ---------------------------------------------------------------- Markov rule KATs

def _alpha(full, prefix, suffix, middle, n0, n1, n2):
    p = full / n0 if n0 else float("nan")
    p0 = ((prefix / n1) * (suffix / n1)) / (middle / n2)
    return np.float32((p - p0) / p0)


def test_kat_acaca_k3():
    # "ACACA", K=3: 1-mers A3 C2 (n2=5); 2-mers AC2 CA2 (n1=4); 3-mers ACA2 CAC1 (n0=3).
    # Candidates ACA (prefix AC, suffix CA) and CAC.  alpha(ACA) = (2/3 - 5/8)/(5/8) = 1/15,
    # alpha(CAC) = (1/3 - 5/12)/(5/12) = -1/5; normalised: (1, -3)/sqrt(10).
    r = O.cv_native(b"ACACA", 3)
    assert list(r["keys"]) == [21, 442]  # A=0, C=1: 0*441+1*21+0, 1*441+0*21+1
    assert (r["n0"], r["n1"], r["n2"]) == (3, 4, 5)
    assert list(r["c0"]) == [2, 1] and list(r["c2m"]) == [2, 3]
    assert r["alpha"][0] == _alpha(2, 2, 2, 2, 3, 4, 5) and abs(r["alpha"][0] - 1 / 15) < 1e-7
    assert r["alpha"][1] == np.float32(-0.2)
    assert np.allclose(r["values"], [1 / math.sqrt(10), -3 / math.sqrt(10)], atol=1e-6)


def test_kat_homopolymer_is_empty():
    # "AAAAA", K=3: p = 3/3 = 1 and p0 = (4/4 * 4/4) / (5/5) = 1 -> alpha == 0 exactly,
    # the only candidate is dropped (native.cu:408 keeps bits != 0).
    r = O.cv_native(b"AAAAA", 3)
    assert len(r["keys"]) == 0 and r["candidates"] == 1


@pytest.mark.parametrize("alphabet,k,seq", [
    ("DNA", 3, b"T\nCGC"), ("DNA", 5, b"CACAC\nAAA"), ("DNA", 7, b"TTCTCGA\nTTTTTTT"),
    ("protein", 3, b"AII\nRRR"), ("protein", 5, b"PPPP\nHHHHHM"), ("protein", 6, b"RRRRRR\nMLVITL"),
    ("protein", 3, b"RRRRRRRRRYYYYY\nSSSS")])
def test_kat_alpha_zero_is_dropped(alphabet, k, seq):
    """A seen K-mer whose alpha is exactly 0 (p == p0: a homopolymer protein of K
    residues beside another protein) is dropped (native.cu:402-458): the vector
    holds one entry fewer than the candidates, in both formulations of the rule."""
    a = O.cv_native(seq, k, alphabet, formulation="slots", with_values=False)
    b = O.cv_native(seq, k, alphabet, with_values=False)
    assert np.array_equal(a["keys"], b["keys"])
    assert np.array_equal(a["alpha"].view(np.uint32), b["alpha"].view(np.uint32))
    assert 0 < len(b["keys"]) == b["candidates"] - 1
    assert np.all(b["alpha"] != 0)


def test_kat_unseen_kmers_minus_one():
    # "ACA\nCC", K=3: n0=1 (ACA), n1=3 (AC, CA, CC), n2=5 (A A C C C -> A2 C3).
    # Candidates ACA ACC CAC CCA CCC; only ACA was seen:
    # alpha(ACA) = (1 - 5/27) / (5/27) = 22/5; the others (0 - p0)/p0 = -1.
    r = O.cv_native(b"ACA\nCC", 3)
    assert list(r["keys"]) == [21, 22, 442, 462, 463]
    assert r["alpha"][0] == np.float32(4.4)
    assert list(r["alpha"][1:]) == [-1.0, -1.0, -1.0, -1.0]
    norm = float(np.float32(4.4) * np.float32(4.4)) + 4.0
    assert r["norm"] == norm
    assert r["values"][1] == np.float32(-1.0 / math.sqrt(norm))


def test_kat_no_full_windows_gives_nan():
    # "AC\nCA", K=3: no 3-window (n0 = 0): p = 0/0 -> NaN alpha, kept (bits != 0).
    r = O.cv_native(b"AC\nCA", 3)
    assert list(r["keys"]) == [21, 442]
    assert np.all(np.isnan(r["alpha"])) and np.all(np.isnan(r["values"]))


def test_kat_invalid_letters_break_windows():
    # B, J, O, U, Z and lower case are not in the protein alphabet (native.cu:96-123)
    for bad in b"BJOUZa1\n":
        s = b"ACDE" + bytes([bad]) + b"FGHI"
        k1, k2, tot = O.count_tables(s, 4)
        assert tot == (2, 4, 6), (chr(bad), tot)  # 4-windows: ACDE, FGHI


def test_x_is_a_letter_and_y_is_19():
    r = O.cv_native(b"XYXYX", 3)
    # X = 20, Y = 19: XYX = 20*441 + 19*21 + 20
    assert 20 * 441 + 19 * 21 + 20 in set(r["keys"].tolist())


# ---------------------------------------------------------------- formulations agree

@pytest.mark.parametrize("k", [3, 4, 5, 6])
def test_slot_loop_equals_candidates_protein(k):
    for seed in range(3):
        s = O.bindings_input(seed, 20000)
        a = O.cv_native(s, k, formulation="slots", with_values=False)
        b = O.cv_native(s, k, with_values=False)
        assert np.array_equal(a["keys"], b["keys"])
        assert np.array_equal(a["alpha"].view(np.uint32), b["alpha"].view(np.uint32))
        for f in ("c0", "c1p", "c1s", "c2m"):
            assert np.array_equal(a[f], b[f])


@pytest.mark.parametrize("k", [3, 5, 7, 9, 10])
def test_slot_loop_equals_candidates_dna(k):
    s = O.bindings_input(1, 20000, "DNA")
    a = O.cv_native(s, k, "DNA", formulation="slots", with_values=False)
    b = O.cv_native(s, k, "DNA", with_values=False)
    assert np.array_equal(a["keys"], b["keys"])
    assert np.array_equal(a["alpha"].view(np.uint32), b["alpha"].view(np.uint32))


@pytest.mark.parametrize("k", [4, 5, 6])
def test_count_tables_match_enumeration(k):
    s = O.bindings_input(2, 30000)
    k1, k2, tot = O.count_tables(s, k)
    r = O.cv_native(s, k, with_values=False)
    assert (r["n0"], r["n1"], r["n2"]) == tot
    assert tot[1] == int(k1.sum()) and tot[2] == int(k2.sum())


# ---------------------------------------------------------------- relation to the Java CPU path

@pytest.mark.parametrize("k", [3, 4, 5, 6])
def test_java_cpu_path_matches_rule(k):
    s = O.bindings_input(4, 20000)
    jk, jv = O.java_build(s, k)
    r = O.cv_native(s, k)
    # Java keeps alpha == 0 slots (p0 != 0 test only), the device rule drops them
    assert set(r["keys"].tolist()) <= set(jk.tolist())
    assert len(jk) - len(r["keys"]) <= r["candidates"] - len(r["keys"])
    idx = np.searchsorted(jk, r["keys"])
    # float probabilities vs double: values agree to float precision
    assert np.max(np.abs(jv[idx] - r["values"])) < 1e-5


def test_compare_oracles_agree():
    for n, ratio in [(1000, 0.5), (10000, 1.0), (10000, 0.0)]:
        lk, lv, rk, rv, _ = O.bindings_compare_case(1, n, ratio)
        j = O.java_compare(lk, lv, rk, rv)
        f = O.compare_fp64(lk.view(np.uint32), lv, rk.view(np.uint32), rv)
        # Java multiplies in float; the FP64 oracle multiplies exactly
        assert abs(j - f) <= 1e-6 * max(1.0, abs(f))
        if ratio == 0.0:
            assert f == 0.0


def test_fp64_oracle_exact_on_dyadic_values():
    keys = np.arange(0, 4000, 2, dtype=np.uint32)
    a = np.full(len(keys), 0.5, np.float32)
    b = np.full(len(keys), 0.25, np.float32)
    assert O.compare_fp64(keys, a, keys, b) == len(keys) * 0.125
