"""This project's library against the reference's own library on the same inputs.

The reference's CUDA file (phylogenetics/src/main/cpp/native.cu) is compiled
unmodified for sm_103a (``make -C oracle ref``) and driven through its C ABI beside
ours, on the same device buffers:

* builds (native.cu:258-477 vs buildCompositionVector here): sizes, keys and the
  padding bit-identical; values within 1 float ulp (both normalise by
  float(alpha) / sqrt(norm), but the reference sums the norm in CUB's order and
  this library exactly);
* compares (native.cu:645-703 vs compareCompositionVectors here): C within 1e-12
  relative on identical inputs.  The sizes at which the reference's compare may
  race with itself (ceil((nl + nr) / 256) a multiple of 32, native.cu:660-675) are
  left out and counted.

Inputs: the build sweep of BindingsTest.testBuildVectors (BindingsTest.java:79-119,
disabled in the reference, run here against the reference's GPU build) for protein
K = 3..7 and DNA K = 3..10; full-size synthetic proteomes at K = 5, 6, 7; the
compare sweep of BindingsTest.testCompareVectors (:159-213); pairs of full-size
vectors.

Skipped only where the reference's source was never staged; once it is staged,
a missing library is a failure.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rocket_gb300 import synth
from rocket_gb300.bindings import Bindings

import refabi
from gpu_helpers import to_device_bytes, ulp_diff

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    if not refabi.staged():
        pytest.skip("the reference's native.cu was not staged (make -C oracle stage-ref)")
    return refabi.load()


class Pair:
    """One device input and two output buffers, scratch for both libraries."""

    def __init__(self):
        self.scratch = {}

    def ref_scratch(self, alphabet, k, max_size):
        need = refabi.scratch_bytes(alphabet, k, max_size)
        key = ("ref", alphabet, k)
        if key not in self.scratch or self.scratch[key].numel() < need:
            self.scratch.pop(key, None)
            self.scratch[key] = torch.empty(need, dtype=torch.uint8, device="cuda")
        return self.scratch[key]

    def our_scratch(self, alphabet, k, max_size):
        need = Bindings.INSTANCE.estimateScratchMemory(alphabet, k, max_size)
        key = ("ours", alphabet, k)
        if key not in self.scratch or self.scratch[key].numel() < need:
            self.scratch.pop(key, None)
            self.scratch[key] = torch.empty(need, dtype=torch.uint8, device="cuda")
        return self.scratch[key]


@pytest.fixture(scope="module")
def bufs():
    b = Pair()
    yield b
    b.scratch.clear()
    torch.cuda.empty_cache()


def build_both(bufs, seq: bytes, k: int, alphabet: str, max_size: int):
    st = torch.cuda.current_stream().cuda_stream
    d_in = to_device_bytes(seq)
    out = []
    for who in ("ref", "ours"):
        keys = torch.full((max_size,), 0x1234, dtype=torch.int32, device="cuda")
        vals = torch.full((max_size,), 7.0, dtype=torch.float32, device="cuda")
        size = np.zeros(1, np.int32)
        if who == "ref":
            scr = bufs.ref_scratch(alphabet, k, max_size)
            rc = refabi.build(st, scr, alphabet, k, d_in, len(seq), keys, vals, size, max_size)
        else:
            scr = bufs.our_scratch(alphabet, k, max_size)
            rc = Bindings.INSTANCE.buildCompositionVector(
                st, scr.data_ptr(), scr.numel(), alphabet, k, d_in.data_ptr(), len(seq),
                keys.data_ptr(), vals.data_ptr(), size, max_size)
        torch.cuda.synchronize()
        assert rc == 0, (who, rc)
        out.append((int(size[0]), keys.cpu().numpy().view(np.uint32), vals.cpu().numpy()))
    return out


def assert_same_vector(r, o):
    (nr, kr, vr), (no, ko, vo) = r, o
    assert nr == no
    assert np.array_equal(kr, ko)                      # keys and padding keys
    assert np.array_equal(vr[nr:], vo[no:])            # padding values
    assert ulp_diff(vr[:nr], vo[:no]) <= 1
    return int(np.count_nonzero(vr[:nr].view(np.uint32) != vo[:no].view(np.uint32)))


@pytest.mark.parametrize("alphabet,k", [("protein", k) for k in range(3, 8)] +
                         [("DNA", k) for k in range(3, 11)])
def test_build_bindings_sweep(ref, bufs, alphabet, k):
    """BindingsTest.testBuildVector's inputs and max size (1000 n, :79-97)."""
    differ = 0
    total = 0
    for n in (10, 100, 1000, 10000):
        for seed in range(5):
            seq = O.bindings_input(seed, n, alphabet)
            r, o = build_both(bufs, seq, k, alphabet, 1000 * n)
            differ += assert_same_vector(r, o)
            total += r[0]
    assert total > 0
    # values that differ by one ulp come from the norm's last bits only
    assert differ <= max(8, total // 1000), (differ, total)


@pytest.mark.parametrize("k", [5, 6, 7])
def test_build_full_size_proteomes(ref, bufs, k):
    """Full-size synthetic proteomes: four of 1,500 proteins, the largest and the
    smallest of the uneven set (12,000 and 300 proteins)."""
    uni = synth.workload("uniform256", n=4)
    ends = synth.generate(2, 2, [12000, 300], 0.01, 0.2)  # the uneven sizes' clip bounds
    seqs = [uni.get(i) for i in range(4)] + [ends.get(0), ends.get(1)]
    for s in seqs:
        max_size = min(21 ** k, 8 * len(s) + 4096)
        r, o = build_both(bufs, s, k, "protein", max_size)
        assert r[0] > 1000
        assert_same_vector(r, o)


def test_build_zero_alpha_cases(ref, bufs):
    """Inputs in which a seen K-mer's alpha is exactly 0 (dropped by both), and a
    homopolymer whose vector is empty: the same sizes, keys and values as the
    reference build."""
    from test_gpu_build import ZERO_ALPHA_CASES
    cases = list(ZERO_ALPHA_CASES) + [("protein", 5, b"Q" * 50), ("DNA", 8, b"C" * 50)]
    sizes = []
    for alphabet, k, seq in cases:
        r, o = build_both(bufs, seq, k, alphabet, 64)
        assert_same_vector(r, o)
        sizes.append(r[0])
    assert sizes[-1] == 0 and sizes[-2] == 0 and min(sizes[:-2]) > 0


def compare_both(bufs, lk, lv, rk, rv):
    st = torch.cuda.current_stream().cuda_stream
    n = max(len(lk), len(rk), 1)
    t = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (lk, lv, rk, rv)]
    res = []
    for who in ("ref", "ours"):
        d_out = torch.full((1,), -5.0, dtype=torch.float64, device="cuda")
        if who == "ref":
            scr = bufs.ref_scratch("DNA", 3, n)  # BindingsTest.compareVectorGPU's context (:134)
            rc = refabi.compare(st, scr, t[0], t[1], len(lk), t[2], t[3], len(rk), d_out)
        else:
            scr = bufs.our_scratch("DNA", 3, n)
            rc = Bindings.INSTANCE.compareCompositionVectors(
                st, scr.data_ptr(), scr.numel(), t[0].data_ptr(), t[1].data_ptr(), len(lk),
                t[2].data_ptr(), t[3].data_ptr(), len(rk), d_out.data_ptr())
        torch.cuda.synchronize()
        assert rc == 0, (who, rc)
        res.append(float(d_out.item()))
    return res


def test_compare_bindings_sweep(ref, bufs):
    """BindingsTest.testCompareVectors (:204-213): n x overlap ratio x seed."""
    raced = []
    checked = 0
    for n in (10, 100, 1000, 10000, 100000):
        for ratio in (0.0, 0.5, 1.0):
            for seed in range(4):
                lk, lv, rk, rv, _ = O.bindings_compare_case(seed, n, ratio)
                if refabi.compare_block_race(len(lk), len(rk)):
                    raced.append((n, ratio, seed, len(lk), len(rk)))
                    continue
                c_ref, c_ours = compare_both(bufs, lk, lv, rk, rv)
                assert abs(c_ref - c_ours) <= 1e-12 * max(1.0, abs(c_ref)), (n, ratio, seed)
                checked += 1
    assert checked >= 50
    assert len(raced) <= 6, raced


def test_compare_full_size_vectors(ref, bufs):
    """Pairs of full-size K = 6 vectors built by the reference, compared by both."""
    uni = synth.workload("uniform256", n=5)
    vecs = []
    for i in range(5):
        s = uni.get(i)
        max_size = 8 * len(s) + 4096
        (n, k, v), _ = build_both(bufs, s, 6, "protein", max_size)
        vecs.append((k[:n].view(np.int32).copy(), v[:n].copy()))
    checked = 0
    for i in range(5):
        for j in range(i, 5):
            lk, lv = vecs[i]
            rk, rv = vecs[j]
            if refabi.compare_block_race(len(lk), len(rk)):
                continue
            c_ref, c_ours = compare_both(bufs, lk, lv, rk, rv)
            assert abs(c_ref - c_ours) <= 1e-12 * max(1.0, abs(c_ref)), (i, j, c_ref, c_ours)
            exact = O.compare_fp64(lk.view(np.uint32), lv, rk.view(np.uint32), rv)
            assert abs(c_ours - exact) <= 1e-12
            checked += 1
    assert checked >= 10


def test_plain_path_timing_against_the_reference(ref, bufs):
    """The reference's own library and this one, timed on the same GB300 through the
    same synchronous calls (the plain per-proteome / per-pair path Rocket drives):
    buildCompositionVector on a full-size proteome (1,500 proteins, K = 6) and
    compareCompositionVectors on two of its vectors.  Prints both; this library must
    not be slower."""
    import time
    uni = synth.workload("uniform256", n=2)
    seqs = [uni.get(0), uni.get(1)]
    st = torch.cuda.current_stream().cuda_stream
    max_size = 8 * max(len(s) for s in seqs) + 4096
    d_in = [to_device_bytes(s) for s in seqs]
    keys = [torch.empty(max_size, dtype=torch.int32, device="cuda") for _ in range(4)]
    vals = [torch.empty(max_size, dtype=torch.float32, device="cuda") for _ in range(4)]
    size = np.zeros(1, np.int32)
    rs = bufs.ref_scratch("protein", 6, max_size)
    os_ = bufs.our_scratch("protein", 6, max_size)

    def build(who, i, slot):
        if who == "ref":
            rc = refabi.build(st, rs, "protein", 6, d_in[i], len(seqs[i]), keys[slot],
                              vals[slot], size, max_size)
        else:
            rc = Bindings.INSTANCE.buildCompositionVector(
                st, os_.data_ptr(), os_.numel(), "protein", 6, d_in[i].data_ptr(), len(seqs[i]),
                keys[slot].data_ptr(), vals[slot].data_ptr(), size, max_size)
        assert rc == 0
        return int(size[0])

    n = {}
    for who, base in (("ref", 0), ("ours", 2)):
        for i in range(2):
            n[(who, i)] = build(who, i, base + i)
    t = {}
    for who, base in (("ref", 0), ("ours", 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            build(who, 0, base)
        t[("build", who)] = (time.perf_counter() - t0) / 5
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for who, base in (("ref", 0), ("ours", 2)):
        nl, nr = n[(who, 0)], n[(who, 1)]
        if who == "ref" and refabi.compare_block_race(nl, nr):
            pytest.skip("these sizes race in the reference's compare")
        args = (keys[base], vals[base], nl, keys[base + 1], vals[base + 1], nr)
        for rep in range(21):
            if rep == 1:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
            if who == "ref":
                rc = refabi.compare(st, rs, args[0], args[1], nl, args[3], args[4], nr, out)
            else:
                rc = Bindings.INSTANCE.compareCompositionVectors(
                    st, os_.data_ptr(), os_.numel(), args[0].data_ptr(), args[1].data_ptr(), nl,
                    args[3].data_ptr(), args[4].data_ptr(), nr, out.data_ptr())
            assert rc == 0
        t[("compare", who)] = (time.perf_counter() - t0) / 20
    print(f"\nplain path on this GPU, {n[('ours', 0)]:,} + {n[('ours', 1)]:,} entries: "
          f"build {1000 * t[('build', 'ref')]:.2f} ms (reference) vs "
          f"{1000 * t[('build', 'ours')]:.2f} ms; compare {1000 * t[('compare', 'ref')]:.3f} ms "
          f"(reference) vs {1000 * t[('compare', 'ours')]:.3f} ms")
    assert t[("build", "ours")] <= t[("build", "ref")]
    assert t[("compare", "ours")] <= t[("compare", "ref")]
