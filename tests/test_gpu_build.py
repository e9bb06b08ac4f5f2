"""Composition-vector construction on the device vs the oracle's restatement of
native.cu's rule: keys and counts bit-exact, values within 1 ulp (the norm is an
exactly rounded sum on both sides, so they are normally identical)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rocket_gb300 import _native, synth
from rocket_gb300.engine import BatchBuilder

from gpu_helpers import build_gpu, ulp_diff, to_device_bytes

pytestmark = pytest.mark.gpu


def check_against_oracle(seq, k, alphabet="protein", max_size=None):
    n, keys, vals = build_gpu(seq, k, alphabet, max_size)
    r = O.cv_native(seq, k, alphabet)
    assert n == len(r["keys"])
    assert np.array_equal(keys[:n], r["keys"])
    assert ulp_diff(vals[:n], r["values"]) <= 1
    # padding (native.cu:473-474)
    assert np.all(keys[n:] == 0xFFFFFFFF) and np.all(vals[n:] == 0)
    return n


@pytest.mark.parametrize("seq,k,expect", [
    (b"ACACA", 3, 2), (b"AAAAA", 3, 0), (b"ACA\nCC", 3, 5), (b"AC\nCA", 3, 2),
    (b"", 3, 0), (b"A", 3, 0), (b"AC", 3, 0), (b"ACDEFGHIKLMNPQRSTVWYX", 6, None),
    (b"ACDE\nFGHI", 4, None), (b"XYXYX", 3, None),
])
def test_known_answers(seq, k, expect):
    n = check_against_oracle(seq, k)
    if expect is not None:
        assert n == expect


# Inputs in which a seen K-mer has alpha exactly 0 (p == p0 in the reference's
# double arithmetic, native.cu:387-394): a homopolymer protein of K residues, whose
# one K-mer has full, prefix, suffix and middle counts proportional to the window
# totals, beside a protein whose K-mer survives.  Found by a seeded search over
# small inputs with the oracle (a seen candidate missing from the output); the
# rule drops alpha-0 slots (native.cu:402-458), so these vectors hold fewer
# entries than candidates.
ZERO_ALPHA_CASES = [
    ("DNA", 3, b"T\nCGC"), ("DNA", 4, b"TTTT\nCGTG"), ("DNA", 5, b"CACAC\nAAA"),
    ("DNA", 6, b"CAATAG\nGGGGGG"), ("DNA", 7, b"TTCTCGA\nTTTTTTT"),
    ("protein", 3, b"AII\nRRR"), ("protein", 4, b"ALCP\nEEEE"), ("protein", 5, b"PPPP\nHHHHHM"),
    ("protein", 6, b"RRRRRR\nMLVITL"), ("protein", 3, b"RRRRRRRRRYYYYY\nSSSS"),
]


@pytest.mark.parametrize("alphabet,k,seq", ZERO_ALPHA_CASES)
def test_zero_alpha_dropped(alphabet, k, seq):
    r = O.cv_native(seq, k, alphabet, with_values=False)
    assert 0 < len(r["keys"]) < r["candidates"]  # a seen candidate is dropped
    assert check_against_oracle(seq, k, alphabet) == len(r["keys"])


@pytest.mark.parametrize("alphabet,k", [("protein", 6), ("protein", 4), ("protein", 3),
                                        ("DNA", 5)])
def test_zero_alpha_batched(alphabet, k):
    """The same inputs inside a build batch (protein K = 6: compact (K-1)-mer tables),
    with a homopolymer proteome (no surviving entry at all) and normal proteomes: every
    vector against the oracle, and every pair and self product through the pair engine."""
    from rocket_gb300.engine import PairEngine
    p = synth.workload("uneven1024", n=2, scale=0.02)
    cases = [s for a, kk, s in ZERO_ALPHA_CASES if a == alphabet and kk == k]
    if alphabet == "DNA":
        normal = [O.bindings_input(3, 2000, "DNA"), O.bindings_input(4, 500, "DNA")]
        homo = b"G" * 40
    else:
        normal = [p.get(0), p.get(1)]
        homo = b"W" * 40
    seqs = [normal[0]] + cases + [homo, normal[0][:300] + b"K" * 30 + normal[1][:300], normal[1]]
    off = np.zeros(len(seqs) + 1, np.int64)
    np.cumsum([len(x) for x in seqs], out=off[1:])
    data = torch.from_numpy(np.frombuffer(b"".join(seqs), np.uint8).copy()).cuda()
    arena = BatchBuilder(alphabet, k, max_batch=4).build(data, off)
    torch.cuda.synchronize()
    ref = [O.cv_native(x, k, alphabet) for x in seqs]
    assert len(ref[len(cases) + 1]["keys"]) == 0  # the homopolymer keeps nothing
    for i, r in enumerate(ref):
        kk, v = arena.host_vector(i)
        assert np.array_equal(kk, r["keys"]), i
        assert ulp_diff(v, r["values"]) <= 1, i
    eng = PairEngine(arena)
    eng.ensure_index()
    out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
    eng.run(eng.plan_triangle(), out)
    C = out.cpu().numpy()
    for i in range(len(seqs)):
        for j in range(i, len(seqs)):
            c = O.compare_fp64(ref[i]["keys"], ref[i]["values"], ref[j]["keys"], ref[j]["values"])
            assert abs(C[i, j] - c) <= 2e-6, (i, j, C[i, j], c)


@pytest.mark.parametrize("k", [3, 4, 5, 6, 7])
def test_bindings_sweep_protein(k):
    # the sweep of BindingsTest.testBuildVectors (n x seeds, :99-112)
    for n in (10, 100, 1000, 10000):
        for seed in range(5):
            check_against_oracle(O.bindings_input(seed, n), k)


@pytest.mark.parametrize("k", [3, 5, 7, 9])
def test_bindings_sweep_dna(k):
    for n in (10, 100, 1000, 10000):
        for seed in range(5):
            check_against_oracle(O.bindings_input(seed, n, "DNA"), k, "DNA")


def test_dna_k10():
    check_against_oracle(O.bindings_input(9, 50000, "DNA"), 10, "DNA")


@pytest.mark.parametrize("k", [5, 6, 7])
def test_synthetic_proteome(k):
    p = synth.workload("uniform256", n=2, scale=0.2)
    check_against_oracle(p.get(1), k)


def test_batched_build_k7_compact_tables():
    """Protein K = 7: (K-1)-mer tables of 21^6 entries are kept compact (one entry per
    seen (K-1)-mer); two batches, keys and values against the oracle."""
    p = synth.workload("uneven1024", n=5, scale=0.05)
    d = torch.from_numpy(p.data).cuda()
    arena = BatchBuilder("protein", 7, max_batch=3).build(d, p.offsets)
    torch.cuda.synchronize()
    for i in range(5):
        r = O.cv_native(p.get(i), 7)
        k, v = arena.host_vector(i)
        assert np.array_equal(k, r["keys"])
        assert ulp_diff(v, r["values"]) <= 1


def test_full_size_proteome_k6():
    p = synth.workload("uniform256", n=1)
    n = check_against_oracle(p.get(0), 6)
    assert n > 10 ** 6


def test_exact_capacity_and_overflow():
    s = O.bindings_input(2, 3000)
    r = O.cv_native(s, 4)
    n = len(r["keys"])
    assert check_against_oracle(s, 4, max_size=n) == n  # size == max: no padding
    with pytest.raises(_native.CudaException) as e:
        build_gpu(s, 4, max_size=n - 1)
    assert e.value.code == 999


@pytest.mark.parametrize("alphabet,k", [("protein", 2), ("protein", 11), ("protein", 8),
                                        ("rna", 5), ("DNA", 2)])
def test_argument_errors(alphabet, k):
    from rocket_gb300.bindings import Bindings
    d_in = to_device_bytes(b"ACDEFGHIK")
    keys = torch.empty(64, dtype=torch.int32, device="cuda")
    vals = torch.empty(64, dtype=torch.float32, device="cuda")
    scr = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    size = np.zeros(1, np.int32)
    rc = Bindings.INSTANCE.buildCompositionVector(
        torch.cuda.current_stream().cuda_stream, scr.data_ptr(), scr.numel(), alphabet, k,
        d_in.data_ptr(), 9, keys.data_ptr(), vals.data_ptr(), size, 64)
    assert rc == 999


def test_batched_build_equals_single_and_counts():
    p = synth.workload("uneven1024", n=6, scale=0.05)
    d = torch.from_numpy(p.data).cuda()
    b = BatchBuilder("protein", 6, max_batch=4)  # two sub-batches
    arena = b.build(d, p.offsets)
    torch.cuda.synchronize()
    assert arena.n == 6
    for i in range(6):
        r = O.cv_native(p.get(i), 6)
        k, v = arena.host_vector(i)
        assert np.array_equal(k, r["keys"])
        assert ulp_diff(v, r["values"]) <= 1
        assert arena.off[i] % 4 == 0
        assert abs(arena.norms[i] - r["norm"]) <= 1e-12 * r["norm"]
    # count tables of the last plan (proteomes 4, 5; the second batch, on the builder's
    # second scratch when two batches are in flight)
    L = _native.load()
    scr = b._scratch[1] if b.overlap else b._scratch[0]
    k1 = np.zeros(21 ** 5, np.uint32)
    k2 = np.zeros(21 ** 4, np.uint32)
    tot = np.zeros(3, np.uint32)
    cand = int(np.sum(np.minimum(8 * p.lengths()[4:] + 65536, 21 ** 6)))
    _native.check(L.phyloBuildBatchCounts(torch.cuda.current_stream().cuda_stream,
                                          scr.data_ptr(), scr.numel(), b"protein", 6, 2, cand, 1,
                                          k1.ctypes.data, k2.ctypes.data, tot.ctypes.data))
    e1, e2, et = O.count_tables(p.get(5), 6)
    assert np.array_equal(k1, e1) and np.array_equal(k2, e2) and tuple(tot) == et


def test_batched_build_grows_a_small_arena():
    """An arena too small for the build grows while two batches are in flight (each
    growth copies the old buffers on the build's stream, and the next emit may run on
    the side stream): the vectors equal those of a build into a fresh arena."""
    p = synth.workload("uneven1024", n=7, scale=0.03)
    d = torch.from_numpy(p.data).cuda()
    ref = BatchBuilder("protein", 6, max_batch=2).build(d, p.offsets)
    b = BatchBuilder("protein", 6, max_batch=2)  # four batches, two in flight
    small = b.new_arena(64, 7)
    got = b.build(d, p.offsets, arena=small)
    torch.cuda.synchronize()
    assert got.n == ref.n == 7 and got.keys.numel() > 64
    assert np.array_equal(got.off, ref.off) and np.array_equal(got.nnz, ref.nnz)
    for i in range(7):
        k0, v0 = ref.host_vector(i)
        k1, v1 = got.host_vector(i)
        assert np.array_equal(k0, k1) and np.array_equal(v0.view(np.uint32), v1.view(np.uint32))


def test_batched_counts_k7_compact_tables():
    """Protein K = 7 keeps both the (K-1)- and the (K-2)-mer counts compact (one
    entry per seen (K-1)- / (K-2)-mer of the batch); phyloBuildBatchCounts expands
    them: both tables and the totals equal the oracle's dense ones."""
    p = synth.workload("uneven1024", n=3, scale=0.03)
    d = torch.from_numpy(p.data).cuda()
    b = BatchBuilder("protein", 7, max_batch=2)  # two sub-batches
    arena = b.build(d, p.offsets)
    torch.cuda.synchronize()
    for i in range(3):
        r = O.cv_native(p.get(i), 7)
        k, v = arena.host_vector(i)
        assert np.array_equal(k, r["keys"])
        assert ulp_diff(v, r["values"]) <= 1
    L = _native.load()
    scr = b._scratch[1] if b.overlap else b._scratch[0]
    k1 = np.zeros(21 ** 6, np.uint32)
    k2 = np.zeros(21 ** 5, np.uint32)
    tot = np.zeros(3, np.uint32)
    cand = int(np.sum(np.minimum(8 * p.lengths()[2:] + 65536, 21 ** 7)))
    _native.check(L.phyloBuildBatchCounts(torch.cuda.current_stream().cuda_stream,
                                          scr.data_ptr(), scr.numel(), b"protein", 7, 1, cand, 0,
                                          k1.ctypes.data, k2.ctypes.data, tot.ctypes.data))
    e1, e2, et = O.count_tables(p.get(2), 7)
    assert np.array_equal(k1, e1) and np.array_equal(k2, e2) and tuple(tot) == et


def test_build_from_pinned_host_residues():
    """build(host=...) copies each batch's residues from pinned memory just ahead of
    the batch (the copies overlap earlier batches); the arena equals a build from
    residues already on the device, also when the device buffer held other data."""
    p = synth.workload("uneven1024", n=7, scale=0.03)
    b1 = BatchBuilder("protein", 6, max_batch=3)
    ref = b1.build(torch.from_numpy(p.data).cuda(), p.offsets)
    pinned = torch.from_numpy(p.data).pin_memory()
    seq = torch.full((p.data.size,), ord("W"), dtype=torch.uint8, device="cuda")
    b2 = BatchBuilder("protein", 6, max_batch=3)
    got = b2.build(seq, p.offsets, host=pinned)
    torch.cuda.synchronize()
    assert got.n == ref.n == 7
    # one batch: a single copy, ordered before the build on its stream
    seq1 = torch.full((p.data.size,), ord("W"), dtype=torch.uint8, device="cuda")
    one = BatchBuilder("protein", 6, max_batch=24).build(seq1, p.offsets, host=pinned)
    torch.cuda.synchronize()
    for i in range(7):
        k1, v1 = ref.host_vector(i)
        for arena in (got, one):
            k2, v2 = arena.host_vector(i)
            assert np.array_equal(k1, k2) and np.array_equal(v1, v2)
