"""Golden vectors from the reference's own library, for the CPU tests that pin the oracle.

The reference's CUDA file (phylogenetics/src/main/cpp/native.cu) is compiled unmodified
by ``make -C oracle ref`` (``build()`` does it where the source is staged) and driven
through its C ABI (tests/refabi.py).  Run on a GPU host after ``build()``:

    python tests/golden/make_reference_golden.py

It writes tests/golden/reference_vectors.npz:

* builds: for every case, the reference's vector size, keys (delta-coded) and values
  for the inputs of BindingsTest.testBuildVector (BindingsTest.java:79-97: protein K =
  3..7, DNA K = 3..10, inputs of 10, 100 and 1000 proteins of seed 0) and for small
  literal inputs (edge cases: empty, shorter than K, invalid letters, a seen K-mer with
  alpha exactly 0, homopolymers whose vector is empty);
* compares: the reference's C for the cases of BindingsTest.testCompareVectors
  (:159-213: n = 10 .. 10,000, overlap 0, 0.5, 1, seeds 0..3), except the sizes at which
  the reference's compare races with itself (refabi.compare_block_race).

Inputs are not stored except the literal ones: BindingsTest's generators are
reimplemented exactly by the oracle (java.util.Random), so the tests regenerate them.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

LITERALS = [
    ("protein", 3, b""), ("protein", 3, b"A"), ("protein", 3, b"AC"), ("protein", 3, b"ACACA"),
    ("protein", 3, b"AAAAA"), ("protein", 3, b"ACA\nCC"), ("protein", 3, b"XYXYX"),
    ("protein", 4, b"ACDE\nFGHI"), ("protein", 6, b"ACDEFGHIKLMNPQRSTVWYX"),
    ("protein", 5, b"ACDBJOUZ" * 8), ("protein", 5, b"Q" * 50), ("DNA", 8, b"C" * 50),
    ("DNA", 3, b"T\nCGC"), ("DNA", 4, b"TTTT\nCGTG"), ("DNA", 5, b"CACAC\nAAA"),
    ("DNA", 6, b"CAATAG\nGGGGGG"), ("DNA", 7, b"TTCTCGA\nTTTTTTT"),
    ("protein", 3, b"AII\nRRR"), ("protein", 4, b"ALCP\nEEEE"), ("protein", 5, b"PPPP\nHHHHHM"),
    ("protein", 6, b"RRRRRR\nMLVITL"), ("protein", 3, b"RRRRRRRRRYYYYY\nSSSS"),
]
SWEEP = [("protein", k, n) for k in range(3, 8) for n in (10, 100, 1000)] + \
        [("DNA", k, n) for k in range(3, 11) for n in (10, 100, 1000)]
COMPARES = [(seed, n, ratio) for n in (10, 100, 1000, 10000) for ratio in (0.0, 0.5, 1.0)
            for seed in range(4)]


def main():
    import torch
    import refabi
    from oracle import oracle as O

    if not refabi.staged():
        raise SystemExit("the reference's native.cu is not staged (make -C oracle stage-ref)")
    st = torch.cuda.current_stream().cuda_stream
    A = {"protein": 21, "DNA": 4}

    def ref_build(alphabet, k, seq, max_size):
        d_in = torch.from_numpy(np.frombuffer(seq + b"\0", np.uint8).copy()).cuda()
        need = refabi.scratch_bytes(alphabet, k, max_size)
        scr = torch.empty(max(need, 1), dtype=torch.uint8, device="cuda")
        keys = torch.full((max_size,), 0x1234, dtype=torch.int32, device="cuda")
        vals = torch.full((max_size,), 7.0, dtype=torch.float32, device="cuda")
        size = np.zeros(1, np.int32)
        rc = refabi.build(st, scr, alphabet, k, d_in, len(seq), keys, vals, size, max_size)
        torch.cuda.synchronize()
        assert rc == 0, (alphabet, k, rc)
        n = int(size[0])
        return keys[:n].cpu().numpy().view(np.uint32), vals[:n].cpu().numpy()

    meta, keys, vals, lit = [], [], [], []
    for alphabet, k, n in SWEEP:
        seq = O.bindings_input(0, n, alphabet)
        kk, vv = ref_build(alphabet, k, seq, min(A[alphabet] ** k, 1000 * n))
        meta.append((0 if alphabet == "protein" else 1, k, n, -1, len(kk)))
        keys.append(kk)
        vals.append(vv)
    for i, (alphabet, k, seq) in enumerate(LITERALS):
        kk, vv = ref_build(alphabet, k, seq, min(A[alphabet] ** k, 21 * len(seq) + 64))
        meta.append((0 if alphabet == "protein" else 1, k, 0, i, len(kk)))
        keys.append(kk)
        vals.append(vv)
    cmp_meta, cmp_c = [], []
    for seed, n, ratio in COMPARES:
        lk, lv, rk, rv, _ = O.bindings_compare_case(seed, n, ratio)
        if refabi.compare_block_race(len(lk), len(rk)):
            continue
        t = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (lk, lv, rk, rv)]
        scr = torch.empty(refabi.scratch_bytes("DNA", 3, max(len(lk), len(rk), 1)),
                          dtype=torch.uint8, device="cuda")
        out = torch.full((1,), -5.0, dtype=torch.float64, device="cuda")
        rc = refabi.compare(st, scr, t[0], t[1], len(lk), t[2], t[3], len(rk), out)
        torch.cuda.synchronize()
        assert rc == 0
        cmp_meta.append((seed, n, ratio))
        cmp_c.append(float(out.item()))
    allk = np.concatenate(keys) if keys else np.zeros(0, np.uint32)
    # keys delta-coded within each vector (they ascend): the file compresses well
    starts = np.cumsum([0] + [len(x) for x in keys])
    deltas = allk.astype(np.int64).copy()
    for a, b in zip(starts[:-1], starts[1:]):
        if b > a:
            deltas[a + 1:b] = np.diff(allk[a:b].astype(np.int64))
    np.savez_compressed(os.path.join(HERE, "reference_vectors.npz"),
                        meta=np.array(meta, np.int64), key_deltas=deltas.astype(np.uint32),
                        values=np.concatenate(vals), cmp_meta=np.array(cmp_meta, np.float64),
                        cmp_c=np.array(cmp_c, np.float64))
    print(f"{len(meta)} vectors ({len(allk)} entries), {len(cmp_c)} compares")


if __name__ == "__main__":
    main()
