"""Full-scale parity at the batched configuration: uneven1024 (1,024 proteomes of
0.1-4 M residues, K = 6, 523,776 pairs), and the pair engines at K = 5 and K = 7.

* Every one of the 1,024 vectors against the oracle's restatement of the
  reference rule (native.cu:220-474): sizes and keys bit for bit, values within
  one float ulp.  The oracle runs in a pool of worker processes (started with
  `spawn`); each returns a digest of its vector, and any vector whose value digest
  differs is fetched and compared element by element.
* All 523,776 pairs of the window engine (the default batched path) against the
  postings engine, an independent kernel whose products are exactly rounded and
  whose sums are exact integers: |dD| <= 1e-6 everywhere.  (The multi-pair
  merge kernel would have to read 8 (N - 1) sum(nnz) = 42 TB for all pairs.)
* Both engines against the FP64 oracle (exact products, compensated double
  sums, C merge loop) on 2,000+ pairs that include all pairs of the 32 largest
  proteomes: |dD| <= 1e-6 for both.  (The postings engine rounds each product
  once to 2^-46 and sums exactly, so |dC| <= (shared keys) * 2^-47, at most
  1.6e-7 here; most of a pair's products are the same constant -- the alpha = -1
  entries -- so their rounding errors add up rather than cancel.)
* K = 5 and K = 7 arenas through both pair engines, with 16 x 256 window items
  and the arena-walk rank index (uneven vector lengths), against the FP64 oracle.

Measured |dD| (max and 99th percentile) is printed for the record.
"""
import concurrent.futures as cf
import ctypes
import multiprocessing as mp
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from rocket_gb300 import synth
from rocket_gb300.engine import BatchBuilder, EngineConfig, PairEngine

pytestmark = pytest.mark.gpu


def device_digest(keys: torch.Tensor, values: torch.Tensor):
    """oracle.digest() computed on the device (int64 wraps like uint64)."""
    k = keys.to(torch.int64) & 0xFFFFFFFF
    v = values.view(torch.int32).to(torch.int64) & 0xFFFFFFFF
    i = torch.arange(k.numel(), dtype=torch.int64, device=k.device)
    hk = int(((k + 1) * (2 * i + 1)).sum().item()) & 0xFFFFFFFFFFFFFFFF
    hv = int(((v + 7) * (i + 3)).sum().item()) & 0xFFFFFFFFFFFFFFFF
    return k.numel(), hk, hv


@pytest.fixture(scope="module")
def uneven():
    # the pool starts before this module's first GPU work in the worker-free parent
    ctx = mp.get_context("spawn")
    pool = cf.ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 4), mp_context=ctx)
    wl = synth.workload("uneven1024")
    arena = BatchBuilder("protein", 6).build(torch.from_numpy(wl.data).cuda(), wl.offsets)
    torch.cuda.synchronize()
    yield wl, arena, pool
    pool.shutdown()
    del arena
    torch.cuda.empty_cache()


def test_uneven1024_every_vector_matches_the_oracle(uneven):
    wl, arena, pool = uneven
    n = len(wl)
    assert arena.n == n
    # largest first, so the pool's tail is short
    order = np.argsort(-wl.lengths())
    futs = {int(i): pool.submit(O.cv_native_digest, (wl.get(int(i)), 6)) for i in order}
    value_mismatch = []
    for i, fut in futs.items():
        m, hk, hv = fut.result(timeout=3600)
        k, v = arena.vector(i)
        dm, dhk, dhv = device_digest(k, v)
        assert dm == m == int(arena.nnz[i]), (i, dm, m)
        assert dhk == hk, f"keys of vector {i} differ from the oracle's"
        if dhv != hv:
            value_mismatch.append(i)
    # vectors whose value bits differ somewhere: element by element, within one ulp
    from gpu_helpers import ulp_diff
    for i in value_mismatch[:16]:
        r = O.cv_native(wl.get(i), 6)
        assert ulp_diff(arena.host_vector(i)[1], r["values"]) <= 1, i
    assert len(value_mismatch) <= 16, len(value_mismatch)
    print(f"\nuneven1024: {n} vectors, {int(arena.nnz.sum()):,} entries; keys bit-exact; "
          f"value digests differ in {len(value_mismatch)} vectors (all within 1 ulp)")


def _engine_matrix(arena, cfg):
    eng = PairEngine(arena, cfg)
    eng.ensure_index()
    C = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
    eng.run(eng.plan_triangle(), C)
    if cfg.algorithm == "postings":
        assert eng.device_status() == 0
    return C.cpu().numpy()


@pytest.fixture(scope="module")
def uneven_matrices(uneven):
    wl, arena, _ = uneven
    win = _engine_matrix(arena, EngineConfig(algorithm="window", wshift=11, tile_rows=16,
                                             tile_cols=256))
    post = _engine_matrix(arena, EngineConfig(algorithm="postings", block=128, wshift=9))
    return win, post


def test_uneven1024_all_pairs_window_vs_postings(uneven, uneven_matrices):
    wl, arena, _ = uneven
    win, post = uneven_matrices
    n = arena.n
    iu = np.triu_indices(n, 1)
    dD = np.abs(win[iu] - post[iu]) / 2
    assert len(dD) == 523776
    print(f"\nuneven1024 window engine vs postings engine, all {len(dD):,} pairs: max |dD| "
          f"{dD.max():.3g}, p99 {np.percentile(dD, 99):.3g}")
    assert dD.max() <= 1e-6
    assert np.array_equal(win, win.T) and np.array_equal(post, post.T)
    # the self products: 1 up to the rounding of the unit vectors
    assert np.abs(np.diag(win) - 1.0).max() <= 1e-6
    assert np.abs(np.diag(post) - 1.0).max() <= 1e-6


def test_uneven1024_fp64_oracle_pairs(uneven, uneven_matrices):
    wl, arena, _ = uneven
    win, post = uneven_matrices
    n = arena.n
    big = np.argsort(-arena.nnz)[:32]
    rng = np.random.default_rng(11)
    others = rng.choice(np.setdiff1d(np.arange(n), big), 96, replace=False)
    pool_v = np.concatenate([big, others])
    pairs = [(int(min(a, b)), int(max(a, b))) for x, a in enumerate(big) for b in big[x + 1:]]
    while len(pairs) < 2048:
        a, b = (int(x) for x in rng.choice(pool_v, 2, replace=False))
        pairs.append((min(a, b), max(a, b)))
    host = {int(v): arena.host_vector(int(v)) for v in pool_v}
    L = O.lib()
    P32 = ctypes.POINTER(ctypes.c_uint32)
    PF = ctypes.POINTER(ctypes.c_float)

    def fp64(p):
        (ka, va), (kb, vb) = host[p[0]], host[p[1]]
        return L.oracle_compare_fp64(ka.ctypes.data_as(P32), va.ctypes.data_as(PF), len(ka),
                                     kb.ctypes.data_as(P32), vb.ctypes.data_as(PF), len(kb))

    with cf.ThreadPoolExecutor(16) as ex:  # the C loop runs without the GIL
        exact = np.array(list(ex.map(fp64, pairs)))
    for name, C, tol in (("window", win, 1e-6), ("postings", post, 1e-7)):
        got = np.array([C[a, b] for a, b in pairs])
        dD = np.abs(got - exact) / 2
        print(f"\nuneven1024 {name} engine vs FP64 oracle, {len(pairs)} pairs (all pairs of the "
              f"32 largest): max |dD| {dD.max():.3g}, p99 {np.percentile(dD, 99):.3g}")
        assert dD.max() <= tol, name


@pytest.mark.parametrize("k", [5, 7])
def test_pair_engines_at_k(k):
    """sweep512-distributed sizes, scaled down; 16 x 256 window items, the
    arena-walk rank index, and the postings engine, against the FP64 oracle."""
    p = synth.workload("sweep512", n=40, scale=0.05)
    arena = BatchBuilder("protein", k).build(torch.from_numpy(p.data).cuda(), p.offsets)
    torch.cuda.synchronize()
    n = arena.n
    vecs = [arena.host_vector(v) for v in range(n)]
    ref = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            ref[i, j] = ref[j, i] = O.compare_fp64(vecs[i][0], vecs[i][1], vecs[j][0], vecs[j][1])
    # the device vectors are the oracle's (keys bit-exact, values within 1 ulp)
    for v in (0, n // 2, n - 1):
        r = O.cv_native(p.get(v), k)
        assert np.array_equal(vecs[v][0], r["keys"])
    entries = int(arena.off[n] - arena.off[0])
    maxlen = int(np.max(np.diff(arena.off[:n + 1])))
    assert -(-maxlen // 1024) * n > 2 * -(-entries // 1024)  # uneven: the arena-walk index
    for cfg, tol in ((EngineConfig(algorithm="window", wshift=11, tile_rows=16, tile_cols=256),
                      1e-6),
                     (EngineConfig(algorithm="window", wshift=10, tile_rows=32, tile_cols=64),
                      1e-6),
                     (EngineConfig(algorithm="postings", block=64, wshift=9), 1e-7)):
        eng = PairEngine(arena, cfg)
        eng.ensure_index()
        out = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        eng.run(eng.plan_triangle(), out)
        dD = np.abs(out.cpu().numpy() - ref) / 2
        assert dD.max() <= tol, (cfg.algorithm, dD.max())
