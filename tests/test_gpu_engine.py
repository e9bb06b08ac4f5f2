"""Batched all-pair engine vs the FP64 oracle: every distance within 1e-6."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rocket_gb300 import synth
from rocket_gb300.engine import BatchBuilder, EngineConfig, PairEngine

from gpu_helpers import ulp_diff

pytestmark = pytest.mark.gpu


def oracle_matrix(p, k=6):
    vecs = [O.cv_native(p.get(i), k) for i in range(len(p))]
    n = len(p)
    C = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            C[i, j] = C[j, i] = O.compare_fp64(vecs[i]["keys"], vecs[i]["values"],
                                               vecs[j]["keys"], vecs[j]["values"])
    return C


@pytest.fixture(scope="module")
def small():
    p = synth.workload("uneven1024", n=20, scale=0.05)
    d = torch.from_numpy(p.data).cuda()
    arena = BatchBuilder("protein", 6).build(d, p.offsets)
    return p, arena, oracle_matrix(p)


@pytest.fixture(scope="module")
def many():
    """90 small proteomes: several 32-row groups and 64-column tiles, ragged edges."""
    p = synth.workload("uneven1024", n=90, scale=0.01)
    d = torch.from_numpy(p.data).cuda()
    arena = BatchBuilder("protein", 6).build(d, p.offsets)
    return p, arena, oracle_matrix(p)


@pytest.mark.parametrize("wshift,fold,rows,compress", [
    (10, 28, 16, True), (9, 8, 16, True), (11, 16, 16, True), (10, 16, 16, False),
    (10, 16, 32, True), (9, 16, 32, True), (10, 8, 32, False)])
def test_allpairs_matches_fp64(small, wshift, fold, rows, compress):
    p, arena, C_ref = small
    eng = PairEngine(arena, EngineConfig(algorithm="window", wshift=wshift, fold=fold,
                                         tile_rows=rows, tile_cols=64 if rows == 32 else 128,
                                         compress=compress))
    eng.ensure_index()
    plan = eng.plan_triangle()
    out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
    eng.run(plan, out)
    C = out.cpu().numpy()
    D, D_ref = (1 - C) / 2, (1 - C_ref) / 2
    err = np.abs(D - D_ref)
    assert err.max() <= 1e-6, err.max()
    # deterministic: a second run is bitwise identical
    out2 = torch.zeros_like(out)
    eng.run(plan, out2)
    assert torch.equal(out, out2)


@pytest.mark.parametrize("block,wshift,compress", [
    (128, 9, True), (128, 6, True), (128, 12, True), (64, 9, True), (64, 11, True),
    (128, 10, False), (64, 12, False)])
def test_postings_matches_fp64(small, block, wshift, compress):
    """Key-major engine: products rounded once to 2^-46 and summed exactly, so every
    C is within (shared keys) * 2^-47 of the FP64 oracle (1e-9 at these sizes);
    window shift 12 leaves a posting capacity below a window's entries, which
    exercises the chunked path."""
    p, arena, C_ref = small
    eng = PairEngine(arena, EngineConfig(algorithm="postings", block=block, wshift=wshift,
                                         compress=compress))
    eng.ensure_index()
    plan = eng.plan_triangle()
    out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
    eng.run(plan, out)
    assert eng.device_status() == 0
    C = out.cpu().numpy()
    assert np.abs(C - C_ref).max() <= 1e-9, np.abs(C - C_ref).max()
    out2 = torch.full_like(out, 3.0)
    eng.run(plan, out2)
    assert torch.equal(out, out2)


@pytest.mark.parametrize("block,wshift", [(64, 9), (64, 7), (128, 8)])
def test_postings_many_blocks(many, block, wshift):
    """90 vectors in blocks of 64: diagonal and off-diagonal tiles, ragged edges; the
    segment count per tile follows the cost model."""
    p, arena, C_ref = many
    eng = PairEngine(arena, EngineConfig(algorithm="postings", block=block, wshift=wshift))
    eng.ensure_index()
    plan = eng.plan_triangle()
    if block == 64:
        assert plan.ntiles == 3
    out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
    eng.run(plan, out)
    assert eng.device_status() == 0
    assert np.abs(out.cpu().numpy() - C_ref).max() <= 1e-9


def test_postings_and_window_agree(many):
    p, arena, _ = many
    outs = []
    for cfg in (EngineConfig(algorithm="postings", block=64, wshift=9),
                EngineConfig(algorithm="window", wshift=10, tile_rows=16, tile_cols=64)):
        eng = PairEngine(arena, cfg)
        eng.ensure_index()
        out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
        eng.run(eng.plan_triangle(), out)
        outs.append(out.cpu().numpy())
    assert np.abs(outs[0] - outs[1]).max() <= 3.6e-6


def test_postings_rectangle_two_arenas(small):
    """Rows and columns from two arenas (raw keys), as the serving path compares a
    query batch with the resident database."""
    p, arena, C_ref = small
    q = synth.workload("uneven1024", n=20, scale=0.05)
    qa = BatchBuilder("protein", 6).build(torch.from_numpy(q.data[:q.offsets[5]].copy()).cuda(),
                                           q.offsets[:6])
    cfg = EngineConfig(algorithm="postings", block=64, wshift=11, compress=False)
    eq = PairEngine(qa, cfg)
    eq.ensure_index()
    ed = PairEngine(arena, cfg)
    ed.ensure_index()
    out = torch.zeros((5, arena.n), dtype=torch.float64, device="cuda")
    plan = eq.plan_rect(np.arange(5), np.arange(arena.n), ldc=arena.n, col_arena=arena)
    eq.run(plan, out, diagonal=False, col_arena=arena)
    # the first five proteomes of both workloads are the same sequences
    assert np.abs(out.cpu().numpy() - C_ref[:5]).max() <= 1e-9


@pytest.mark.parametrize("wshift,rows,cols", [(10, 32, 64), (9, 32, 64), (10, 16, 64),
                                              (9, 16, 32), (10, 16, 32), (11, 16, 128),
                                              (10, 16, 128), (11, 16, 256), (9, 16, 256)])
def test_allpairs_many_tiles(many, wshift, rows, cols):
    p, arena, C_ref = many
    eng = PairEngine(arena, EngineConfig(algorithm="window", wshift=wshift, tile_rows=rows,
                                         tile_cols=cols))
    eng.ensure_index()
    plan = eng.plan_triangle()
    assert plan.ntiles > 2
    out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
    eng.run(plan, out)
    err = np.abs(out.cpu().numpy() - C_ref) / 2
    assert err.max() <= 1e-6, err.max()


def test_tile_rows_agree(many):
    """Both kernels compute the same C to within the accumulation bound."""
    p, arena, _ = many
    outs = []
    for rows, cols in ((16, 64), (32, 64), (16, 32), (16, 256)):
        eng = PairEngine(arena, EngineConfig(algorithm="window", wshift=10, tile_rows=rows,
                                             tile_cols=cols))
        eng.ensure_index()
        out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
        eng.run(eng.plan_triangle(), out)
        outs.append(out.cpu().numpy())
    assert np.abs(outs[0] - outs[1]).max() <= 3.6e-6
    assert np.abs(outs[0] - outs[2]).max() <= 3.6e-6
    assert np.abs(outs[0] - outs[3]).max() <= 3.6e-6


def test_rectangle_plan(small):
    p, arena, C_ref = small
    eng = PairEngine(arena)
    eng.ensure_index()
    rows, cols = np.arange(0, 12), np.arange(12, 20)
    out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
    eng.run(eng.plan_rect(rows, cols, ldc=arena.n), out, diagonal=False)
    C = out.cpu().numpy()
    err = np.abs(C[np.ix_(rows, cols)] - C_ref[np.ix_(rows, cols)]) / 2
    assert err.max() <= 1e-6


def _check_rank_map(arena, keys, rk, union):
    """rk (the arena's rank keys) is one strictly increasing map of every key:
    equal keys get equal ranks in every vector, and a larger key a larger rank."""
    allk = np.concatenate(keys)
    allr = np.concatenate([rk[int(arena.off[v]):int(arena.off[v]) + int(arena.nnz[v])]
                           for v in range(arena.n)])
    order = np.argsort(allk, kind="stable")
    k_s, r_s = allk[order], allr[order]
    same = k_s[1:] == k_s[:-1]
    assert np.all(r_s[1:][same] == r_s[:-1][same])
    assert np.all(r_s[1:][~same] > r_s[:-1][~same])
    assert len(union) <= arena.rank_limit and int(r_s[-1]) < arena.rank_limit


def test_key_ranks(small):
    p, arena, _ = small
    eng = PairEngine(arena, EngineConfig(wshift=10))
    keys = [arena.host_vector(v)[0] for v in range(arena.n)]
    union = np.unique(np.concatenate(keys))
    # a bitmap marked from the keys themselves: ranks in the exact union
    assert arena.union_n == arena.n
    saved = arena.union_n
    arena.union_n, arena.ranked = -1, 0
    eng.ensure_index()
    assert arena.rank_limit == len(union)
    rk = arena.rkeys.cpu().numpy().view(np.uint32)
    for v in range(arena.n):
        o, m, end = int(arena.off[v]), int(arena.nnz[v]), int(arena.off[v + 1])
        assert np.array_equal(rk[o:o + m], np.searchsorted(union, keys[v]))
        assert np.all(rk[o + m:end] == 0xFFFFFFFF)  # padding kept
    # the window index is built on the ranks
    roff = arena.roff.cpu().numpy()
    for v in range(arena.n):
        r = np.searchsorted(union, keys[v])
        expect = np.searchsorted(r, np.arange(arena.R + 1, dtype=np.int64) << 10)
        assert np.array_equal(roff[v, :arena.R + 1], expect)
    # the bitmap the build marked (the candidate keys of every seen (K-1)-mer, a
    # superset of the written keys): one strictly increasing map of the keys, and
    # the window index over it
    arena.union_n, arena.ranked = saved, 0
    eng.ensure_index()
    rk = arena.rkeys.cpu().numpy().view(np.uint32)
    _check_rank_map(arena, keys, rk, union)
    roff = arena.roff.cpu().numpy()
    for v in range(arena.n):
        o, m = int(arena.off[v]), int(arena.nnz[v])
        expect = np.searchsorted(rk[o:o + m], np.arange(arena.R + 1, dtype=np.int64) << 10)
        assert np.array_equal(roff[v, :arena.R + 1], expect)


@pytest.mark.parametrize("wshift", [6, 9, 11])
def test_rank_index_matches_separate_passes(small, wshift):
    """phyloKeyRankIndex (ranks and window index in one pass) gives the ranks of
    phyloKeyRanks and the index phyloWindowIndex builds over them."""
    from rocket_gb300.engine import _p, key_limit
    p, arena, _ = small
    eng = PairEngine(arena, EngineConfig(wshift=wshift))
    eng.ensure_index()
    L, n, R = eng.L, arena.n, arena.R
    limit = key_limit(arena.alphabet, arena.k)
    nb = int(L.phyloKeyRankScratch(limit))
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    maxlen = int(np.max(np.diff(arena.off[:n + 1])))
    rk = torch.full_like(arena.rkeys, 7)
    union = torch.zeros(1, dtype=torch.int64, device="cuda")
    assert L.phyloKeyRanks(0, _p(scratch), nb, limit, _p(arena.keys), _p(arena.vec_off), n,
                           maxlen, 0, _p(rk), _p(union)) == 0
    roff = torch.full_like(arena.roff, 7)
    assert L.phyloWindowIndex(0, _p(rk), _p(arena.vec_off), n, wshift, R, maxlen, _p(roff)) == 0
    torch.cuda.synchronize()
    used = int(arena.off[n])
    keys = [arena.host_vector(v)[0] for v in range(n)]
    exact = np.unique(np.concatenate(keys))
    assert int(union.item()) == len(exact)
    rk_h = rk.cpu().numpy().view(np.uint32)
    for v in range(n):
        o, m = int(arena.off[v]), int(arena.nnz[v])
        assert np.array_equal(rk_h[o:o + m], np.searchsorted(exact, keys[v]))
    # both launch shapes: (slice, vector) CTAs (arena size not given) and the walk
    # over the whole arena (chosen for uneven vectors when the size is given)
    entries = int(arena.off[n] - arena.off[0])
    assert -(-maxlen // 1024) * n > 2 * -(-entries // 1024)  # this arena is uneven
    for given in (0, entries):
        assert L.phyloKeyRanks(0, _p(scratch), nb, limit, _p(arena.keys), _p(arena.vec_off), n,
                               maxlen, 0, 0, _p(union)) == 0
        rk2 = torch.full_like(arena.rkeys, 7)
        roff2 = torch.full_like(arena.roff, 7)
        assert L.phyloKeyRankIndex(0, _p(scratch), nb, limit, _p(arena.keys), _p(arena.vec_off), n,
                                   maxlen, given, 0, wshift, R, _p(rk2), _p(roff2)) == 0
        torch.cuda.synchronize()
        assert torch.equal(rk2[:used], rk[:used])
        assert torch.equal(roff2[:n, :R + 1], roff[:n, :R + 1])


def test_window_index(small):
    p, arena, _ = small
    eng = PairEngine(arena, EngineConfig(wshift=10, compress=False))
    eng.ensure_index()
    roff = arena.roff.cpu().numpy()
    for v in (0, 7, 19):
        keys, _ = arena.host_vector(v)
        expect = np.searchsorted(keys, np.arange(arena.R + 1, dtype=np.int64) << 10)
        assert np.array_equal(roff[v, :arena.R + 1], expect)


def test_multi_pair_merge_matches_fp64(small):
    p, arena, C_ref = small
    eng = PairEngine(arena)
    iu = np.triu_indices(arena.n, 1)
    out = eng.compare_pairs_merge(iu[0], iu[1]).cpu().numpy()
    err = np.abs(out - C_ref[iu]) / 2
    assert err.max() <= 1e-9  # exact products, float-float sums


def test_graph_replay_equals_eager(small):
    p, arena, _ = small
    eng = PairEngine(arena)
    eng.ensure_index()
    plan = eng.plan_triangle()
    eager = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
    eng.run(plan, eager)
    out = torch.zeros_like(eager)
    g = eng.capture(plan, out)
    out.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, eager)


def test_autotune(small, tmp_path, monkeypatch):
    from rocket_gb300.engine import autotune
    p, arena, _ = small
    monkeypatch.setenv("ROCKET_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    r = autotune(arena, repeats=1)
    assert r["algorithm"] in ("postings", "window", "merge") and r["ms"] > 0
    assert len(r["candidates"]) >= 2
    assert autotune(arena)["ms"] == r["ms"]  # served from the cache


def test_directory_driver(tmp_path):
    """The command-line driver: FASTA files in, all-pair JSON out (C, -1 nowhere)."""
    import json
    from rocket_gb300.output import main
    p = synth.workload("uneven1024", n=5, scale=0.01)
    for i in range(len(p)):
        seq = p.get(i).decode().split("\n")
        (tmp_path / f"g{i}.faa").write_text("".join(f">p{j}\n{s}\n" for j, s in enumerate(seq) if s))
    out = tmp_path / "out.json"
    assert main([str(tmp_path), str(out)]) == 0
    d = json.loads(out.read_text())
    C = np.array(d["distance"])
    assert d["files"] == [f"g{i}.faa" for i in range(5)]
    C_ref = oracle_matrix(p)
    assert np.abs(C - C_ref).max() <= 2e-6


def test_batched_ragged_edge_proteomes():
    """A build batch holding an empty proteome, one shorter than K, one of mostly
    invalid symbols, one of exactly K symbols and one of short proteins, between
    two normal ones: every vector, and every pair and self product, against the
    oracle (NaN where the oracle has NaN)."""
    p = synth.workload("uneven1024", n=2, scale=0.02)
    seqs = [p.get(0), b"", b"ACD", b"XBZJOU" * 50, b"ACDEFG", b"MKV\nLLA\nWWWWWW\nAC", p.get(1)]
    off = np.zeros(len(seqs) + 1, np.int64)
    np.cumsum([len(s) for s in seqs], out=off[1:])
    data = torch.from_numpy(np.frombuffer(b"".join(seqs), np.uint8).copy()).cuda()
    arena = BatchBuilder("protein", 6, max_batch=4).build(data, off)
    torch.cuda.synchronize()
    ref = [O.cv_native(s, 6) for s in seqs]
    for i, r in enumerate(ref):
        k, v = arena.host_vector(i)
        assert np.array_equal(k, r["keys"]), i
        assert np.array_equal(np.isnan(v), np.isnan(r["values"])), i
        assert ulp_diff(v, r["values"]) <= 1, i
    eng = PairEngine(arena)
    eng.ensure_index()
    out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device="cuda")
    eng.run(eng.plan_triangle(), out)
    C = out.cpu().numpy()
    for i in range(len(seqs)):
        for j in range(i, len(seqs)):
            c = O.compare_fp64(ref[i]["keys"], ref[i]["values"], ref[j]["keys"], ref[j]["values"])
            if np.isnan(c):
                assert np.isnan(C[i, j]), (i, j)
            else:
                assert abs(C[i, j] - c) <= 2e-6, (i, j, C[i, j], c)
