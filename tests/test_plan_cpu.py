"""The pair planner's host logic on the CPU: coverage, key segments, cost models, order.

A plan is the only thing that tells the persistent pair kernels which pairs and which
key windows to visit, so two properties carry the engine's correctness: every pair the
caller asked for lies in exactly one tile (the self products once more for a triangle),
and each tile's key windows [0, R) are split among its items without a gap or an
overlap.  The estimates order the launch (longest first) and size the segments; the
nnz-product estimate of a tile is checked against the sum it stands for, computed pair
by pair.  The engine is made without a device (no library, no kernel): the planner
reads only the arena's entry counts, window count and key space.
"""
import math
from types import SimpleNamespace

import numpy as np
import pytest

from rocket_gb300.engine import EngineConfig, PairEngine, key_limit


def _engine(nnz, R=64, grid=152 * 2, rank_limit=None, **cfg):
    eng = PairEngine.__new__(PairEngine)
    eng.cfg = EngineConfig(**cfg)
    eng.arena = SimpleNamespace(
        n=len(nnz), nnz=np.asarray(nnz, np.int64), R=R, alphabet="protein", k=6,
        rank_limit=rank_limit if rank_limit is not None else key_limit("protein", 6),
        index_on_ranks=rank_limit is not None)
    eng.grid = grid
    eng.device = "cpu"
    return eng


def _nnz(n, seed):
    rng = np.random.default_rng(seed)
    return np.clip(rng.lognormal(np.log(5e5), 0.9, n), 1e4, 3e6).astype(np.int64)


def _tile_pairs(plan):
    """Pairs (row id, col id) of every tile, as the kernels visit them: a triangle's
    tile drops the positions below its diagonal (upper), keeping the self products."""
    seen = {}
    rows, cols = plan.host_rowids, plan.host_colids
    for t in plan.host_tiles:
        r0, nr, c0, nc = (int(x) for x in t[:4])
        for i in range(r0, r0 + nr):
            for j in range(c0, c0 + nc):
                if plan.upper and j < i:
                    continue
                key = (int(rows[i]), int(cols[j]))
                seen[key] = seen.get(key, 0) + 1
    return seen


def _check_segments(plan, R):
    """Each tile's items split [0, R) into consecutive, non-empty, disjoint ranges."""
    items = plan.host_items
    by_tile = {}
    for it, t in zip(items, plan.item_tile):
        by_tile.setdefault(int(t), []).append((int(it[4]), int(it[5])))
    assert sorted(by_tile) == list(range(plan.ntiles))
    for t, segs in by_tile.items():
        segs.sort()
        assert segs[0][0] == 0 and segs[-1][1] == R, (t, segs)
        for (a0, a1), (b0, b1) in zip(segs, segs[1:]):
            assert a1 == b0, (t, segs)
        assert all(b > a for a, b in segs), (t, segs)
        tl = plan.host_tiles[t]
        for it in items[plan.item_tile == t]:  # every item carries its tile's shape
            assert tuple(int(x) for x in it[:4]) == tuple(int(x) for x in tl[:4])


@pytest.mark.parametrize("cfg", [
    dict(algorithm="window", tile_rows=16, tile_cols=256, items_per_cta=16),
    dict(algorithm="window", tile_rows=16, tile_cols=128),
    dict(algorithm="window", tile_rows=32, tile_cols=64, wshift=10),
    dict(algorithm="postings", block=128, wshift=9, items_per_cta=4),
    dict(algorithm="postings", block=64, wshift=9),
])
@pytest.mark.parametrize("n", [1, 2, 17, 300])
def test_triangle_covers_every_pair_once(cfg, n):
    R = 40
    eng = _engine(_nnz(n, n), R=R, **cfg)
    plan = eng.plan_triangle()
    assert plan.diag and plan.upper and plan.pairs == n * (n - 1) // 2
    seen = _tile_pairs(plan)
    # each unordered pair once (as row <= col in the nnz-sorted order), each self product once
    unordered = {}
    for (i, j), c in seen.items():
        key = (min(i, j), max(i, j))
        unordered[key] = unordered.get(key, 0) + c
    assert len(unordered) == n * (n + 1) // 2
    assert set(unordered.values()) == {1}
    _check_segments(plan, R)
    assert np.all(np.diff(plan.est) <= 0)  # longest items first
    assert plan.nitems == len(plan.host_items) == len(plan.est)


@pytest.mark.parametrize("cfg", [
    dict(algorithm="window", tile_rows=16, tile_cols=256),
    dict(algorithm="window", tile_rows=16, tile_cols=64, wshift=10),
    dict(algorithm="postings", block=128, wshift=9),
])
def test_rectangle_covers_every_pair_once(cfg):
    rng = np.random.default_rng(3)
    nnz = _nnz(200, 5)
    rows = rng.choice(200, 37, replace=False)
    cols = rng.choice(200, 150, replace=False)
    R = 23
    eng = _engine(nnz, R=R, **cfg)
    plan = eng.plan_rect(rows, cols, ldc=200)
    assert not plan.upper and plan.pairs == 37 * 150
    seen = _tile_pairs(plan)
    assert set(seen) == {(int(r), int(c)) for r in rows for c in cols}
    assert set(seen.values()) == {1}
    _check_segments(plan, R)
    # rows and columns are visited longest vector first
    assert np.all(np.diff(nnz[plan.host_rowids]) <= 0)
    assert np.all(np.diff(nnz[plan.host_colids]) <= 0)


def test_window_segments_fill_the_grid():
    """Window tiles get S segments each, enough that the items number at least
    items_per_cta x the grid where the windows allow, and no segment thinner than
    min_windows_per_item windows."""
    # 1,024 proteomes on 2^11-rank windows (29,872 of them), one 512-thread CTA per SM
    eng = _engine(_nnz(1024, 1), R=29872, grid=152, tile_rows=16, tile_cols=256,
                  items_per_cta=16)
    plan = eng.plan_triangle()
    ntiles = plan.ntiles
    assert ntiles == sum(math.ceil((1024 - r0) / 256) for r0 in range(0, 1024, 16)) == 160
    assert plan.S == math.ceil(16 * 152 / ntiles) == 16
    assert plan.nitems == ntiles * plan.S == 2560
    thin = _engine(_nnz(1024, 1), R=1867, grid=304, tile_rows=16, tile_cols=256,
                   items_per_cta=16)  # 31 segments wanted, 1,867 // 64 = 29 allowed
    assert thin.plan_triangle().S == 29
    few = _engine(_nnz(64, 2), R=100, tile_rows=16, tile_cols=256)
    assert few.plan_triangle().S == 100 // few.cfg.min_windows_per_item
    fixed = _engine(_nnz(64, 2), R=100, tile_rows=16, tile_cols=256, segments=7)
    assert fixed.plan_triangle().S == 7


def test_postings_segments_follow_the_cost():
    """Postings tiles take segments in proportion to their estimate, so that the
    items' estimates come out about equal (within the rounding of one segment)."""
    eng = _engine(_nnz(900, 4), R=4000, grid=152, algorithm="postings", block=128,
                  items_per_cta=4, rank_limit=45_000_000)
    plan = eng.plan_triangle()
    cost = eng.tile_costs(plan.host_rowids, plan.host_colids,
                          [tuple(int(x) for x in t[:4]) + (int(t[6]),) for t in plan.host_tiles],
                          eng.arena.nnz, eng.arena.nnz)
    S_t = plan.host_tiles[:, 5]
    target = cost.sum() / (4 * eng.grid)
    assert np.array_equal(S_t, np.clip(np.ceil(cost / target), 1, 4000).astype(np.int64))
    per_item = cost / S_t
    assert per_item.max() <= target * 1.0001
    assert plan.nparts == int(S_t.sum()) == plan.nitems


def test_nnz_product_model_is_the_pairwise_sum():
    """nnz_product of a tile = sum over its pairs of nnz_i nnz_j / U (+ entries and
    windows); a diagonal tile counts each pair once and each self product once."""
    nnz = _nnz(40, 9)
    U = 1_000_000
    eng = _engine(nnz, R=10, rank_limit=U, algorithm="postings", block=64)
    rows = np.argsort(-nnz, kind="stable")
    tiles = [(0, 16, 0, 16, 1), (0, 16, 16, 24, 0), (16, 24, 16, 24, 1), (5, 7, 30, 9, 0)]
    m = eng.tile_cost_models(rows, rows, tiles, nnz, nnz)
    for (r0, nr, c0, nc, d), got in zip(tiles, m["nnz_product"]):
        rn = nnz[rows[r0:r0 + nr]].astype(np.float64)
        cn = nnz[rows[c0:c0 + nc]].astype(np.float64)
        if d:
            prod = sum(rn[i] * rn[j] for i in range(nr) for j in range(i, nr)) / U
            ent = rn.sum()
        else:
            prod = float(np.outer(rn, cn).sum()) / U
            ent = rn.sum() + cn.sum()
        want = (eng.PB_COST_PRODUCT * prod + eng.PB_COST_ENTRY * ent + eng.PB_COST_WINDOW * 10)
        assert got == pytest.approx(want, rel=1e-12)
    for (r0, nr, c0, nc, d), got in zip(tiles, m["linear"]):
        sr = float(nnz[rows[r0:r0 + nr]].sum())
        sc = float(nnz[rows[c0:c0 + nc]].sum())
        assert got == pytest.approx(eng.cfg.tile_rows * sc + 2.0 * sr + 64.0 * 10, rel=1e-12)


def test_item_cost_models_split_tile_estimates():
    """Per-item estimates (the cost-model fit's inputs) are the tile's estimate
    times the item's share of its windows, and add up to the tile's estimate."""
    eng = _engine(_nnz(100, 6), R=50, tile_rows=16, tile_cols=128, items_per_cta=8, grid=40)
    plan = eng.plan_triangle()
    m = eng.item_cost_models(plan)
    tiles = [tuple(int(x) for x in t[:4]) + (0,) for t in plan.host_tiles]
    whole = eng.tile_cost_models(plan.host_rowids, plan.host_colids, tiles,
                                 eng.arena.nnz, eng.arena.nnz)
    for name in ("linear", "nnz_product"):
        sums = np.bincount(plan.item_tile, weights=m[name], minlength=plan.ntiles)
        np.testing.assert_allclose(sums, whole[name], rtol=1e-12)
    # the window kernel's launch order follows its own (linear) estimate
    np.testing.assert_allclose(plan.est, m["linear"], rtol=1e-12)


@pytest.mark.parametrize("algorithm", ["window", "postings"])
@pytest.mark.parametrize("diagonal", [True, False])
def test_nonfinite_vectors_recomputed_pairs(algorithm, diagonal):
    """Pairs with a vector whose norm is not finite (a proteome without K-windows)
    are recomputed by the merge path: exactly those pairs of the plan (the self
    products only when the diagonal is asked for), written to both mirror slots."""
    import torch
    n = 40
    eng = _engine(_nnz(n, 8), R=16, algorithm=algorithm, block=64, tile_rows=16,
                  tile_cols=128)
    norms = np.ones(n)
    bad = [3, 17, 39]
    norms[bad] = np.nan
    eng.arena.norms = norms
    plan = eng.plan_triangle(ldc=n)
    calls = []

    def fake_merge(pa, pb, col_arena=None, stream=None):
        calls.append((pa.copy(), pb.copy()))
        return torch.from_numpy(1000.0 + pa * n + pb)

    eng.compare_pairs_merge = fake_merge
    out = torch.full((n * n,), -1.0, dtype=torch.float64)
    eng._fix_nonfinite(plan, out, None, diag=diagonal)
    (pa, pb), = calls
    got = {(int(a), int(b)) for a, b in zip(pa, pb)}
    assert len(got) == len(pa)  # each pair once
    want = set()
    for i in range(n):
        for j in range(i, n):
            if (i in bad or j in bad) and (i != j or diagonal):
                want.add((i, j))
    assert {(min(a, b), max(a, b)) for a, b in got} == want
    o = out.view(n, n).numpy()
    for a, b in got:
        assert o[a, b] == o[b, a] == 1000.0 + a * n + b
    assert np.count_nonzero(o != -1.0) == 2 * len(want) - sum(1 for a, b in want if a == b)
    # nothing to do when every norm is finite
    eng.arena.norms = np.ones(n)
    eng._fix_nonfinite(plan, out, None, diag=diagonal)
    assert len(calls) == 1
