"""Serving loop: continuous batching against a device-resident database.

Each request's result must be identical whether it ran alone or merged with
other requests into one batch, and within 1e-6 (on D) of the FP64 oracle."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rocket_gb300 import synth
from rocket_gb300.engine import EngineConfig
from rocket_gb300.serve import Request, ServingEngine

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def data():
    p = synth.workload("serve2048", n=14, scale=0.03, extra=10)
    db = p.subset(range(14))
    # requests of 1-3 proteomes
    sizes = [1, 2, 1, 3, 1, 2]
    reqs, i = [], 14
    for s in sizes:
        reqs.append(p.subset(range(i, i + s)))
        i += s
    return p, db, reqs


def _server(db, slots=2, max_batch=6):
    srv = ServingEngine("protein", 6, budget_bytes=40e9, slots=slots, max_batch=max_batch,
                        cfg=EngineConfig(segments=4))
    srv.load(db)
    srv.start()
    return srv


def test_alone_equals_mixed(data):
    p, db, queries = data
    srv = _server(db)
    mixed = [srv.submit(Request(i, q, append=False)) for i, q in enumerate(queries)]
    for r in mixed:
        assert r.done.wait(300) and r.error is None, r.error
    srv.stop()
    assert len({r.batch_id for r in mixed}) < len(mixed)  # some requests shared a batch
    for q, r in zip(queries, mixed):
        srv1 = _server(db, slots=1)
        alone = srv1.submit(Request(0, q, append=False))
        assert alone.done.wait(300) and alone.error is None
        srv1.stop()
        assert alone.db_n == r.db_n == len(db)
        assert np.array_equal(alone.result, r.result)  # bitwise


def test_results_match_oracle(data):
    p, db, queries = data
    srv = _server(db)
    reqs = [srv.submit(Request(i, q, append=False)) for i, q in enumerate(queries[:3])]
    for r in reqs:
        assert r.done.wait(300) and r.error is None
    srv.stop()
    dbv = [O.cv_native(db.get(j), 6) for j in range(len(db))]
    for r, q in zip(reqs, queries[:3]):
        for a in range(len(q)):
            qa = O.cv_native(q.get(a), 6)
            for j in range(len(db)):
                exact = O.compare_fp64(qa["keys"], qa["values"], dbv[j]["keys"], dbv[j]["values"])
                assert abs((1 - r.result[a, j]) / 2 - (1 - exact) / 2) <= 1e-6


def test_appended_queries_join_the_database(data):
    p, db, queries = data
    srv = _server(db, slots=1)
    r0 = srv.submit(Request(0, queries[1], append=True))
    assert r0.done.wait(300) and r0.error is None
    r1 = srv.submit(Request(1, queries[0], append=True))
    assert r1.done.wait(300) and r1.error is None
    srv.stop()
    assert r1.db_n == len(db) + len(queries[1])
    # the new columns are the first request's proteomes
    q0 = O.cv_native(queries[0].get(0), 6)
    for a in range(len(queries[1])):
        v = O.cv_native(queries[1].get(a), 6)
        exact = O.compare_fp64(q0["keys"], q0["values"], v["keys"], v["values"])
        assert abs(r1.result[0, len(db) + a] - exact) / 2 <= 1e-6


def test_tuned_width_serves_the_oracle(data):
    """tune() times query-shaped rectangles under each item width and keeps the
    fastest; requests served with it match the oracle."""
    p, db, queries = data
    srv = ServingEngine("protein", 6, budget_bytes=40e9, slots=2, max_batch=6,
                        cfg=EngineConfig(segments=4))
    srv.load(db)
    t = srv.tune(widths=(128, 256), rows=8)
    assert t["tile_cols"] in (128, 256) and len(t["candidates"]) == 2
    assert srv.cfg.tile_cols == t["tile_cols"]
    srv.start()
    r = srv.submit(Request(0, queries[3], append=False))
    assert r.done.wait(300) and r.error is None, r.error
    srv.stop()
    dbv = [O.cv_native(db.get(j), 6) for j in range(len(db))]
    for a in range(len(queries[3])):
        qa = O.cv_native(queries[3].get(a), 6)
        for j in range(len(db)):
            exact = O.compare_fp64(qa["keys"], qa["values"], dbv[j]["keys"], dbv[j]["values"])
            assert abs(r.result[a, j] - exact) / 2 <= 1e-6
