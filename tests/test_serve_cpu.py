"""Host-side serving logic that needs no GPU: HBM budget admission."""
import threading
import time

import pytest

from rocket_gb300.serve import Budget


def test_budget_blocks_until_release():
    b = Budget(100.0)
    b.reserve(60.0)
    got = []

    def second():
        b.reserve(50.0)
        got.append(time.perf_counter())

    t = threading.Thread(target=second)
    t0 = time.perf_counter()
    t.start()
    time.sleep(0.2)
    assert not got  # 60 + 50 > 100: waits
    b.release(60.0)
    t.join(5)
    assert got and got[0] - t0 >= 0.2
    assert b.used == 50.0 and b.peak == 60.0


def test_budget_refuses_what_can_never_fit():
    b = Budget(10.0)
    with pytest.raises(MemoryError):
        b.reserve(11.0)


def test_budget_times_out():
    b = Budget(10.0)
    b.reserve(8.0)
    with pytest.raises(TimeoutError):
        b.reserve(5.0, timeout=0.1)


def test_budget_refuses_oversize_while_others_hold_memory():
    """A request larger than the whole budget fails at once, also while other
    batches hold part of it (it could never be admitted, however much they free)."""
    b = Budget(10.0)
    b.reserve(4.0)
    t0 = time.perf_counter()
    with pytest.raises(MemoryError):
        b.reserve(11.0, timeout=5.0)
    assert time.perf_counter() - t0 < 1.0
    assert b.used == 4.0


# -- the dispatcher (continuous batching) with stand-in slots: no device work --------

from types import SimpleNamespace  # noqa: E402

import numpy as np  # noqa: E402

from rocket_gb300.serve import Request, ServingEngine  # noqa: E402


class _Q:
    """A query batch of n proteomes (only its size matters to the dispatcher)."""

    def __init__(self, n):
        self.n = n
        self.data = np.zeros(0, np.uint8)
        self.offsets = np.zeros(n + 1, np.int64)

    def __len__(self):
        return self.n

    def lengths(self):
        return np.full(self.n, 1000, np.int64)


def _server(slots, max_batch, hold=0.05):
    srv = ServingEngine(slots=slots, max_batch=max_batch, budget_bytes=1e12)
    srv.db = SimpleNamespace(snapshot=lambda: 0)
    srv.slots = [SimpleNamespace(idx=i, busy=False) for i in range(slots)]
    runs, lock = [], threading.Lock()
    active = [0, 0]  # now, most at once

    def run_batch(slot, reqs, bid):
        with lock:
            active[0] += 1
            active[1] = max(active[1], active[0])
            runs.append((bid, slot.idx, [r.rid for r in reqs]))
        time.sleep(hold)
        with lock:
            active[0] -= 1
        for r in reqs:
            r.done.set()
        with srv.cv:
            slot.busy = False
            srv.completed.extend(reqs)
            srv.cv.notify_all()

    srv._run_batch = run_batch
    srv.running = True
    t = threading.Thread(target=srv._dispatch, daemon=True)
    t.start()
    srv.threads = [t]
    return srv, runs, active


def test_dispatch_packs_queued_requests_in_order():
    """Queued requests are taken in arrival order and packed into one batch while
    their proteomes fit max_batch; at most `slots` batches run at once."""
    srv, runs, active = _server(slots=2, max_batch=64, hold=0.2)
    sizes = [40, 20, 10, 64, 1, 63, 5]
    with srv.cv:  # queue everything before the dispatcher can take any
        reqs = [Request(i, _Q(n)) for i, n in enumerate(sizes)]
        srv.queue.extend(reqs)
        srv.cv.notify_all()
    for r in reqs:
        assert r.done.wait(10)
    srv.stop()
    assert [rid for _, _, ids in sorted(runs) for rid in ids] == list(range(len(sizes)))
    assert [ids for _, _, ids in sorted(runs)] == [[0, 1], [2], [3], [4, 5], [6]]
    for _, _, ids in runs:
        assert sum(sizes[i] for i in ids) <= 64
    assert active[1] == 2
    assert srv.batches == 5 and len(srv.completed) == len(sizes)


def test_dispatch_single_slot_runs_one_batch_at_a_time():
    srv, runs, active = _server(slots=1, max_batch=8, hold=0.02)
    reqs = [srv.submit(Request(i, _Q(3))) for i in range(6)]
    for r in reqs:
        assert r.done.wait(10)
    srv.stop()
    assert active[1] == 1
    assert sorted(rid for _, _, ids in runs for rid in ids) == list(range(6))
    assert all(sum(3 for _ in ids) <= 8 for _, _, ids in runs)


def test_failed_admission_releases_nothing():
    """A batch whose HBM estimate exceeds the budget fails (each request gets the
    error) without touching what the budget holds for others."""
    srv = ServingEngine(slots=1, budget_bytes=100.0)
    srv.db = SimpleNamespace(snapshot=lambda: 10)
    srv.budget.reserve(30.0)  # held by someone else
    srv._estimate = lambda reqs, db_n: 1000.0
    slot = SimpleNamespace(idx=0, busy=True)
    reqs = [Request(0, _Q(2)), Request(1, _Q(3))]
    srv._run_batch(slot, reqs, 0)
    assert all(r.done.is_set() and "MemoryError" in r.error for r in reqs)
    assert srv.budget.used == 30.0
    assert not slot.busy and srv.completed == reqs


# -- appends become visible only once their copies have completed -------------------

import torch  # noqa: E402

from rocket_gb300.engine import Arena, EngineConfig  # noqa: E402
from rocket_gb300.serve import Database  # noqa: E402


class _CopyDone:
    """Stands in for the CUDA event recorded behind an append's copies."""
    made = []

    def __init__(self):
        self.done = False
        _CopyDone.made.append(self)

    def record(self, stream=None):
        pass

    def query(self):
        return self.done


def _staged(nnz, R):
    off = np.concatenate([[0], np.cumsum(nnz)]).astype(np.int64)
    used = int(off[-1])
    keys = torch.arange(used, dtype=torch.int32)
    vals = torch.ones(used, dtype=torch.float32)
    return Arena("protein", 3, keys, vals, torch.from_numpy(off.copy()),
                 np.asarray(nnz, np.int64), off, np.ones(len(nnz)), n=len(nnz),
                 roff=torch.zeros((len(nnz), R + 1), dtype=torch.int32), R=R, indexed=len(nnz))


def test_appends_visible_after_their_copies(monkeypatch):
    """A batch's snapshot counts an append's vectors only once the copies queued
    behind the appending slot's work have completed, and in append order: a later
    append that completes first waits for the earlier one."""
    monkeypatch.setattr(torch.cuda, "Event", _CopyDone)
    _CopyDone.made = []
    db = Database("protein", 3, 1000, 10, EngineConfig(segments=4, compress=False), "cpu")
    assert db.append(_staged([4, 8], db.R), None)
    assert db.arena.n == 2 and db.snapshot() == 0  # copies in flight
    first, = _CopyDone.made
    first.done = True
    assert db.snapshot() == 2
    assert db.append(_staged([12], db.R), None)
    assert db.append(_staged([4, 4, 4], db.R), None)
    second, third = _CopyDone.made[1:]
    third.done = True
    assert db.arena.n == 6 and db.snapshot() == 2  # the earlier append is still in flight
    second.done = True
    assert db.snapshot() == 6
    # the arena holds the vectors in append order, each on its own offsets
    assert list(db.arena.off) == [0, 4, 12, 24, 28, 32, 36]
    assert list(db.arena.vec_off[:7].numpy()) == list(db.arena.off)
    assert list(db.arena.nnz) == [4, 8, 12, 4, 4, 4]
    # over capacity: refused, nothing published
    assert not db.append(_staged([4] * 5, db.R), None)
    assert db.refused == 5 and db.snapshot() == 6 and len(_CopyDone.made) == 3
