"""Serving: a device-resident database of composition vectors answering
queries of newly arriving proteomes.

Each query (one or more proteomes) is vector-built on the device, compared
against every database vector, and then appended to the database.  This is the
long-running counterpart of Rocket's per-item pipeline, where a DeviceWorker
builds items into device cache slots and correlates pairs of resident items
(rocket/scheduler/DeviceWorker.java:118-323, rocket/cache/DeviceCache.java):

* Admission by HBM budget: the database reserves its arena once; every batch
  reserves an estimate of its working memory (build scratch, staged vectors,
  window index, partial blocks, result matrix) and waits while the total would
  exceed the budget.
* Continuous batching: a dispatcher hands work to ``slots`` workers, each with
  its own CUDA stream.  Whenever a slot frees up, all queued requests that fit
  in one batch (``max_batch`` proteomes) are merged into its next batch, so
  requests that arrive while others run join the next free slot, and batches
  of different slots overlap on the device.
* Results do not depend on the mix: rows are the batch's query vectors,
  columns the database vectors, and the key-space segmentation is fixed
  (EngineConfig.segments), so every (query, database) pair is summed in the
  same order whether its query ran alone or with others.
* Appends copy the staged vectors into the database arena (preallocated to its
  share of the budget, so concurrent batches reading older entries are never
  disturbed) and extend the window index; a later batch's snapshot includes them
  once those copies have completed on the device.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import threading
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from . import _native
from .engine import Arena, BatchBuilder, EngineConfig, PairEngine, key_limit
from .synth import Proteomes


@dataclass
class Request:
    rid: int
    proteomes: Proteomes
    append: bool = True
    t_arrival: float = 0.0
    t_start: float = 0.0
    t_done: float = 0.0
    db_n: int = 0                       # database vectors this request was compared against
    result: Optional[np.ndarray] = None  # C[query, db] (float64)
    batch_id: int = -1
    error: Optional[str] = None
    done: threading.Event = field(default_factory=threading.Event)

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrival

    def distances(self) -> np.ndarray:
        return (1.0 - self.result) * 0.5


class Budget:
    """HBM accounting: reserve() blocks while the total would exceed the budget."""

    def __init__(self, total: float):
        self.total = float(total)
        self.used = 0.0
        self.peak = 0.0
        self.cv = threading.Condition()

    def reserve(self, nbytes: float, timeout: float = 600.0) -> None:
        with self.cv:
            if nbytes > self.total:  # would never fit, however much is released
                raise MemoryError(f"request needs {nbytes / 1e9:.1f} GB, budget {self.total / 1e9:.1f} GB")
            ok = self.cv.wait_for(lambda: self.used + nbytes <= self.total, timeout=timeout)
            if not ok:
                raise TimeoutError("HBM budget admission timed out")
            self.used += nbytes
            self.peak = max(self.peak, self.used)

    def release(self, nbytes: float) -> None:
        with self.cv:
            self.used -= nbytes
            self.cv.notify_all()


class Database:
    """Device-resident vectors with room to grow (a preallocated arena)."""

    def __init__(self, alphabet: str, k: int, capacity_entries: int, capacity_vectors: int,
                 cfg: EngineConfig, device):
        self.device = device
        self.cfg = cfg
        W = 1 << cfg.wshift
        self.R = (key_limit(alphabet, k) + W - 1) // W
        self.arena = Arena(alphabet, k,
                           torch.empty(capacity_entries, dtype=torch.int32, device=device),
                           torch.empty(capacity_entries, dtype=torch.float32, device=device),
                           torch.zeros(capacity_vectors + 1, dtype=torch.int64, device=device),
                           np.zeros(0, np.int64), np.zeros(1, np.int64), np.zeros(0, np.float64))
        self.arena.roff = torch.empty((capacity_vectors, self.R + 1), dtype=torch.int32,
                                      device=device)
        self.arena.wshift, self.arena.R = cfg.wshift, self.R
        self.capacity_entries = capacity_entries
        self.capacity_vectors = capacity_vectors
        self.lock = threading.Lock()
        self.appended = 0
        self.refused = 0
        self.visible = 0  # vectors a batch may read: their copies have completed
        # (vector count after an append, event recorded behind that append's copies),
        # in append order
        self.pending: collections.deque = collections.deque()

    def bytes_reserved(self) -> float:
        return self.capacity_entries * 8.0 + self.capacity_vectors * (self.R + 1) * 4.0

    def snapshot(self) -> int:
        """Vectors a new batch compares against.  An append's vectors count only once
        its copies have completed on the device: they are queued on the appending
        slot's stream behind that slot's own pair kernel, while a batch of another
        slot runs on its own stream and would otherwise read entries, offsets and
        window rows still in flight."""
        with self.lock:
            while self.pending and self.pending[0][1].query():
                self.visible = self.pending.popleft()[0]
            return self.visible

    def append(self, staged: Arena, stream: torch.cuda.Stream) -> bool:
        """Copies the staged vectors (built and indexed) behind the current ones."""
        with self.lock:
            a = self.arena
            n_new = staged.n
            used = staged.used
            if a.n + n_new > self.capacity_vectors or a.used + used > self.capacity_entries:
                self.refused += n_new
                return False
            base = a.used
            with torch.cuda.stream(stream):
                a.keys[base:base + used].copy_(staged.keys[:used], non_blocking=True)
                a.values[base:base + used].copy_(staged.values[:used], non_blocking=True)
                a.vec_off[a.n:a.n + n_new + 1].copy_(staged.vec_off[:n_new + 1] + base,
                                                      non_blocking=True)
                # window offsets are relative to each vector's start: copied as is
                a.roff[a.n:a.n + n_new].copy_(staged.roff[:n_new], non_blocking=True)
                done = torch.cuda.Event()
                done.record(stream)
            self.pending.append((a.n + n_new, done))
            a.nnz = np.concatenate([a.nnz, staged.nnz[:n_new]])
            a.norms = np.concatenate([a.norms, staged.norms[:n_new]])
            a.off = np.concatenate([a.off[:a.n + 1], base + staged.off[1:n_new + 1]])
            a.n += n_new
            a.indexed = a.n
            self.appended += n_new
            return True


class _Slot:
    def __init__(self, idx: int, server: "ServingEngine"):
        self.idx = idx
        self.server = server
        self.stream = torch.cuda.Stream(device=server.device)
        self.builder = BatchBuilder(server.alphabet, server.k, device=server.device,
                                    max_batch=server.max_batch)
        self.staged: Optional[Arena] = None
        self.engine: Optional[PairEngine] = None
        self.busy = False


class ServingEngine:
    def __init__(self, alphabet: str = "protein", k: int = 6, budget_bytes: float = 120e9,
                 slots: int = 2, max_batch: int = 64, cfg: Optional[EngineConfig] = None,
                 device=None):
        self.alphabet = alphabet
        self.k = k
        self.device = torch.device(device if device is not None else "cuda")
        self.budget = Budget(budget_bytes)
        self.max_batch = max_batch
        # queries and the database are separate arenas: the pair kernel reads raw keys
        self.cfg = dataclasses.replace(cfg or EngineConfig(segments=16), compress=False)
        if self.cfg.segments <= 0:
            raise ValueError("serving needs a fixed number of key segments")
        self.nslots = slots
        self.db: Optional[Database] = None
        self.queue: collections.deque = collections.deque()
        self.cv = threading.Condition()
        self.running = False
        self.batches = 0
        self.pairs = 0
        self.completed: List[Request] = []
        self.threads: List[threading.Thread] = []
        self.slots: List[_Slot] = []
        self.tuned: Optional[dict] = None

    # -- database -----------------------------------------------------------
    def load(self, proteomes: Proteomes, capacity_vectors: Optional[int] = None,
             capacity_entries: Optional[int] = None) -> Database:
        """Builds the database from host proteomes into a preallocated arena."""
        lens = proteomes.lengths()
        if capacity_vectors is None:
            capacity_vectors = 2 * len(proteomes)
        if capacity_entries is None:
            capacity_entries = int(2 * np.sum(8 * lens + 64))
        db = Database(self.alphabet, self.k, capacity_entries, capacity_vectors, self.cfg,
                      self.device)
        self.budget.reserve(db.bytes_reserved())
        builder = BatchBuilder(self.alphabet, self.k, device=self.device, max_batch=self.max_batch)
        stream = torch.cuda.current_stream(self.device)
        seq = torch.from_numpy(proteomes.data).to(self.device)
        # build into a staging arena of exactly the database's capacity class
        built = builder.build(seq, proteomes.offsets, stream=stream)
        eng = PairEngine(built, self.cfg)
        eng.ensure_index(stream)
        if not db.append(built, stream):
            raise MemoryError("database does not fit its capacity")
        torch.cuda.synchronize(self.device)
        db.appended = 0
        self.db = db
        return db

    def tune(self, widths=(128, 256), rows: int = 64, repeats: int = 2) -> dict:
        """Chooses the width of the pair items for query batches: a rectangle of the
        first ``rows`` database vectors against the whole database (the shape of a
        full query batch) is timed under each width and the fastest kept (the role of
        the reference's tuner, phylogenetics/tune.py:25-84, for serving).  The
        window width stays: the database's window index is built for it."""
        if self.db is None or self.db.arena.n == 0:
            raise RuntimeError("load a database first")
        db = self.db.arena
        n = db.n
        row_ids = np.arange(min(rows, n))
        out = torch.empty((len(row_ids), n), dtype=torch.float64, device=self.device)
        results = []
        for w in widths:
            cfg = dataclasses.replace(self.cfg, tile_cols=int(w))
            eng = PairEngine(db, cfg)
            plan = eng.plan_rect(row_ids, np.arange(n), ldc=n, col_arena=db)
            eng.run(plan, out, diagonal=False, col_arena=db)  # warm-up
            torch.cuda.synchronize(self.device)
            best = float("inf")
            for _ in range(repeats):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                eng.run(plan, out, diagonal=False, col_arena=db)
                e1.record()
                torch.cuda.synchronize(self.device)
                best = min(best, e0.elapsed_time(e1))
            results.append({"tile_cols": int(w), "ms": best})
        win = min(results, key=lambda r: r["ms"])
        self.cfg = dataclasses.replace(self.cfg, tile_cols=win["tile_cols"])
        self.tuned = dict(win, rows=len(row_ids), db=n, candidates=results)
        return self.tuned

    # -- request flow ----------------------------------------------------------
    def submit(self, req: Request) -> Request:
        req.t_arrival = req.t_arrival or time.perf_counter()
        with self.cv:
            self.queue.append(req)
            self.cv.notify_all()
        return req

    def start(self) -> None:
        if self.db is None:
            raise RuntimeError("load a database first")
        self.running = True
        self.slots = [_Slot(i, self) for i in range(self.nslots)]
        t = threading.Thread(target=self._dispatch, daemon=True)
        t.start()
        self.threads = [t]

    def stop(self, drain: bool = True) -> None:
        if drain:
            with self.cv:
                self.cv.wait_for(lambda: not self.queue and not any(s.busy for s in self.slots))
        with self.cv:
            self.running = False
            self.cv.notify_all()
        for t in self.threads:
            t.join(timeout=60)

    def _estimate(self, reqs: List[Request], db_n: int) -> float:
        lens = np.concatenate([r.proteomes.lengths() for r in reqs])
        nq = len(lens)
        cand = float(np.sum(np.minimum(8 * lens + 65536, key_limit(self.alphabet, self.k))))
        L = _native.load()
        scratch = float(L.phyloBuildBatchScratch(self.alphabet.encode(), self.k,
                                                 min(nq, self.max_batch), int(cand)))
        staged = float(np.sum(8 * lens + 64)) * 8.0
        roff = nq * (self.db.R + 1) * 4.0
        ti = self.cfg.tile_rows
        tj = self.cfg.tile_cols
        tiles = math.ceil(nq / ti) * math.ceil(max(db_n, 1) / tj)
        parts = tiles * self.cfg.segments * ti * tj * 8.0
        out = nq * max(db_n, 1) * 8.0
        return scratch + staged + roff + parts + out

    def _dispatch(self) -> None:
        while True:
            with self.cv:
                self.cv.wait_for(lambda: not self.running or
                                 (self.queue and any(not s.busy for s in self.slots)))
                if not self.running:
                    return
                slot = next(s for s in self.slots if not s.busy)
                batch = [self.queue.popleft()]
                total = len(batch[0].proteomes)
                while self.queue and total + len(self.queue[0].proteomes) <= self.max_batch:
                    r = self.queue.popleft()
                    batch.append(r)
                    total += len(r.proteomes)
                slot.busy = True
                bid = self.batches
                self.batches += 1
            th = threading.Thread(target=self._run_batch, args=(slot, batch, bid), daemon=True)
            th.start()

    def _run_batch(self, slot: _Slot, reqs: List[Request], bid: int) -> None:
        reserved = 0.0
        try:
            db_n = self.db.snapshot()
            need = self._estimate(reqs, db_n)
            self.budget.reserve(need)
            reserved = need  # released below only once actually reserved
            t0 = time.perf_counter()
            for r in reqs:
                r.t_start = t0
                r.batch_id = bid
            self._process(slot, reqs, db_n)
        except Exception as e:  # the request fails, the server keeps running
            for r in reqs:
                r.error = repr(e)
                r.t_done = time.perf_counter()
                r.done.set()
        finally:
            if reserved:
                self.budget.release(reserved)
            with self.cv:
                slot.busy = False
                self.completed.extend(reqs)
                self.cv.notify_all()

    def _process(self, slot: _Slot, reqs: List[Request], db_n: int) -> None:
        dev = self.device
        st = slot.stream
        data = np.concatenate([r.proteomes.data for r in reqs])
        offs = [0]
        for r in reqs:
            o = r.proteomes.offsets
            offs.extend((offs[-1] + o[1:]).tolist())
        offs = np.asarray(offs, np.int64)
        nq = len(offs) - 1
        with torch.cuda.stream(st):
            host = torch.from_numpy(data).pin_memory()
            seq = torch.empty(host.numel(), dtype=torch.uint8, device=dev)
            seq.copy_(host, non_blocking=True)
            staged = slot.builder.build(seq, offs, arena=slot.staged.reset() if slot.staged else None,
                                        stream=st)
            slot.staged = staged
            if slot.engine is None:
                slot.engine = PairEngine(staged, self.cfg)
            eng = slot.engine
            eng.arena = staged
            eng.ensure_index(st)
            out = torch.empty((nq, max(db_n, 1)), dtype=torch.float64, device=dev)
            if db_n > 0:
                plan = eng.plan_rect(np.arange(nq), np.arange(db_n), ldc=db_n,
                                     col_arena=self.db.arena)
                eng.run(plan, out, stream=st, diagonal=False, col_arena=self.db.arena)
            out_h = torch.empty(out.shape, dtype=torch.float64).pin_memory()
            out_h.copy_(out, non_blocking=True)
        if any(r.append for r in reqs):
            # append only the proteomes of requests that asked for it
            keep = np.concatenate([np.full(len(r.proteomes), r.append) for r in reqs])
            if keep.all():
                self.db.append(staged, st)
            else:
                for i in np.flatnonzero(keep):
                    self._append_one(staged, int(i), st)
        st.synchronize()
        t_done = time.perf_counter()
        C = out_h.numpy()[:, :db_n]
        row = 0
        for r in reqs:
            n = len(r.proteomes)
            r.result = C[row:row + n].copy()
            r.db_n = db_n
            r.t_done = t_done
            row += n
            r.done.set()
        with self.cv:
            self.pairs += nq * db_n

    def _append_one(self, staged: Arena, i: int, st) -> None:
        one = Arena(staged.alphabet, staged.k, staged.keys[int(staged.off[i]):],
                    staged.values[int(staged.off[i]):],
                    staged.vec_off[i:i + 2] - int(staged.off[i]), staged.nnz[i:i + 1],
                    np.array([0, staged.off[i + 1] - staged.off[i]], np.int64),
                    staged.norms[i:i + 1], n=1, roff=staged.roff[i:i + 1], wshift=staged.wshift,
                    R=staged.R, indexed=1)
        self.db.append(one, st)


def percentile(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if len(xs) else float("nan")
