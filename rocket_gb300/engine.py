"""Batched composition-vector construction and the all-pair engine.

This is the batched counterpart of the reference's per-item pipeline
(DeviceWorker.loadInput -> preprocessInputGPU for every proteome, then
correlateGPU for every pair; rocket/scheduler/DeviceWorker.java:118-323):

* :class:`BatchBuilder` builds many proteomes per launch sequence into one
  device arena (keys | values | offsets), vectors padded to 4 entries so the
  pair kernel can read them with 16-byte loads.
* :class:`PairEngine` compares every pair of an arena (or a rectangle of row
  and column vectors).  Two algorithms: ``window`` (csrc/allpairs.cu, the
  default) densifies 16 row vectors per key window in shared memory and streams
  column vectors against them; ``postings`` (csrc/postings.cu) regroups each key
  window of a block of row vectors and a block of column vectors by key and forms
  only the products of shared keys, with exact integer sums.  The planner
  sorts vectors by size, cuts the pair matrix into tiles and the key space into
  segments, estimates each item's cost (for postings from the products of the
  tile's vector sizes) and hands items out longest first.

All device memory is held in torch tensors; every kernel is this project's
own (libphylogenetics.so).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np
import torch

from . import _native
from ._native import check

AP_TI = 16          # default rows per work item (16 or 32: selects the pair kernel)
AP_TJ = 128         # default column vectors per work item (512-thread CTAs)
NSYM = {"protein": 21, "DNA": 4}


def _p(t: torch.Tensor) -> int:
    return int(t.data_ptr())


def _stream_handle(stream: Optional[torch.cuda.Stream]) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def key_limit(alphabet: str, k: int) -> int:
    return NSYM[alphabet] ** k


def auto_tile_cols(n_cols: int) -> int:
    """Column vectors per work item for plans over ``n_cols`` columns.  Items of 256
    columns (two lanes per column) spread each window's row scatter and barriers
    over twice the columns, which pays once the row tiles' column spans are mostly
    full; in a triangle over fewer than 384 vectors most 256-column items would be
    half empty, and 128-column items keep more lanes busy."""
    return 256 if n_cols >= 384 else 128


# --------------------------------------------------------------------------
# arena
# --------------------------------------------------------------------------

@dataclass
class Arena:
    """Device-resident composition vectors: vector v is keys/values[off[v] : off[v] + nnz[v]]."""
    alphabet: str
    k: int
    keys: torch.Tensor          # int32 (uint32 bit patterns)
    values: torch.Tensor        # float32
    vec_off: torch.Tensor       # int64 [capacity_vectors + 1]
    nnz: np.ndarray             # int64 [n]
    off: np.ndarray             # int64 [n + 1] host copy of vec_off
    norms: np.ndarray           # float64 [n]
    n: int = 0
    roff: Optional[torch.Tensor] = None
    wshift: int = 0
    R: int = 0
    indexed: int = 0            # vectors covered by roff
    rkeys: Optional[torch.Tensor] = None   # dense key ranks (pair kernel input), or None
    union_bits: Optional[torch.Tensor] = None  # key bitmap the batched build marks
    union_n: int = 0            # vectors whose keys are marked in union_bits
    rank_limit: int = 0         # union size of the ranked vectors
    ranked: int = 0             # vectors covered by rkeys (ranks of all of them change together)
    index_on_ranks: bool = False

    def index_state(self):
        return (self.roff, self.wshift, self.R, self.indexed, self.rkeys, self.rank_limit,
                self.ranked, self.index_on_ranks)

    def restore_index(self, st) -> None:
        (self.roff, self.wshift, self.R, self.indexed, self.rkeys, self.rank_limit, self.ranked,
         self.index_on_ranks) = st

    def pair_keys(self) -> torch.Tensor:
        """The keys the window index and the pair kernel read."""
        return self.rkeys if self.index_on_ranks else self.keys

    @property
    def used(self) -> int:
        return int(self.off[self.n])

    def reset(self) -> "Arena":
        """Forgets the vectors but keeps the device buffers for reuse."""
        self.n = 0
        self.nnz = np.zeros(0, np.int64)
        self.off = np.zeros(1, np.int64)
        self.norms = np.zeros(0, np.float64)
        self.indexed = 0
        self.ranked = 0
        if self.union_bits is not None:
            self.union_bits.zero_()
        self.union_n = 0
        return self

    def vector(self, v: int):
        o, m = int(self.off[v]), int(self.nnz[v])
        return self.keys[o:o + m], self.values[o:o + m]

    def host_vector(self, v: int):
        k, x = self.vector(v)
        return k.cpu().numpy().view(np.uint32), x.cpu().numpy()


def _grow(t: torch.Tensor, n: int) -> torch.Tensor:
    if t.numel() >= n:
        return t
    new = torch.empty(int(n), dtype=t.dtype, device=t.device)
    new[:t.numel()].copy_(t)
    return new


class BatchBuilder:
    """Builds composition vectors of many proteomes into an :class:`Arena`.

    Batches of up to ``max_batch`` proteomes; with ``overlap`` two batches are in
    flight at once, on the caller's stream and a second stream with their own
    scratch, so that one batch's kernels fill the gaps of the other's."""

    def __init__(self, alphabet: str = "protein", k: int = 6, device=None, max_batch: int = 24,
                 overlap: bool = True):
        self.alphabet = alphabet
        self.k = k
        self.device = torch.device(device if device is not None else "cuda")
        self.max_batch = max_batch
        self.overlap = overlap
        self.L = _native.load()
        self._scratch = [None, None]
        self._summary = [None, None]
        self._side = None
        self._copy = None  # stream of the per-batch residue copies (build(host=...))
        self.launches = 0

    def _scratch_for(self, slot: int, B: int, cand_cap: int) -> torch.Tensor:
        n = int(self.L.phyloBuildBatchScratch(self.alphabet.encode(), self.k, B, cand_cap))
        if n < 0:
            raise ValueError(f"invalid build geometry: alphabet={self.alphabet} k={self.k}")
        if self._scratch[slot] is None or self._scratch[slot].numel() < n:
            if self._scratch[slot] is not None:
                torch.cuda.synchronize(self.device)  # queued work may still use the old one
            self._scratch[slot] = None
            self._scratch[slot] = torch.empty(n, dtype=torch.uint8, device=self.device)
        return self._scratch[slot]

    def _summary_for(self, slot: int) -> torch.Tensor:
        n = int(self.L.phyloBuildBatchSummaryBytes(self.max_batch))
        if self._summary[slot] is None or self._summary[slot].numel() < n:
            self._summary[slot] = torch.empty(n, dtype=torch.uint8).pin_memory()
        return self._summary[slot]

    def new_arena(self, capacity_entries: int, capacity_vectors: int) -> Arena:
        keys = torch.empty(max(int(capacity_entries), 4), dtype=torch.int32, device=self.device)
        vals = torch.empty(max(int(capacity_entries), 4), dtype=torch.float32, device=self.device)
        off = torch.zeros(capacity_vectors + 1, dtype=torch.int64, device=self.device)
        return Arena(self.alphabet, self.k, keys, vals, off, np.zeros(0, np.int64),
                     np.zeros(1, np.int64), np.zeros(0, np.float64))

    def build(self, seq: torch.Tensor, seq_off: np.ndarray, arena: Optional[Arena] = None,
              stream: Optional[torch.cuda.Stream] = None,
              host: Optional[torch.Tensor] = None) -> Arena:
        """Builds the proteomes seq[seq_off[i]:seq_off[i+1]] (seq on the device) and
        appends them to ``arena`` (a new one if None).  Work is ordered on ``stream``
        (default: the current stream): later work on it sees the whole build.

        ``host``: the same residues in pinned host memory.  Each batch's range is then
        copied into ``seq`` on a copy stream just ahead of the batch, so the copies of
        later batches overlap the build of earlier ones (the pinned, double-buffered
        ingest of DeviceWorker.java:118-157)."""
        seq_off = np.asarray(seq_off, np.int64)
        n = len(seq_off) - 1
        lens = np.diff(seq_off)
        s_obj = stream if stream is not None else torch.cuda.current_stream(self.device)
        if host is not None and (host.device.type != "cpu" or host.numel() < seq_off[-1]):
            raise ValueError("host residues: a CPU tensor covering seq_off")
        with torch.cuda.stream(s_obj):
            # allocated on the stream the build runs on, so that freeing the arena is
            # ordered after the work queued there
            if arena is None:
                arena = self.new_arena(int(np.sum(8 * lens + 64)) + 1024, n)
            if arena.vec_off.numel() < arena.n + n + 1:
                arena.vec_off = _grow(arena.vec_off, arena.n + n + 1)
            self._build_into(arena, seq, seq_off, lens, s_obj, host)
        return arena

    def _build_into(self, arena: Arena, seq: torch.Tensor, seq_off: np.ndarray, lens: np.ndarray,
                    stream: torch.cuda.Stream, host: Optional[torch.Tensor] = None) -> None:
        n = len(seq_off) - 1
        d_seq_off_all = torch.from_numpy(seq_off).to(self.device, non_blocking=False)
        batches = [(f, min(self.max_batch, n - f)) for f in range(0, n, self.max_batch)]
        if host is not None and len(batches) == 1:  # nothing to overlap: one copy, in order
            seq[:int(seq_off[-1])].copy_(host[:int(seq_off[-1])], non_blocking=True)
            host = None
        if host is not None:  # copies wait for earlier work on the stream (it may read seq)
            if self._copy is None:
                self._copy = torch.cuda.Stream(self.device)
            ready = torch.cuda.Event()
            ready.record(stream)
            self._copy.wait_event(ready)
        overlap = self.overlap and len(batches) > 1
        streams = [stream]
        if overlap:
            if self._side is None:
                self._side = torch.cuda.Stream(self.device)
            start = torch.cuda.Event()
            start.record(stream)
            self._side.wait_event(start)
            streams.append(self._side)
        keep = []  # device tensors used by queued work, held until the build is joined

        def enqueue(bi: int) -> dict:
            first, B = batches[bi]
            slot = bi % len(streams)
            st = streams[slot]
            lens_b = lens[first:first + B]
            cand = int(np.sum(np.minimum(8 * lens_b + 65536, key_limit(self.alphabet, self.k))))
            base = int(seq_off[first])
            end = int(seq_off[first + B])
            if host is not None and end > base:  # this batch's residues, ahead of its build
                with torch.cuda.stream(self._copy):
                    seq[base:end].copy_(host[base:end], non_blocking=True)
                copied = torch.cuda.Event()
                copied.record(self._copy)
                st.wait_event(copied)
            with torch.cuda.stream(st):
                d_off = d_seq_off_all[first:first + B + 1] - base
                scr = self._scratch_for(slot, B, cand)
            d_seq = seq[base:end]
            keep.append(d_off)
            summ = self._summary_for(slot)
            check(self.L.phyloBuildBatchPlanAsync(
                int(st.cuda_stream), _p(scr), scr.numel(), self.alphabet.encode(), self.k, B,
                _p(d_seq) if d_seq.numel() else _p(seq), _p(d_off), cand, summ.data_ptr()))
            ev = torch.cuda.Event()
            ev.record(st)
            return dict(bi=bi, slot=slot, st=st, B=B, first=first, cand=cand, ev=ev, scr=scr,
                        d_off=d_off, d_seq=d_seq)

        def finish(p: dict) -> None:
            B, st, scr = p["B"], p["st"], p["scr"]
            p["ev"].synchronize()
            raw = self._summary[p["slot"]].numpy()
            nnz = raw[:8 * B].view(np.int64).copy()
            norms = raw[8 * B:16 * B].view(np.float64).copy()
            needed = int(raw[16 * B:16 * B + 8].view(np.int64)[0])
            status = int(raw[16 * B + 8:16 * B + 12].view(np.uint32)[0])
            cand = p["cand"]
            if status & 2:  # candidate capacity: redo this batch with the exact count
                torch.cuda.synchronize(self.device)
                cand = needed
                with torch.cuda.stream(st):
                    scr = self._scratch_for(p["slot"], B, cand)
                d_seq = p["d_seq"]
                total_cand = np.zeros(1, np.int64)
                check(self.L.phyloBuildBatchPlan(
                    int(st.cuda_stream), _p(scr), scr.numel(), self.alphabet.encode(), self.k, B,
                    _p(d_seq) if d_seq.numel() else _p(seq), _p(p["d_off"]), cand,
                    nnz.ctypes.data, total_cand.ctypes.data))
                check(self.L.phyloBuildBatchNorms(int(st.cuda_stream), _p(scr), scr.numel(),
                                                  self.alphabet.encode(), self.k, B, cand,
                                                  norms.ctypes.data))
            self.launches += int(self.L.phyloBuildLaunchesPerBatch())
            padded = (nnz + 3) // 4 * 4
            need = arena.used + int(padded.sum()) + 4
            if arena.keys.numel() < need:
                torch.cuda.synchronize(self.device)  # queued emits write the old buffers
                cap = int(max(need, arena.keys.numel() * 1.5))
                arena.keys = _grow(arena.keys, cap)
                arena.values = _grow(arena.values, cap)
                if arena.rkeys is not None:
                    arena.rkeys = None
                if st is not stream:
                    # the copies into the new buffers run on the build's stream and
                    # cover the range this batch's emit (on the side stream) writes
                    grown = torch.cuda.Event()
                    grown.record(stream)
                    st.wait_event(grown)
            # mark the union bitmap for dense key ranks while every vector is marked
            mark = arena.union_n == arena.n
            if mark and arena.union_bits is None:
                nb = int(self.L.phyloKeyRankBitmapBytes(key_limit(self.alphabet, self.k)))
                with torch.cuda.stream(stream):
                    arena.union_bits = torch.zeros(nb // 4, dtype=torch.int32, device=self.device)
                if overlap:
                    ev = torch.cuda.Event()
                    ev.record(stream)
                    st.wait_event(ev)
            check(self.L.phyloBuildBatchEmit(
                int(st.cuda_stream), _p(scr), scr.numel(), self.alphabet.encode(), self.k, B, cand,
                _p(arena.keys), _p(arena.values), _p(arena.vec_off[arena.n:]), arena.used,
                _p(arena.union_bits) if mark else 0))
            if mark:
                arena.union_n += B
            arena.nnz = np.concatenate([arena.nnz, nnz])
            arena.norms = np.concatenate([arena.norms, norms])
            new_off = arena.used + np.concatenate([[0], np.cumsum(padded)])
            arena.off = np.concatenate([arena.off[:arena.n], new_off])
            arena.n += B

        prev = None
        for bi in range(len(batches)):
            cur = enqueue(bi)
            if prev is not None:
                finish(prev)
            if not overlap:
                finish(cur)
                cur = None
            prev = cur
        if prev is not None:
            finish(prev)
        if overlap:
            done = torch.cuda.Event()
            done.record(self._side)
            stream.wait_event(done)
            # tensors the side stream used stay alive until it has finished with them
            for t in keep:
                t.record_stream(self._side)


def upload_proteomes(data: np.ndarray, device=None, pinned: Optional[torch.Tensor] = None,
                     non_blocking: bool = True) -> torch.Tensor:
    """Host residue bytes -> device tensor (through pinned memory)."""
    h = torch.from_numpy(np.ascontiguousarray(data))
    if pinned is None:
        pinned = h.pin_memory()
    else:
        pinned[:h.numel()].copy_(h)
    d = torch.empty(h.numel(), dtype=torch.uint8, device=device or "cuda")
    d.copy_(pinned[:h.numel()], non_blocking=non_blocking)
    return d


# --------------------------------------------------------------------------
# pair engine
# --------------------------------------------------------------------------

@dataclass
class PairPlan:
    rowids: torch.Tensor       # int32 device
    colids: torch.Tensor
    tiles: torch.Tensor        # int32 device [ntiles, 4] (window) or [ntiles, 8] (postings)
    items: torch.Tensor        # int32 device [nitems, 8]
    ntiles: int
    nitems: int
    S: int                     # segments per tile (window); the largest per-tile count (postings)
    upper: bool
    mirror: bool
    ldc: int
    est: np.ndarray            # estimated cost per item (launch order)
    pairs: int                 # valid pairs covered
    host_items: np.ndarray = field(default=None)
    diag: bool = False         # the tiles also cover every vector with itself
    algorithm: str = "window"
    nparts: int = 0            # partial blocks the items write
    host_rowids: np.ndarray = field(default=None)
    host_colids: np.ndarray = field(default=None)
    host_tiles: np.ndarray = field(default=None)
    item_tile: np.ndarray = field(default=None)  # tile of each item (launch order)
    item_share: np.ndarray = field(default=None)  # fraction of its tile's windows per item


@dataclass
class EngineConfig:
    algorithm: str = "window"  # "window" or "postings" (key-major, exact integer sums)
    wshift: Optional[int] = None  # key window = 2^wshift ranks (default 9 postings, 11 window)
    block: int = 128         # postings: vectors per side of a work item (128 or 64)
    tile_rows: int = AP_TI   # row vectors per work item (16 or 32)
    tile_cols: int = AP_TJ   # column vectors per work item (128, 64 or 32; 64 with 32 rows)
    fold: int = 28           # products per FP32 accumulator between compensated folds:
                             # |dC| <= (fold + 2) 2^-24 for unit vectors -> |dD| <= 8.9e-7
    items_per_cta: int = 8   # work items per persistent CTA (the tuner's 16 x 256 and
                             # 16 x 128 window entries use 16: on 1,024 uneven proteomes
                             # the pair kernel took 773 / 555 / 551 ms at 4 / 8 / 16)
    min_windows_per_item: int = 64
    segments: int = 0        # key segments per tile; 0 = chosen from the plan size.  A fixed
                             # value makes each pair's arithmetic independent of the plan.
    compress: bool = True    # run the pair kernel on dense key ranks (one arena only)

    def __post_init__(self):
        if self.algorithm not in ("postings", "window"):
            raise ValueError(f"unknown pair algorithm {self.algorithm!r}")
        if self.wshift is None:
            self.wshift = 9 if self.algorithm == "postings" else 11


class PairEngine:
    def __init__(self, arena: Arena, config: Optional[EngineConfig] = None):
        self.arena = arena
        self.cfg = config or EngineConfig()
        self.L = _native.load()
        self.device = arena.keys.device
        ctas = ctypes.c_int(0)
        if self.cfg.algorithm == "postings":
            if self.L.phyloPostingsCapacity(self.cfg.block, self.cfg.wshift) < 0:
                raise ValueError(f"unsupported postings block {self.cfg.block} / window shift "
                                 f"{self.cfg.wshift} (blocks 128 or 64)")
            check(self.L.phyloPostingsPrepare(self.cfg.block, self.cfg.wshift, ctypes.byref(ctas)))
        else:
            if self.L.phyloPairsSmemBytes(self.cfg.wshift, self.cfg.tile_rows,
                                          self.cfg.tile_cols) < 0:
                raise ValueError(f"unsupported pair tile {self.cfg.tile_rows} x "
                                 f"{self.cfg.tile_cols} (16 x 256, 16 x 128, 16 x 64, 16 x 32 "
                                 "or 32 x 64)")
            check(self.L.phyloPairsPrepare(self.cfg.wshift, self.cfg.tile_rows,
                                           self.cfg.tile_cols, ctypes.byref(ctas)))
        self.ctas_per_sm = max(1, ctas.value)
        props = torch.cuda.get_device_properties(self.device)
        self.sms = props.multi_processor_count
        self.grid = self.sms * self.ctas_per_sm
        self.counter = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.part = None
        self.launches = 0
        self.cmp_scratch = None
        self.self_part = None
        self._rank_scratch = None
        self._rank_marked = False  # the last rank prefix used the build's union bitmap

    # -- window index ------------------------------------------------------
    def ensure_index(self, stream=None) -> None:
        """Builds (or extends to newly appended vectors) the window index; with
        ``compress``, first replaces the keys by their ranks in the union of the
        arena's keys (recomputed for all vectors when vectors were appended).
        Buffers are allocated, filled and read back on ``stream``, the stream the
        index kernels run on."""
        with torch.cuda.stream(stream):  # no-op for None: the current stream
            self._ensure_index(stream)

    def _ensure_index(self, stream) -> None:
        a = self.arena
        W = 1 << self.cfg.wshift
        st = _stream_handle(stream)
        rerank = self.cfg.compress and (a.rkeys is None or a.ranked != a.n)
        if rerank:
            self._rank_prefix(a, st)
        limit = a.rank_limit if self.cfg.compress else key_limit(a.alphabet, a.k)
        R = max(1, (limit + W - 1) // W)
        if (a.roff is None or a.wshift != self.cfg.wshift or a.R != R
                or a.index_on_ranks != self.cfg.compress):
            a.roff = torch.empty((max(a.n, 1), R + 1), dtype=torch.int32, device=self.device)
            a.wshift, a.R, a.indexed = self.cfg.wshift, R, 0
            a.index_on_ranks = self.cfg.compress
        if a.roff.shape[0] < a.n:
            new = torch.empty((int(a.n * 1.5) + 1, R + 1), dtype=torch.int32, device=self.device)
            new[:a.roff.shape[0]].copy_(a.roff)
            a.roff = new
        if rerank:
            # every vector's ranks may have changed: ranks and index in one pass
            maxlen = int(np.max(np.diff(a.off[:a.n + 1]))) if a.n else 1
            check(self.L.phyloKeyRankIndex(
                st, _p(self._rank_scratch), self._rank_scratch.numel(),
                key_limit(a.alphabet, a.k), _p(a.keys), _p(a.vec_off), a.n, maxlen,
                int(a.off[a.n] - a.off[0]), _p(a.union_bits) if self._rank_marked else 0,
                self.cfg.wshift, R, _p(a.rkeys), _p(a.roff)))
            entries = int(a.off[a.n] - a.off[0])
            flat = entries > 0 and -(-maxlen // 1024) * a.n > 2 * -(-entries // 1024)
            self.launches += 2 if flat else 1
            a.ranked = a.indexed = a.n
        if a.indexed < a.n:
            maxlen = int(np.max(np.diff(a.off[a.indexed:a.n + 1])))
            check(self.L.phyloWindowIndex(
                st, _p(a.pair_keys()), _p(a.vec_off[a.indexed:]), a.n - a.indexed,
                self.cfg.wshift, R, maxlen, _p(a.roff[a.indexed])))
            self.launches += 1
            a.indexed = a.n

    def _rank_prefix(self, a: Arena, st: int) -> None:
        """Union bitmap prefix of the arena's keys (in the rank scratch) and the
        union size; the ranks themselves come with the window index."""
        limit = key_limit(a.alphabet, a.k)
        nb = int(self.L.phyloKeyRankScratch(limit))
        if self._rank_scratch is None or self._rank_scratch.numel() < nb:
            self._rank_scratch = torch.empty(nb, dtype=torch.uint8, device=self.device)
        if a.rkeys is None or a.rkeys.numel() < a.keys.numel():
            a.rkeys = torch.empty(a.keys.numel(), dtype=torch.int32, device=self.device)
        union = torch.zeros(1, dtype=torch.int64, device=self.device)
        maxlen = int(np.max(np.diff(a.off[:a.n + 1]))) if a.n else 1
        self._rank_marked = a.union_bits is not None and a.union_n == a.n
        check(self.L.phyloKeyRanks(st, _p(self._rank_scratch), self._rank_scratch.numel(), limit,
                                   _p(a.keys), _p(a.vec_off), a.n, maxlen,
                                   _p(a.union_bits) if self._rank_marked else 0, 0, _p(union)))
        self.launches += 4 if self._rank_marked else 5
        a.rank_limit = int(union.cpu().item())  # synchronises: the window count depends on it

    # -- planning ------------------------------------------------------------
    def _segments(self, ntiles: int) -> int:
        if self.cfg.segments > 0:
            return int(min(self.cfg.segments, max(1, self.arena.R)))
        target = self.cfg.items_per_cta * self.grid
        S = max(1, math.ceil(target / max(ntiles, 1)))
        return int(max(1, min(S, self.arena.R // self.cfg.min_windows_per_item)))

    def _tiles(self, nrows: int, ncols: int, triangle: bool):
        """(row0, nrow, col0, ncol, diag) over positions in the sorted row and
        column lists.  Window tiles of a triangle start at their first row's own
        vector, so every vector also meets itself (the self products, the diagonal
        of the reference's matrix, Main.java:196); postings tiles of a triangle are
        blocks i <= j, and a diagonal block holds each pair and self product once."""
        tiles = []
        if self.cfg.algorithm == "postings":
            B = self.cfg.block
            for r0 in range(0, nrows, B):
                for c0 in range(r0 if triangle else 0, ncols, B):
                    tiles.append((r0, min(B, nrows - r0), c0, min(B, ncols - c0),
                                  int(triangle and c0 == r0)))
            return tiles
        ti, tj = self.cfg.tile_rows, self.cfg.tile_cols
        for r0 in range(0, nrows, ti):
            nr = min(ti, nrows - r0)
            c = r0 if triangle else 0
            while c < ncols:
                nc = min(tj, ncols - c)
                tiles.append((r0, nr, c, nc, 0))
                c += nc
        return tiles

    # cost model of the postings kernel per tile (calibrated against the kernel's
    # per-item clock64 durations): products + entries regrouped + windows visited
    PB_COST_PRODUCT = 1.0
    PB_COST_ENTRY = 4.0
    PB_COST_WINDOW = 3000.0

    def tile_costs(self, rowids, colids, tiles, row_nnz, col_nnz) -> np.ndarray:
        """Estimated cost of each tile.  Postings: the nnz-product estimate of the
        shared-key products, sum over the tile's pairs of nnz_i * nnz_j / U (U =
        the size of the key space the kernel runs on), plus the entries regrouped
        and the windows visited.  Window kernel: its linear model (16 products per
        column entry, the row scatter and a cost per window)."""
        models = self.tile_cost_models(rowids, colids, tiles, row_nnz, col_nnz)
        return models["nnz_product"] if self.cfg.algorithm == "postings" else models["linear"]

    def tile_cost_models(self, rowids, colids, tiles, row_nnz, col_nnz) -> dict:
        """Both cost estimates per tile.  ``nnz_product``: the shared-key products a
        tile forms, sum over its pairs of nnz_i * nnz_j / U (U = the size of the key
        space the kernel runs on; a diagonal tile counts each pair once and every
        self product), plus the entries regrouped and the windows visited (the
        postings kernel's work).  ``linear``: the window kernel's work, 16 (or
        tile_rows) products per column entry, the row scatter and a cost per
        window."""
        a = self.arena
        R = a.R
        tl = np.asarray([t[:5] for t in tiles], np.int64).reshape(-1, 5)
        cr = np.concatenate([[0.0], np.cumsum(row_nnz[rowids].astype(np.float64))])
        cc = np.concatenate([[0.0], np.cumsum(col_nnz[colids].astype(np.float64))])
        sr = cr[tl[:, 0] + tl[:, 1]] - cr[tl[:, 0]]
        sc = cc[tl[:, 2] + tl[:, 3]] - cc[tl[:, 2]]
        U = float(max(a.rank_limit if a.index_on_ranks else key_limit(a.alphabet, a.k), 1))
        q = np.concatenate([[0.0], np.cumsum(row_nnz[rowids].astype(np.float64) ** 2)])
        sq = q[tl[:, 0] + tl[:, 1]] - q[tl[:, 0]]
        diag = tl[:, 4] == 1
        prod = np.where(diag, (sr * sr + sq) / (2.0 * U), sr * sc / U)
        ent = np.where(diag, sr, sr + sc)
        return {
            "nnz_product": (self.PB_COST_PRODUCT * prod + self.PB_COST_ENTRY * ent +
                            self.PB_COST_WINDOW * R),
            "linear": self.cfg.tile_rows * sc + 2.0 * sr + 64.0 * R,
        }

    def item_cost_models(self, plan: "PairPlan") -> dict:
        """Both estimates per item of ``plan`` (launch order): the tile's estimate
        times the item's share of the tile's windows."""
        tiles = [tuple(int(x) for x in t[:4]) + ((int(t[6]) if len(t) > 6 else 0),)
                 for t in plan.host_tiles]
        m = self.tile_cost_models(plan.host_rowids, plan.host_colids, tiles,
                                  self.arena.nnz, self.arena.nnz)
        return {k: v[plan.item_tile] * plan.item_share for k, v in m.items()}

    def _finish_plan(self, rowids, colids, tiles, upper, mirror, ldc, pairs,
                     row_nnz=None, col_nnz=None) -> PairPlan:
        a = self.arena
        ntiles = len(tiles)
        R = a.R
        row_nnz = a.nnz if row_nnz is None else row_nnz
        col_nnz = a.nnz if col_nnz is None else col_nnz
        rowids = np.asarray(rowids, np.int64)
        colids = np.asarray(colids, np.int64)
        cost = self.tile_costs(rowids, colids, tiles, row_nnz, col_nnz)
        tl = np.asarray([t[:5] for t in tiles], np.int64).reshape(-1, 5)
        if self.cfg.algorithm == "postings":
            # segments per tile in proportion to its cost, so that items cost about
            # the same; a tile's windows are split evenly among its segments
            if self.cfg.segments > 0:
                S_t = np.full(ntiles, min(self.cfg.segments, max(R, 1)), np.int64)
            else:
                target = cost.sum() / max(self.cfg.items_per_cta * self.grid, 1)
                S_t = np.clip(np.ceil(cost / max(target, 1e-9)), 1, max(R, 1)).astype(np.int64)
            part0 = np.concatenate([[0], np.cumsum(S_t)])
            t_of = np.repeat(np.arange(ntiles, dtype=np.int64), S_t)
            s_of = np.arange(len(t_of), dtype=np.int64) - part0[t_of]
            items = np.empty((len(t_of), 8), np.int64)
            items[:, 0:4] = tl[t_of, 0:4]
            items[:, 4] = s_of * R // S_t[t_of]
            items[:, 5] = (s_of + 1) * R // S_t[t_of]
            items[:, 6] = np.arange(len(t_of), dtype=np.int64)
            items[:, 7] = tl[t_of, 4]
            est = cost[t_of] / S_t[t_of]
            host_tiles = np.zeros((ntiles, 8), np.int64)
            host_tiles[:, 0:4] = tl[:, 0:4]
            host_tiles[:, 4] = part0[:-1]
            host_tiles[:, 5] = S_t
            host_tiles[:, 6] = tl[:, 4]
            S = int(S_t.max()) if ntiles else 0
            nparts = int(part0[-1])
        else:
            S = self._segments(ntiles)
            # item t * S + s: tile t over windows [s R / S, (s + 1) R / S)
            t_of = np.repeat(np.arange(ntiles, dtype=np.int64), S)
            s_of = np.tile(np.arange(S, dtype=np.int64), ntiles)
            items = np.empty((ntiles * S, 8), np.int64)
            items[:, 0:4] = tl[t_of, 0:4]
            items[:, 4] = s_of * R // S
            items[:, 5] = (s_of + 1) * R // S
            items[:, 6] = np.arange(ntiles * S, dtype=np.int64)
            items[:, 7] = t_of
            est = cost[t_of] / S
            host_tiles = tl[:, 0:4].copy()
            nparts = ntiles * S
        share = (items[:, 5] - items[:, 4]) / max(R, 1)
        order = np.argsort(-est, kind="stable")
        items = items[order]
        est = est[order]
        item_tile = t_of[order]
        share = share[order]
        dev = self.device
        return PairPlan(
            rowids=torch.from_numpy(rowids.astype(np.int32)).to(dev),
            colids=torch.from_numpy(colids.astype(np.int32)).to(dev),
            tiles=torch.from_numpy(host_tiles.astype(np.int32)).to(dev),
            items=torch.from_numpy(items.astype(np.int32)).to(dev),
            ntiles=ntiles, nitems=len(items), S=S, upper=upper, mirror=mirror, ldc=ldc,
            est=est, pairs=pairs, host_items=items, algorithm=self.cfg.algorithm,
            nparts=nparts, host_rowids=rowids, host_colids=colids, host_tiles=host_tiles,
            item_tile=item_tile, item_share=share)

    def plan_triangle(self, ids: Optional[Sequence[int]] = None, ldc: Optional[int] = None) -> PairPlan:
        """All pairs i < j among ``ids`` (default: every vector of the arena), and
        every vector with itself."""
        a = self.arena
        ids = np.arange(a.n) if ids is None else np.asarray(ids, np.int64)
        order = np.argsort(-a.nnz[ids], kind="stable")
        perm = ids[order]
        N = len(perm)
        tiles = self._tiles(N, N, True)
        plan = self._finish_plan(perm, perm, tiles, True, True, ldc or a.n, N * (N - 1) // 2)
        plan.diag = True
        return plan

    def plan_rect(self, row_ids: Sequence[int], col_ids: Sequence[int], ldc: int,
                  col_arena: Optional[Arena] = None) -> PairPlan:
        """Every (row, column) pair; out[row_id * ldc + col_id].  Rows are vectors
        of this engine's arena, columns of ``col_arena`` (default: the same)."""
        a = self.arena
        ca = col_arena if col_arena is not None else a
        rows = np.asarray(row_ids, np.int64)
        cols = np.asarray(col_ids, np.int64)
        rows = rows[np.argsort(-a.nnz[rows], kind="stable")]
        cols = cols[np.argsort(-ca.nnz[cols], kind="stable")]
        tiles = self._tiles(len(rows), len(cols), False)
        return self._finish_plan(rows, cols, tiles, False, False, ldc, len(rows) * len(cols),
                                 a.nnz, ca.nnz)

    # -- execution -------------------------------------------------------------
    def _parts(self, plan: PairPlan) -> torch.Tensor:
        if plan.algorithm == "postings":
            need = plan.nparts * self.cfg.block * self.cfg.block * 2  # int64 as int32 pairs
        else:
            need = plan.ntiles * plan.S * self.cfg.tile_rows * self.cfg.tile_cols * 2
        if self.part is None or self.part.numel() < need:
            self.part = torch.empty(max(need, 2), dtype=torch.float32, device=self.device)
        return self.part

    def run(self, plan: PairPlan, out: torch.Tensor, stream=None, item_cycles: torch.Tensor = None,
            diagonal: bool = True, events=None, col_arena: Optional[Arena] = None) -> None:
        """Writes C of every planned pair into ``out`` (float64, row-major, ldc).
        ``events`` = (start, end) CUDA events recorded around the pair kernel."""
        a = self.arena
        if plan.algorithm != self.cfg.algorithm:
            raise ValueError(f"plan made for the {plan.algorithm} kernel, engine runs "
                             f"{self.cfg.algorithm}")
        s_obj = stream if stream is not None else torch.cuda.current_stream(self.device)
        st = int(s_obj.cuda_stream)
        with torch.cuda.stream(s_obj):  # buffers on the stream the kernels use
            part = self._parts(plan)
            self.counter.zero_()
        if events is not None:
            events[0].record(s_obj)
        ca = col_arena if col_arena is not None else a
        if ca is not a and (a.index_on_ranks or ca.index_on_ranks):
            raise ValueError("dense key ranks need rows and columns in the same arena "
                             "(EngineConfig(compress=False) for two arenas)")
        cyc = _p(item_cycles) if item_cycles is not None else 0
        if plan.algorithm == "postings":
            check(self.L.phyloPostingsLaunch(
                st, _p(a.pair_keys()), _p(a.values), _p(a.vec_off), _p(a.roff),
                _p(ca.pair_keys()), _p(ca.values), _p(ca.vec_off), _p(ca.roff), a.R,
                self.cfg.wshift, _p(plan.rowids), _p(plan.colids), _p(plan.items), plan.nitems,
                _p(self.counter), _p(part), _p(self.status), cyc, self.cfg.block, self.grid))
            if events is not None:
                events[1].record(s_obj)
            check(self.L.phyloPostingsReduce(
                st, _p(part), _p(plan.tiles), plan.ntiles, self.cfg.block, _p(plan.rowids),
                _p(plan.colids), _p(out), plan.ldc, int(plan.diag and diagonal),
                int(plan.mirror)))
        else:
            check(self.L.phyloPairsLaunch(
                st, _p(a.pair_keys()), _p(a.values), _p(a.vec_off), _p(a.roff),
                _p(ca.pair_keys()), _p(ca.values), _p(ca.vec_off), _p(ca.roff), a.R,
                self.cfg.wshift, _p(plan.rowids), _p(plan.colids), _p(plan.items), plan.nitems,
                _p(self.counter), _p(part), self.cfg.fold, cyc, self.cfg.tile_rows,
                self.cfg.tile_cols, self.grid))
            if events is not None:
                events[1].record(s_obj)
            check(self.L.phyloPairsReduce(
                st, _p(part), _p(plan.tiles), plan.ntiles, plan.S, self.cfg.tile_rows,
                self.cfg.tile_cols, _p(plan.rowids), _p(plan.colids), _p(out), plan.ldc,
                (2 if plan.diag and diagonal else 1) if plan.upper else 0, int(plan.mirror)))
        self.launches += 3  # counter fill, pair kernel, reduction
        if diagonal and plan.upper and not plan.diag:
            maxlen = int(np.max(np.diff(a.off[:a.n + 1]))) if a.n else 1
            nb = int(self.L.phyloSelfDotPartBytes(a.n, maxlen))
            if self.self_part is None or self.self_part.numel() < nb:
                with torch.cuda.stream(s_obj):
                    self.self_part = torch.empty(max(nb, 8), dtype=torch.uint8,
                                                 device=self.device)
            check(self.L.phyloSelfDot(st, _p(a.values), _p(a.vec_off), a.n, maxlen,
                                      _p(self.self_part), _p(out), plan.ldc))
            self.launches += 2
        self._fix_nonfinite(plan, out, s_obj, col_arena, diag=diagonal and plan.diag)

    def device_status(self) -> int:
        """DeviceError bits the postings kernel recorded (synchronises); 0 = none."""
        return int(self.status.item())

    def _fix_nonfinite(self, plan: PairPlan, out: torch.Tensor, stream,
                       col_arena: Optional[Arena] = None, diag: bool = False) -> None:
        """Vectors whose values are NaN/inf: recompute their pairs with the
        merge-path kernel, which only multiplies values of shared keys (as the
        reference does)."""
        ra = self.arena
        ca = col_arena if col_arena is not None else ra
        bad_r = ~np.isfinite(ra.norms[:ra.n])
        bad_c = ~np.isfinite(ca.norms[:ca.n])
        if not bad_r.any() and not bad_c.any():
            return
        rows, cols = plan.host_rowids, plan.host_colids
        pa, pb = [], []
        for t in plan.host_tiles:
            r0, nr, c0, nc = (int(x) for x in t[:4])
            I, J = np.meshgrid(np.arange(r0, r0 + nr), np.arange(c0, c0 + nc), indexing="ij")
            I, J = I.ravel(), J.ravel()
            if plan.upper:  # positions: pairs i < j, and i == j when the plan holds the diagonal
                keep = (I < J) | (diag & (I == J))
                I, J = I[keep], J[keep]
            r, c = rows[I], cols[J]
            sel = bad_r[r] | bad_c[c]
            pa.append(r[sel])
            pb.append(c[sel])
        pa = np.concatenate(pa) if pa else np.zeros(0, np.int64)
        pb = np.concatenate(pb) if pb else np.zeros(0, np.int64)
        if len(pa) == 0:
            return
        vals = self.compare_pairs_merge(pa, pb, col_arena=col_arena, stream=stream)
        flat = out.view(-1)
        with torch.cuda.stream(stream):
            idx = torch.from_numpy(pa * plan.ldc + pb).to(self.device)
            flat.index_copy_(0, idx, vals)
            if plan.mirror:
                flat.index_copy_(0, torch.from_numpy(pb * plan.ldc + pa).to(self.device), vals)

    # -- merge-path algorithm over explicit pairs -------------------------------
    def _nnz_dev(self, arena: Arena) -> torch.Tensor:
        """The arena's entry counts on the device, copied on every call (a few KB):
        an arena object is reset and rebuilt in place (a serving slot's query
        arena), so neither its identity nor its size says its counts are unchanged.
        Allocated and copied on the current stream, which the caller's kernels use
        (from pageable memory: staged before the call returns, like the pair lists)."""
        return torch.from_numpy(arena.nnz[:arena.n].astype(np.int32)).to(self.device,
                                                                          non_blocking=True)

    def compare_pairs_merge(self, pa, pb, col_arena: Optional[Arena] = None, stream=None,
                            out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """C of pairs (pa[p] in this arena, pb[p] in col_arena) with the
        multi-pair merge-path kernels; returns a float64 device tensor."""
        a = self.arena
        ca = col_arena if col_arena is not None else a
        pa = np.asarray(pa, np.int64)
        pb = np.asarray(pb, np.int64)
        P = len(pa)
        if out is None:
            out = torch.empty(P, dtype=torch.float64, device=self.device)
        if P == 0:
            return out
        te = int(self.L.phyloCompareTileElements())
        tiles = int(np.sum((a.nnz[pa] + ca.nnz[pb] + te - 1) // te))
        nbytes = int(self.L.phyloComparePairsManyScratch(P, tiles))
        if getattr(self, "_many_scratch", None) is None or self._many_scratch.numel() < nbytes:
            self._many_scratch = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        s_obj = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(s_obj):
            dpa = torch.from_numpy(pa.astype(np.int32)).to(self.device, non_blocking=True)
            dpb = torch.from_numpy(pb.astype(np.int32)).to(self.device, non_blocking=True)
            na = self._nnz_dev(a)
            nb = na if ca is a else self._nnz_dev(ca)
        check(self.L.phyloComparePairsMany(
            int(s_obj.cuda_stream), _p(self._many_scratch), self._many_scratch.numel(),
            _p(a.keys), _p(a.values), _p(a.vec_off), _p(na),
            _p(ca.keys), _p(ca.values), _p(ca.vec_off), _p(nb),
            _p(dpa), _p(dpb), P, tiles, _p(out)))
        self.launches += 7
        return out


    # -- CUDA graph of the pair phase -----------------------------------------
    def capture(self, plan: PairPlan, out: torch.Tensor, diagonal: bool = True,
                col_arena: Optional[Arena] = None) -> torch.cuda.CUDAGraph:
        """Captures counter reset, pair kernel, reduction (and self products)
        for this plan into a CUDA graph; replay() reruns them with one launch.
        The arena and plan buffers must stay alive and unchanged in shape."""
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        # warm run outside the capture: sizes scratch buffers, sets attributes
        self.run(plan, out, stream=s, diagonal=diagonal, col_arena=col_arena)
        s.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.run(plan, out, stream=s, diagonal=diagonal, col_arena=col_arena)
        torch.cuda.current_stream(self.device).wait_stream(s)
        return g


# ------------------------------------------------------------------------------
# autotuner
# ------------------------------------------------------------------------------

def _tune_cache_path() -> str:
    import os
    return os.environ.get("ROCKET_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "rocket_gb300",
                                       "tune.json"))


def tune_key(arena: Arena, n_rows: int, n_cols: int) -> str:
    nnz = arena.nnz[:arena.n]
    bucket = int(np.round(np.log2(max(float(nnz.mean()), 1.0)) * 2))
    return f"{arena.alphabet}-k{arena.k}-r{int(np.log2(max(n_rows, 1)))}-c{int(np.log2(max(n_cols, 1)))}-n{bucket}"


TUNE_SPACE = [
    dict(algorithm="postings", block=128, wshift=9, items_per_cta=4),
    dict(algorithm="postings", block=128, wshift=9, items_per_cta=8),
    dict(algorithm="postings", block=128, wshift=8, items_per_cta=4),
    dict(algorithm="postings", block=128, wshift=10, items_per_cta=4),
    dict(algorithm="postings", block=64, wshift=9, items_per_cta=4),
    dict(algorithm="postings", block=64, wshift=10, items_per_cta=4),
    dict(algorithm="window", wshift=11, tile_rows=16, tile_cols=256, fold=28, items_per_cta=16),
    dict(algorithm="window", wshift=11, tile_rows=16, tile_cols=128, fold=28, items_per_cta=16),
    dict(algorithm="window", wshift=10, tile_rows=16, tile_cols=64, fold=28, items_per_cta=4),
    dict(algorithm="window", wshift=10, tile_rows=32, tile_cols=64, fold=28, items_per_cta=4),
]


def autotune(arena: Arena, ids=None, space=None, repeats: int = 2, use_cache: bool = True,
             include_merge: bool = True, verbose: bool = False, prune: float = 0.0) -> dict:
    """Times the pair kernels under each configuration of ``space`` (postings and
    window kernels, and optionally the merge-path kernel) on the all-pair plan of
    ``ids`` and returns the fastest, caching it per (alphabet, K, size class) in a
    JSON file (the role of phylogenetics/tune.py:25-84 and the tuning entry point
    native.cu:782-838, over this library's own tunables).  ``prune`` > 0: a
    candidate whose first (warm) run is slower than prune x the best time so far is
    recorded with that time and not repeated."""
    import json
    import os
    import time
    space = space or TUNE_SPACE
    n = arena.n if ids is None else len(ids)
    key = tune_key(arena, n, n)
    path = _tune_cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            return cache[key]
    results = []
    out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device=arena.keys.device)
    for cfg in space:
        eng = PairEngine(arena, EngineConfig(**cfg))
        saved = arena.index_state()
        eng.ensure_index()
        plan = eng.plan_triangle(ids)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        eng.run(plan, out, diagonal=False)
        e1.record()
        torch.cuda.synchronize()
        first = e0.elapsed_time(e1)
        so_far = min([r["ms"] for r in results], default=float("inf"))
        best = float("inf")
        if prune > 0 and first > prune * so_far:
            best, repeats_here = first, 0
        else:
            repeats_here = repeats
        for _ in range(repeats_here):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            eng.run(plan, out, diagonal=False)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        results.append(dict(cfg, ms=best))
        arena.restore_index(saved)
        if verbose:
            print(results[-1], flush=True)
    if include_merge:
        eng = PairEngine(arena)
        idx = np.arange(arena.n) if ids is None else np.asarray(ids)
        iu = np.triu_indices(len(idx), 1)
        pa, pb = idx[iu[0]], idx[iu[1]]
        eng.compare_pairs_merge(pa, pb)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(repeats):
            t0 = time.perf_counter()
            eng.compare_pairs_merge(pa, pb)
            torch.cuda.synchronize()
            best = min(best, 1000 * (time.perf_counter() - t0))
        results.append(dict(algorithm="merge", ms=best))
        if verbose:
            print(results[-1], flush=True)
    winner = min(results, key=lambda r: r["ms"])
    entry = dict(winner, candidates=results)
    if use_cache:
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            cache[key] = entry
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return entry


def distances(c: torch.Tensor) -> torch.Tensor:
    """D = (1 - C) / 2."""
    return (1.0 - c) * 0.5
