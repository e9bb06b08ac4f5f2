"""Benchmark: pairwise composition-vector distances per second on GB300.

One step = the whole hot path over one batch: build the composition vectors of
every proteome (K-mer counting, Markov alpha, normalisation) from the residue
bytes, index them, and compute C (hence D = (1 - C) / 2) for every pair.

  value   device-resident: the residue bytes are in HBM when a step starts;
          CUDA events on the launching stream around each step; L2 flushed
          (512 MB write) between steps, outside the timed events.
  e2e     through the public batched API with host buffers: pinned host bytes
          -> H2D -> build -> pairs -> D2H of the C matrix, wall clock per step.
  roofline  the pair kernel (k_allpairs): algorithmic bytes 8 * (nnz_i + nnz_j)
          per pair over its event-timed duration, against the measured HBM copy
          bandwidth; values above 1 come from reuse of resident vectors (shared
          memory tiles and L2), not from DRAM traffic.
  cpu_baseline  the reference's CPU path (CompositionVectorKernels.buildCPU /
          compareCPU, restated in C under oracle/) on a bounded sample,
          OpenMP over proteomes and over pairs, extrapolated to the workload.

``--impl reference`` prints the reference arm: that CPU path, timed the same
way, as the line's value.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "uniform256"
WORKLOAD_TEXTS = {
    "cpu16": ("cpu16: 16 synthetic proteomes x 1,500 proteins (lognormal lengths, median "
              "300 aa), seed 0, branch substitution rate 0.05, K={k} protein, all {pairs:,} "
              "pairs i<j (+ the {n} self products)"),
    "uniform256": ("uniform256: 256 synthetic proteomes x 1,500 proteins (lognormal lengths, "
                   "median 300 aa), seed 1, branch substitution rate U(0.01, 0.2), K={k} "
                   "protein, all {pairs:,} pairs i<j (+ the {n} self products)"),
    "uneven1024": ("uneven1024: 1,024 synthetic proteomes, seed 2, protein counts lognormal "
                   "(median 1,900, sigma 0.9) clipped to [300, 12,000], lengths lognormal "
                   "(median 300 aa), branch substitution rate U(0.01, 0.2), K={k} protein, all "
                   "{pairs:,} pairs i<j (+ the {n} self products)"),
    "sweep512": ("sweep512: 512 synthetic proteomes, seed 3, protein counts lognormal (median "
                 "1,900, sigma 0.9) clipped to [300, 12,000], K={k} protein, all {pairs:,} pairs "
                 "i<j (+ the {n} self products)"),
}


def workload_text(name, k, n):
    return WORKLOAD_TEXTS[name].format(k=k, pairs=n * (n - 1) // 2, n=n)


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_per_launch(kernel: str, workload: str, wshift: int):
    """DRAM bytes (read + write) of one pair-kernel launch, from the committed
    ncu summary of the same kernel, workload and window width (a line
    `dram_bytes_per_launch = N` in profiles/dram_<kernel>_<workload>_w<shift>.md)."""
    path = os.path.join(ROOT, "profiles", f"dram_{kernel}_{workload}_w{wshift}.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.strip().startswith("dram_bytes_per_launch"):
                return float(line.split("=")[1].strip().replace(",", ""))
    return None


class ClockSampler:
    """nvidia-smi samples during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _barrier_max(value: float, world: int) -> float:
    """Maximum of `value` over the ranks (the slowest replica sets the time)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------
# CPU baseline (the reference's CPU path, restated in C under oracle/)
# ----------------------------------------------------------------------------

def cpu_baseline(wl, n_pairs_total, n_build_total, seconds=15.0, threads=0, seed=0, k=6):
    from oracle import oracle as O
    O.lib()
    threads = threads or O.max_threads()
    rng = np.random.default_rng(seed)
    nb = min(len(wl), max(threads, 4))
    ids = rng.choice(len(wl), nb, replace=False)
    t0 = time.perf_counter()
    vecs = O.java_build_many([wl.get(int(i)) for i in ids], k, threads=threads)
    t_build = time.perf_counter() - t0
    build_rate = nb / t_build                                      # proteomes / s
    pairs = [(a, b) for a in range(nb) for b in range(a + 1, nb)]
    budget = max(1.0, seconds - t_build)
    done, t_cmp = 0, 0.0
    while t_cmp < budget and done < 100000:
        chunk = pairs * max(1, (4 * threads) // max(len(pairs), 1))
        t0 = time.perf_counter()
        O.java_compare_pairs(vecs, chunk, threads=threads)
        t_cmp += time.perf_counter() - t0
        done += len(chunk)
    pair_rate = done / t_cmp                                        # pairs / s
    total = n_build_total / build_rate + n_pairs_total / pair_rate
    return {
        "value": n_pairs_total / total, "unit": "pairs/s", "cores": threads, "kind": "port",
        "sample": (f"buildCPU of {nb} proteomes ({t_build:.1f} s) + compareCPU of {done} pairs "
                   f"({t_cmp:.1f} s), OpenMP {threads} threads; extrapolated to "
                   f"{n_build_total} builds + {n_pairs_total} pairs"),
        "build_per_s": build_rate, "pairs_per_s_compare_only": pair_rate,
    }


def plain_path(arena, wl, seq, dev, n_pairs, n_build, peak, sample_pairs=400, sample_builds=16,
               seed=7, k=6):
    """The drop-in path as the reference drives it: one synchronous
    buildCompositionVector per proteome and one synchronous
    compareCompositionVectors per pair (CompositionVectorKernels.java:91-135),
    timed on a sample and extrapolated.  Also the merge-path kernel alone:
    asynchronous back-to-back pairs (random pairs, so the two vectors are not
    L2-resident), algorithmic bytes 8*(nl+nr) per pair over the event time."""
    import torch
    from rocket_gb300 import _native
    from rocket_gb300.kernels import CompositionVectorKernels
    L = _native.load()
    rng = np.random.default_rng(seed)
    maxn = int(arena.nnz.max())
    ker = CompositionVectorKernels("protein", k, maxn + 1024, int(wl.lengths().max()), device=dev)
    st = ker.stream
    keys = torch.empty(maxn + 1024, dtype=torch.int32, device=dev)
    vals = torch.empty(maxn + 1024, dtype=torch.float32, device=dev)
    ids = rng.choice(len(wl), min(sample_builds, len(wl)), replace=False)
    for i in ids[:2]:  # warm-up
        ker.build_vector_gpu(seq[int(wl.offsets[i]):int(wl.offsets[i + 1])], keys, vals)
    t0 = time.perf_counter()
    for i in ids:
        ker.build_vector_gpu(seq[int(wl.offsets[i]):int(wl.offsets[i + 1])], keys, vals)
    t_build = (time.perf_counter() - t0) / len(ids)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    pi = rng.integers(0, arena.n, size=sample_pairs)
    pj = (pi + 1 + rng.integers(0, arena.n - 1, size=sample_pairs)) % arena.n

    def vec(v):
        o, m = int(arena.off[v]), int(arena.nnz[v])
        return arena.keys[o:o + m], arena.values[o:o + m], m

    for a, b in zip(pi[:4], pj[:4]):  # warm-up
        ka, va, na = vec(a)
        kb, vb, nb = vec(b)
        ker.compare_vectors_gpu(ka, va, na, kb, vb, nb, out)
    t0 = time.perf_counter()
    for a, b in zip(pi, pj):
        ka, va, na = vec(a)
        kb, vb, nb = vec(b)
        ker.compare_vectors_gpu(ka, va, na, kb, vb, nb, out)
    t_pair = (time.perf_counter() - t0) / sample_pairs
    # merge-path kernels alone: all sampled pairs in one multi-pair launch
    from rocket_gb300.engine import PairEngine
    eng = PairEngine(arena)
    nbytes = int(8 * (arena.nnz[pi].sum() + arena.nnz[pj].sum()))
    eng.compare_pairs_merge(pi, pj)  # warm-up (scratch, attributes)
    torch.cuda.synchronize()
    ms = []
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        eng.compare_pairs_merge(pi, pj)
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    k_s = min(ms) / 1000.0
    gbs = nbytes / k_s / 1e9
    total = n_build * t_build + n_pairs * t_pair
    return {
        "value": n_pairs / total, "unit": "pairs/s",
        "sample": (f"{len(ids)} synchronous buildCompositionVector calls ({1000 * t_build:.2f} ms "
                   f"each) + {sample_pairs} synchronous compareCompositionVectors calls "
                   f"({1000 * t_pair:.3f} ms each), extrapolated to {n_build} builds + "
                   f"{n_pairs} pairs"),
        "merge_kernel": {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "pairs_per_s": sample_pairs / k_s,
                         "note": f"phyloComparePairsMany over {sample_pairs} random pairs in one "
                                 "launch sequence (tile count, scan, partition, intersect, reduce); "
                                 "algorithmic bytes 8*(nl+nr) per pair; best of 3"},
    }


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return 0
    from rocket_gb300 import synth
    wl = synth.workload(args.workload, n=args.proteomes)
    n = len(wl)
    n_pairs = n * (n - 1) // 2
    vals = []
    base = None
    for s in range(args.warmup + args.steps):
        r = cpu_baseline(wl, n_pairs, n, seconds=args.ref_seconds, seed=s, k=args.k)
        if s >= args.warmup:
            vals.append(r["value"])
            base = r
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": "pairwise CV distances/s", "value": value,
        "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * n_pairs / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 (java float path)", "data": "synthetic",
        "config": {"workload": workload_text(args.workload, args.k, n)},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": base["cores"],
                         "kind": base["kind"], "sample": base["sample"]},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------

def run_ours(args):
    import torch
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    from rocket_gb300 import synth
    from rocket_gb300.engine import BatchBuilder, EngineConfig, PairEngine, auto_tile_cols

    wl = synth.workload(args.workload, n=args.proteomes)
    N = len(wl)
    n_pairs = N * (N - 1) // 2
    if args.tile_cols == 0:
        args.tile_cols = 64 if args.tile_rows == 32 else auto_tile_cols(N)
    stream = torch.cuda.current_stream(dev)
    pinned = torch.from_numpy(wl.data).pin_memory()
    seq = torch.empty(pinned.numel(), dtype=torch.uint8, device=dev)
    seq.copy_(pinned)
    builder = BatchBuilder("protein", args.k, device=dev, max_batch=args.max_batch,
                           overlap=not args.no_overlap)
    cfg = EngineConfig(wshift=args.wshift, fold=args.fold, items_per_cta=args.items_per_cta,
                       tile_rows=args.tile_rows, tile_cols=args.tile_cols,
                       compress=not args.no_compress)
    out = torch.zeros((N, N), dtype=torch.float64, device=dev)
    out_host = torch.zeros((N, N), dtype=torch.float64).pin_memory()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    arena = None
    engine = None
    kernel_ms = []
    state = {}

    def step(record_kernel=False, host=None):
        nonlocal arena, engine
        ev = None
        if record_kernel:
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
            ev[2].record(stream)
        arena = builder.build(seq, wl.offsets, arena=arena.reset() if arena is not None else None,
                              stream=stream, host=host)
        if engine is None:
            engine = PairEngine(arena, cfg)
        engine.arena = arena
        if record_kernel:
            ev[3].record(stream)
        engine.ensure_index(stream)
        if record_kernel:
            ev[4].record(stream)
        plan = engine.plan_triangle()
        engine.run(plan, out, stream=stream, events=ev)
        state["plan"] = plan
        return ev

    # warm-up
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    nnz = arena.nnz.copy()
    plan = state["plan"]
    alg_bytes = 0
    rows = plan.rowids.cpu().numpy()
    # algorithmic bytes of one pair launch: sum over pairs i<j of 8 (nnz_i + nnz_j)
    alg_bytes = int(8 * (N - 1) * nnz.sum())

    # timed device-resident steps
    launches0 = builder.launches + engine.launches
    step_ms = []
    phase_ms = []
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index or 0) as clocks:
        for s in range(args.steps):
            flush.fill_(s & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ev = step(record_kernel=True)
            e1.record(stream)
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            kernel_ms.append(ev[0].elapsed_time(ev[1]))
            phase_ms.append((ev[2].elapsed_time(ev[3]), ev[3].elapsed_time(ev[4]),
                             ev[4].elapsed_time(ev[0]), ev[1].elapsed_time(e1)))
    launches = (builder.launches + engine.launches - launches0) // args.steps
    total_s = sum(step_ms) / 1000.0
    total_s = _barrier_max(total_s, world)
    value = world * args.steps * n_pairs / total_s

    # end to end through the public API with host buffers
    e2e_ms = []
    h2d = int(wl.data.nbytes + wl.offsets.nbytes)
    d2h = int(N * N * 8)
    for s in range(max(1, args.steps)):
        flush.fill_(s & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step(host=pinned)  # each batch's residues copied from pinned memory ahead of it
        out_host.copy_(out, non_blocking=True)
        stream.synchronize()
        e2e_ms.append(1000.0 * (time.perf_counter() - t0))
    e2e_s = _barrier_max(sum(e2e_ms) / 1000.0, world)
    e2e_value = world * len(e2e_ms) * n_pairs / e2e_s

    if rank != 0:
        return 0
    peak, peak_kind = _peaks()
    k_ms = float(np.mean(kernel_ms))
    achieved = alg_bytes / (k_ms / 1000.0) / 1e9
    kernel_name = ("k_allpairs32" if args.tile_rows == 32 else "k_allpairs") + \
        f"_{args.tile_rows}x{args.tile_cols}"
    traffic = _traffic_per_launch(kernel_name, args.workload, args.wshift)
    line = {
        "metric": "pairwise CV distances/s", "value": value, "unit": "pairs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(step_ms)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {
            "workload": workload_text(args.workload, args.k, N),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "flushed between steps (512 MB write, outside the timed events)",
            "nnz_mean": float(nnz.mean()), "nnz_total": int(nnz.sum()),
            "window_shift": args.wshift, "tile_rows": args.tile_rows,
            "tile_cols": args.tile_cols, "fold": args.fold,
            "key_ranks": not args.no_compress, "windows": int(engine.arena.R),
            "items": plan.nitems,
            "segments": plan.S,
        },
        "breakdown_ms": {"build": float(np.mean([p[0] for p in phase_ms])),
                         "key_ranks_and_window_index": float(np.mean([p[1] for p in phase_ms])),
                         "plan_and_launch_gap": float(np.mean([p[2] for p in phase_ms])),
                         "pair_kernel": k_ms,
                         "reduce_and_self": float(np.mean([p[3] for p in phase_ms])),
                         "step": float(np.mean(step_ms))},
        "roofline": {
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic,
            "kernel": kernel_name,
            "note": (f"{peak_kind} peak; algorithmic bytes 8*(nnz_i+nnz_j) per pair = "
                     f"{alg_bytes / 1e9:.1f} GB per launch; frac > 1 = reuse of resident "
                     "vectors in shared memory and L2, not DRAM bandwidth"),
        },
        "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": float(np.mean(e2e_ms))},
        "clocks": clocks.summary(),
        "gpu_launches": int(launches),
    }
    if not args.no_plain:
        line["plain"] = plain_path(arena, wl, seq, dev, n_pairs, N, peak, k=args.k)
    if not args.no_cpu_baseline:
        cb = cpu_baseline(wl, n_pairs, N, seconds=args.ref_seconds, k=args.k)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


# ----------------------------------------------------------------------------
# serving
# ----------------------------------------------------------------------------

SERVE_TEXT = ("serve2048: device-resident database of 2,048 synthetic proteomes (seed 4, protein "
              "counts lognormal median 1,900 sigma 0.9 clipped to [300, 12,000]), K=6; query "
              "batches of U(1..64) proteomes of the same distribution arriving as a Poisson "
              "process; each query built, compared with the whole database, then appended; "
              "HBM budget 120 GB")


def run_serve(args):
    import torch
    from rocket_gb300 import synth
    from rocket_gb300.engine import EngineConfig
    from rocket_gb300.serve import Request, ServingEngine, percentile

    rng = np.random.default_rng(4)
    sizes = rng.integers(1, 65, size=args.query_batches)
    n_db = args.db
    if args.tile_cols == 0:  # a query batch has few row tiles: 128-column items keep the SMs busy
        args.tile_cols = 64 if args.tile_rows == 32 else 128
    total_q = int(sizes.sum())
    t0 = time.perf_counter()
    wl = synth.workload("serve2048", n=n_db, extra=total_q + args.warmup)
    t_gen = time.perf_counter() - t0
    db = wl.subset(range(n_db))
    srv = ServingEngine("protein", 6, budget_bytes=args.budget_gb * 1e9, slots=args.slots,
                        max_batch=64, cfg=EngineConfig(wshift=args.wshift, fold=args.fold,
                                                       tile_rows=args.tile_rows,
                                                       tile_cols=args.tile_cols,
                                                       segments=args.segments))
    lens = db.lengths()
    capacity_entries = int(min(np.sum(8 * wl.lengths() + 64),
                               (args.budget_gb * 1e9 - 20e9) / 8.0))
    t0 = time.perf_counter()
    srv.load(db, capacity_vectors=len(wl), capacity_entries=capacity_entries)
    torch.cuda.synchronize()
    t_load = time.perf_counter() - t0
    srv.start()
    nxt = n_db
    # warm-up requests (one proteome each), not measured
    for w in range(args.warmup):
        r = srv.submit(Request(-1 - w, wl.subset([nxt]), append=False))
        nxt += 1
        r.done.wait(600)
    batches = []
    for b in range(args.query_batches):
        batches.append(wl.subset(range(nxt, nxt + int(sizes[b]))))
        nxt += int(sizes[b])
    gaps = rng.exponential(1.0 / args.rate, size=args.query_batches)
    reqs = []
    t_start = time.perf_counter()
    t_next = t_start
    with ClockSampler(0) as clocks:
        for b, q in enumerate(batches):
            t_next += gaps[b]
            delay = t_next - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            reqs.append(srv.submit(Request(b, q, append=True, t_arrival=time.perf_counter())))
        for r in reqs:
            r.done.wait(3600)
        srv.stop()
    errors = [r.error for r in reqs if r.error]
    lat = [1000.0 * r.latency for r in reqs if not r.error]
    t_end = max(r.t_done for r in reqs)
    pairs = sum(len(r.proteomes) * r.db_n for r in reqs if not r.error)
    line = {
        "metric": "serve latency per query batch", "p50_ms": percentile(lat, 50),
        "p99_ms": percentile(lat, 99), "max_ms": max(lat) if lat else None,
        "value": pairs / (t_end - t_start), "unit": "pairs/s (sustained)",
        "requests": len(reqs), "query_proteomes": total_q, "errors": len(errors),
        "arrival_rate_per_s": args.rate, "slots": args.slots, "batches_run": srv.batches,
        "db_start": n_db, "db_end": srv.db.arena.n, "db_appends_refused": srv.db.refused,
        "hbm_budget_gb": args.budget_gb, "hbm_reserved_peak_gb": srv.budget.peak / 1e9,
        "db_load_s": t_load, "generate_s": t_gen, "data": "synthetic",
        "config": {"workload": SERVE_TEXT, "segments": args.segments, "window_shift": args.wshift},
        "clocks": clocks.summary(),
    }
    if errors:
        line["first_error"] = errors[0]
    print(json.dumps(line), flush=True)
    return 0 if not errors else 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--wshift", type=int, default=11)
    ap.add_argument("--no-overlap", action="store_true",
                    help="build one batch at a time instead of two in flight")
    ap.add_argument("--no-compress", action="store_true",
                    help="pair kernel on raw keys instead of dense key ranks")
    ap.add_argument("--tile-rows", type=int, default=16, choices=[16, 32],
                    help="row vectors per pair-kernel work item (selects the kernel)")
    ap.add_argument("--tile-cols", type=int, default=0, choices=[0, 32, 64, 128, 256],
                    help="column vectors per pair-kernel work item (0: 256 for all-pair "
                         "triangles over 384 or more proteomes, else 128)")
    ap.add_argument("--fold", type=int, default=28,
                    help="products per FP32 accumulator between compensated folds (multiple of 4)")
    ap.add_argument("--items-per-cta", type=int, default=8)
    ap.add_argument("--max-batch", type=int, default=24)
    ap.add_argument("--ref-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the per-pair ABI measurement")
    ap.add_argument("--proteomes", type=int, default=None,
                    help="use only the first N proteomes (small profiling cases)")
    ap.add_argument("--mode", default="allpairs", choices=["allpairs", "serve"])
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOAD_TEXTS))
    ap.add_argument("--k", type=int, default=6, help="K-mer length (protein)")
    ap.add_argument("--db", type=int, default=2048, help="serve: database proteomes")
    ap.add_argument("--query-batches", type=int, default=24, help="serve: arriving query batches")
    ap.add_argument("--rate", type=float, default=8.0, help="serve: query batches per second")
    ap.add_argument("--slots", type=int, default=2, help="serve: concurrent batches")
    ap.add_argument("--segments", type=int, default=16, help="serve: key segments per tile")
    ap.add_argument("--budget-gb", type=float, default=120.0, help="serve: HBM budget")
    args = ap.parse_args()
    if args.mode == "serve":
        return run_serve(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
