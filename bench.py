"""Benchmark: pairwise composition-vector distances per second on GB300.

One step = the whole hot path over one batch: build the composition vectors of
every proteome (K-mer counting, Markov alpha, normalisation) from the residue
bytes, index them (dense key ranks, window index), and compute C (hence
D = (1 - C) / 2) for every pair and every vector with itself.

Default workload: uneven1024, 1,024 proteomes of very uneven sizes, all 523,776
pairs (the batched configuration the metric is quoted on).

  value    device-resident: the residue bytes are in HBM when a step starts;
           CUDA events on the launching stream around each step; L2 flushed
           (512 MB write) between steps, outside the timed events.  The pair
           phase is the autotuned engine configuration (chosen during warm-up)
           replayed as one CUDA graph (counter reset, pair kernel, reduction).
  e2e      through the public batched API with host buffers: pinned host bytes
           -> H2D (per build batch, overlapped) -> build -> index -> pairs -> D2H
           of the N x N matrix, wall clock per step.
  roofline the pair kernel: DRAM bytes per launch (from an ncu capture of the
           same kernel, table below) over the event-timed pair phase, against
           the measured HBM copy bandwidth; beside it the kernel's actual bound
           (shared-memory wavefronts) and the algorithmic-bytes figure of one
           read of both vectors per pair, labelled as reuse.
  cpu_baseline  the reference's CPU path (CompositionVectorKernels.buildCPU /
           compareCPU, restated in C under oracle/) on a bounded sample, OpenMP
           over proteomes and over pairs, extrapolated to the workload (flagged).
  plain    the drop-in ABI driven as the reference's plug-in drives it (one
           synchronous build per proteome, one synchronous compare per pair),
           sampled and extrapolated (flagged); plus the multi-pair merge kernel.
  serve    a short serving run: database of 2,048 proteomes, Poisson arrivals of
           query batches at a rate the server sustains; p50/p99 latency.

``--impl reference`` prints the reference arm: the reference's CPU path, timed
the same way, as the line's value; ms_per_step is the wall time a step took.
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

WORKLOAD = "uneven1024"
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

# DRAM bytes (read + write) and shared-memory wavefronts of one pair-kernel launch,
# from ncu captures of the same kernel instantiation on the same workload
# (profiles/ncu_pair_kernel_counters_fullsize.md gives the commands and figures).  Keyed by
# (kernel, workload, K, window shift); a launch of anything else reports null.
PAIR_KERNEL_COUNTERS = {
    ("k_allpairs<512,1,2>", "uneven1024", 6, 11): {"dram_bytes": 826_724_824_832,
                                                   "smem_wavefronts": 132_650_445_958},
    ("k_allpairs<512,1,2>", "uniform256", 6, 11): {"dram_bytes": 39_084_610_560,
                                                   "smem_wavefronts": 7_810_281_080},
    ("k_allpairs<512,1,2>", "sweep512", 7, 11): {"dram_bytes": 63_618_668_800,
                                                 "smem_wavefronts": 19_710_517_806},
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

def cpu_baseline(wl, n_pairs_total, n_build_total, seconds=15.0, threads=0, seed=0, k=6,
                 n_sample=0):
    """Times buildCPU on a seeded sample of proteomes (n_sample, default one per
    thread and at least 4) and compareCPU on pairs of them for about `seconds`, and
    extrapolates to the whole workload."""
    from oracle import oracle as O
    O.lib()
    threads = threads or O.max_threads()
    rng = np.random.default_rng(seed)
    nb = min(len(wl), n_sample or max(threads, 4))
    ids = rng.choice(len(wl), nb, replace=False)
    t_start = time.perf_counter()
    t0 = time.perf_counter()
    vecs = O.java_build_many([wl.get(int(i)) for i in ids], k, threads=threads)
    t_build = time.perf_counter() - t0
    build_rate = nb / t_build                                      # proteomes / s
    # (one sampled proteome: its vector against itself)
    pairs = [(a, b) for a in range(nb) for b in range(a + 1, nb)] or [(0, 0)]
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
        "extrapolated": {"sampled_builds": int(nb), "sampled_pairs": int(done),
                         "builds": int(n_build_total), "pairs": int(n_pairs_total)},
        "build_per_s": build_rate, "pairs_per_s_compare_only": pair_rate,
        "wall_s": time.perf_counter() - t_start,
    }


def plain_path(arena, wl, seq, dev, n_pairs, n_build, peak, sample_pairs=400, sample_builds=16,
               seed=7, k=6):
    """The drop-in path as the reference drives it: one synchronous
    buildCompositionVector per proteome and one synchronous
    compareCompositionVectors per pair (CompositionVectorKernels.java:45-89),
    timed on a sample and extrapolated.  Also one compareCompositionVectors call
    alone (the synchronous ABI latency) and the multi-pair merge kernel:
    random pairs back to back in one launch sequence (the two vectors are not
    L2-resident), algorithmic bytes 8*(nl+nr) per pair over the event time."""
    import ctypes
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
    # one synchronous ABI call on two vectors of the median size, C-level loop
    med = np.argsort(arena.nnz)[len(arena.nnz) // 2: len(arena.nnz) // 2 + 2]
    (ka, va, na), (kb, vb, nb) = vec(int(med[0])), vec(int(med[1]))
    scr = ker.scratch
    handle = ker.stream_handle
    torch.cuda.synchronize()
    for _ in range(20):
        L.compareCompositionVectors(handle, scr.data_ptr(), scr.numel(), ka.data_ptr(),
                                    va.data_ptr(), na, kb.data_ptr(), vb.data_ptr(), nb,
                                    out.data_ptr())
    reps = 200
    t0 = time.perf_counter()
    for _ in range(reps):
        rc = L.compareCompositionVectors(handle, scr.data_ptr(), scr.numel(), ka.data_ptr(),
                                         va.data_ptr(), na, kb.data_ptr(), vb.data_ptr(), nb,
                                         out.data_ptr())
    t_call = (time.perf_counter() - t0) / reps
    _native.check(rc)
    # merge-path kernels alone: all sampled pairs in one multi-pair launch
    from rocket_gb300.engine import EngineConfig, PairEngine
    eng = PairEngine(arena, EngineConfig(algorithm="window"))
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
                   f"({1000 * t_pair:.3f} ms each, Python plug-in path), extrapolated to "
                   f"{n_build} builds + {n_pairs} pairs"),
        "extrapolated": {"sampled_builds": int(len(ids)), "sampled_pairs": int(sample_pairs),
                         "builds": int(n_build), "pairs": int(n_pairs)},
        "sync_compare_call_ms": 1000.0 * t_call,
        "sync_compare_call_entries": int(na + nb),
        "merge_kernel": {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "pairs_per_s": sample_pairs / k_s,
                         "note": f"phyloComparePairsMany over {sample_pairs} random pairs in one "
                                 "launch sequence (tile count, scan, intersect, reduce); "
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
    vals, walls = [], []
    base = None
    for s in range(args.warmup + args.steps):
        r = cpu_baseline(wl, n_pairs, n, seconds=args.ref_seconds, seed=s, k=args.k)
        if s >= args.warmup:
            vals.append(r["value"])
            walls.append(r["wall_s"])
            base = r
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": "pairwise CV distances/s", "value": value,
        "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.mean(walls)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (java float path)",
        "data": "synthetic",
        "config": {"workload": workload_text(args.workload, args.k, n)},
        "step": ("one bounded sample of the workload: buildCPU of a seeded sample of proteomes "
                 "and compareCPU of pairs of them for about ref_seconds of wall time; value = "
                 "the whole workload's pairs over the time extrapolated from the sample; "
                 "ms_per_step = the wall time a sample took"),
        "extrapolated": base["extrapolated"],
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

# configurations the bench tunes over during warm-up (the tuner's space, trimmed
# to the shapes that can win on full-size K = 6 / K = 7 workloads)
BENCH_TUNE_SPACE = [
    dict(algorithm="window", wshift=11, tile_rows=16, tile_cols=256, fold=28, items_per_cta=16),
    dict(algorithm="window", wshift=11, tile_rows=16, tile_cols=128, fold=28, items_per_cta=16),
    dict(algorithm="window", wshift=11, tile_rows=16, tile_cols=256, fold=28, items_per_cta=8),
    dict(algorithm="window", wshift=11, tile_rows=16, tile_cols=128, fold=28, items_per_cta=8),
    dict(algorithm="postings", block=128, wshift=9, items_per_cta=4),
    dict(algorithm="postings", block=64, wshift=9, items_per_cta=4),
]


def kernel_name(cfg) -> str:
    if cfg.algorithm == "postings":
        return f"k_postings<{cfg.block}>"
    if cfg.tile_rows == 32:
        return "k_allpairs32"
    lpc = 2 if cfg.tile_cols == 256 else 4
    threads = cfg.tile_cols * lpc
    return f"k_allpairs<{threads},{1 if threads == 512 else 512 // threads},{lpc}>"


def fit_cost_model(cycles: np.ndarray, est: np.ndarray) -> dict:
    """Least-squares fit cycles ~ a * est + b over the items: R^2 and the worst
    item's measured / fitted ratio."""
    c = np.asarray(cycles, np.float64)
    e = np.asarray(est, np.float64)
    if len(c) < 3 or np.all(e == e[0]):
        return {"r2": None, "worst_ratio": None}
    A = np.stack([e, np.ones_like(e)], 1)
    coef, *_ = np.linalg.lstsq(A, c, rcond=None)
    fit = A @ coef
    ss_res = float(np.sum((c - fit) ** 2))
    ss_tot = float(np.sum((c - c.mean()) ** 2))
    worst = float(np.max(c / np.maximum(fit, 1.0)))
    return {"r2": 1.0 - ss_res / ss_tot if ss_tot > 0 else None, "worst_ratio": worst}


def run_ours(args):
    import dataclasses
    import torch
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    from rocket_gb300 import synth
    from rocket_gb300.engine import BatchBuilder, EngineConfig, PairEngine, autotune

    t0 = time.perf_counter()
    wl = synth.workload(args.workload, n=args.proteomes)
    t_gen = time.perf_counter() - t0
    N = len(wl)
    n_pairs = N * (N - 1) // 2
    stream = torch.cuda.current_stream(dev)
    pinned = torch.from_numpy(wl.data).pin_memory()
    seq = torch.empty(pinned.numel(), dtype=torch.uint8, device=dev)
    seq.copy_(pinned)
    builder = BatchBuilder("protein", args.k, device=dev, max_batch=args.max_batch,
                           overlap=not args.no_overlap)
    out = torch.zeros((N, N), dtype=torch.float64, device=dev)
    out_host = torch.zeros((N, N), dtype=torch.float64).pin_memory()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    # warm-up 1: build, then tune the pair engine on the built arena
    arena = builder.build(seq, wl.offsets, stream=stream)
    torch.cuda.synchronize()
    tuned = None
    space = [c for c in BENCH_TUNE_SPACE
             if (not args.algorithm or c["algorithm"] == args.algorithm)
             and (not args.tile_cols or c.get("tile_cols") == args.tile_cols)]
    if args.wshift:
        space = [dict(c, wshift=args.wshift) if c["algorithm"] == "window" else c for c in space]
    fields = {f.name for f in dataclasses.fields(EngineConfig)}
    if not args.no_tune and len(space) > 1:
        t0 = time.perf_counter()
        tuned = autotune(arena, space=space, repeats=1, use_cache=False, include_merge=False,
                         prune=1.5)
        t_tune = time.perf_counter() - t0
        cfg = EngineConfig(**{k: v for k, v in tuned.items() if k in fields})
    else:
        cfg = EngineConfig(**{k: v for k, v in space[0].items() if k in fields})
        t_tune = 0.0
    engine = PairEngine(arena, cfg)
    engine.ensure_index(stream)
    plan = engine.plan_triangle()
    graph = None if args.no_graph else engine.capture(plan, out)
    torch.cuda.synchronize()

    def step(events=None, host=None):
        nonlocal arena
        arena = builder.build(seq, wl.offsets, arena=arena.reset(), stream=stream, host=host)
        engine.arena = arena
        if events is not None:
            events[1].record(stream)
        engine.ensure_index(stream)
        if events is not None:
            events[2].record(stream)
        if graph is not None:
            with torch.cuda.stream(stream):
                graph.replay()
        else:
            engine.run(plan, out, stream=stream)
        if events is not None:
            events[3].record(stream)

    for _ in range(max(args.warmup - 1, 0)):
        step()
    torch.cuda.synchronize()
    nnz = arena.nnz.copy()
    alg_bytes = int(8 * (N - 1) * nnz.sum())       # one read of both vectors per pair
    build_bytes = int(wl.data.nbytes + 8 * nnz.sum())  # residues in, key/value lists out

    # timed device-resident steps
    b0, e0 = builder.launches, engine.launches
    step_ms, phase_ms = [], []
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index or 0) as clocks:
        for s in range(args.steps):
            flush.fill_(s & 0xFF)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            ev[0].record(stream)
            step(events=ev)
            torch.cuda.synchronize()
            step_ms.append(ev[0].elapsed_time(ev[3]))
            phase_ms.append((ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2]),
                             ev[2].elapsed_time(ev[3])))
    graph_launches = 2 if graph is not None else 0  # pair kernel + reduction per replay
    launches = (builder.launches - b0 + engine.launches - e0) / args.steps + graph_launches
    total_s = _barrier_max(sum(step_ms) / 1000.0, world)
    value = world * args.steps * n_pairs / total_s
    status = engine.device_status() if cfg.algorithm == "postings" else 0

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
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return 0

    # cost model of the item schedule, fitted to the kernel's per-item durations
    cyc = torch.zeros(max(plan.nitems, 1), dtype=torch.int64, device=dev)
    engine.run(plan, out, item_cycles=cyc)
    torch.cuda.synchronize()
    c = cyc.cpu().numpy()[:plan.nitems]
    models = engine.item_cost_models(plan)
    cost_fit = {name: fit_cost_model(c, est) for name, est in models.items()}
    cost_fit["used"] = "nnz_product" if cfg.algorithm == "postings" else "linear"

    peak, peak_kind = _peaks()
    clk = clocks.summary()
    b_ms, i_ms, p_ms = (float(np.mean([p[j] for p in phase_ms])) for j in range(3))
    name = kernel_name(cfg)
    ctr = PAIR_KERNEL_COUNTERS.get((name, args.workload, args.k, cfg.wshift)) \
        if args.proteomes is None else None
    traffic = float(ctr["dram_bytes"]) if ctr else None
    achieved = traffic / (p_ms / 1000.0) / 1e9 if traffic else None
    sm_hz = (clk["sm_mhz"] or 2070.0) * 1e6
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    roofline = {
        "kernel": name, "bound": "shared", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak if achieved else None, "traffic": traffic,
        "time_ms": p_ms,
        "note": (f"{peak_kind} HBM peak; achieved = DRAM bytes per launch (ncu capture of the "
                 "same kernel, workload and window width) over the event-timed pair phase "
                 "(graph: counter reset, pair kernel, reduction); the kernel's own bound is "
                 "the shared-memory pipe (smem below)"),
        "algorithmic": {
            "bytes": alg_bytes, "GBps": alg_bytes / (p_ms / 1000.0) / 1e9,
            "over_hbm_peak": alg_bytes / (p_ms / 1000.0) / 1e9 / peak,
            "note": "8*(nnz_i + nnz_j) per pair, each vector read once per pair: above 1 = "
                    "reuse of resident vectors (shared memory, L2), not DRAM bandwidth"},
    }
    if ctr and ctr.get("smem_wavefronts"):
        wf = float(ctr["smem_wavefronts"])
        roofline["smem"] = {"wavefronts": wf, "per_s": wf / (p_ms / 1000.0),
                            "peak_per_s": sms * sm_hz, "frac": wf / (p_ms / 1000.0) / (sms * sm_hz),
                            "note": "one shared-memory wavefront per SM per clock at the "
                                    "median sampled SM clock"}
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
            "engine": {k: v for k, v in dataclasses.asdict(cfg).items()
                       if k in ("algorithm", "wshift", "block", "tile_rows", "tile_cols", "fold",
                                "items_per_cta", "compress")},
            "tuned": None if tuned is None else {
                "seconds": t_tune,
                "candidates": [{k: v for k, v in c.items() if k != "candidates"}
                               for c in tuned["candidates"]]},
            "pair_phase": "CUDA graph replay" if graph is not None else "eager launches",
            "windows": int(arena.R), "items": plan.nitems, "tiles": plan.ntiles,
            "cost_model_fit": cost_fit,
            "generate_s": t_gen,
        },
        "breakdown_ms": {"build": b_ms, "key_ranks_and_window_index": i_ms,
                         "pair_phase": p_ms, "step": float(np.mean(step_ms))},
        "roofline": roofline,
        "build_roofline": {"bound": "hbm", "achieved": build_bytes / (b_ms / 1000.0) / 1e9,
                           "peak": peak, "unit": "GB/s",
                           "frac": build_bytes / (b_ms / 1000.0) / 1e9 / peak,
                           "bytes": build_bytes,
                           "note": "residues in + 8 B per output entry (L + 8 nnz per proteome)"},
        "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": float(np.mean(e2e_ms))},
        "clocks": clk,
        "gpu_launches": int(round(launches)),
        "device_status": status,
    }
    del graph
    if not args.no_plain:
        try:
            line["plain"] = plain_path(arena, wl, seq, dev, n_pairs, N, peak, k=args.k)
        except Exception as e:  # an informative leg: recorded, the line is still printed
            line["plain"] = {"error": repr(e)}
    if not args.no_cpu_baseline:
        cb = cpu_baseline(wl, n_pairs, N, seconds=args.ref_seconds, k=args.k)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample",
                                                   "extrapolated")}
        # the same port on one thread (a bounded sample: one proteome, compared with itself)
        c1 = cpu_baseline(wl, n_pairs, N, seconds=2.0, threads=1, k=args.k, n_sample=1)
        line["cpu_baseline"]["single_thread"] = {k: c1[k] for k in ("value", "unit", "cores",
                                                                    "sample", "extrapolated")}
    if not args.no_serve and world == 1:
        del engine, arena, builder, out, flush, seq
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        try:
            line["serve"] = serve_run(args, short=True)
        except Exception as e:  # the serving sub-run must not take the headline line with it
            line["serve"] = {"metric": "serve latency per query batch", "error": repr(e)}
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


# ----------------------------------------------------------------------------
# serving
# ----------------------------------------------------------------------------

SERVE_TEXT = ("serve2048: device-resident database of {db:,} synthetic proteomes (seed 4, protein "
              "counts lognormal median 1,900 sigma 0.9 clipped to [300, 12,000]), K=6; {nb} query "
              "batches of U(1..64) proteomes of the same distribution arriving as a Poisson "
              "process at {rate:g} per second; each query built, compared with the whole "
              "database, then appended; HBM budget {budget:g} GB")


def serve_run(args, short: bool = False) -> dict:
    """Serving measurement; ``short``: the sub-run of the default bench line (fewer
    query batches)."""
    import torch
    from rocket_gb300 import synth
    from rocket_gb300.engine import EngineConfig
    from rocket_gb300.serve import Request, ServingEngine, percentile

    rng = np.random.default_rng(4)
    nbatches = args.serve_batches if short else args.query_batches
    sizes = rng.integers(1, 65, size=nbatches)
    n_db = args.db
    total_q = int(sizes.sum())
    warm = 2
    t0 = time.perf_counter()
    wl = synth.workload("serve2048", n=n_db, extra=total_q + warm)
    t_gen = time.perf_counter() - t0
    db = wl.subset(range(n_db))
    srv = ServingEngine("protein", 6, budget_bytes=args.budget_gb * 1e9, slots=args.slots,
                        max_batch=64, cfg=EngineConfig(algorithm="window", wshift=11, fold=28,
                                                       tile_rows=16, tile_cols=128,
                                                       segments=args.segments))
    capacity_entries = int(min(np.sum(8 * wl.lengths() + 64),
                               (args.budget_gb * 1e9 - 20e9) / 8.0))
    t0 = time.perf_counter()
    srv.load(db, capacity_vectors=len(wl), capacity_entries=capacity_entries)
    torch.cuda.synchronize()
    t_load = time.perf_counter() - t0
    tuned = srv.tune()  # item width for query batches
    srv.start()
    nxt = n_db
    for w in range(warm):  # warm-up requests (one proteome each), not measured
        r = srv.submit(Request(-1 - w, wl.subset([nxt]), append=False))
        nxt += 1
        r.done.wait(600)
    batches = []
    for b in range(nbatches):
        batches.append(wl.subset(range(nxt, nxt + int(sizes[b]))))
        nxt += int(sizes[b])
    gaps = rng.exponential(1.0 / args.rate, size=nbatches)
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
    offered = sum(len(r.proteomes) * r.db_n for r in reqs) / max(sum(gaps), 1e-9)
    line = {
        "metric": "serve latency per query batch", "p50_ms": percentile(lat, 50),
        "p99_ms": percentile(lat, 99), "max_ms": max(lat) if lat else None,
        "value": pairs / (t_end - t_start), "unit": "pairs/s (sustained)",
        "offered_pairs_per_s": offered,
        "requests": len(reqs), "query_proteomes": total_q, "errors": len(errors),
        "arrival_rate_per_s": args.rate, "slots": args.slots, "batches_run": srv.batches,
        "db_start": n_db, "db_end": srv.db.arena.n, "db_appends_refused": srv.db.refused,
        "hbm_budget_gb": args.budget_gb, "hbm_reserved_peak_gb": srv.budget.peak / 1e9,
        "db_load_s": t_load, "generate_s": t_gen, "data": "synthetic",
        "config": {"workload": SERVE_TEXT.format(db=n_db, nb=nbatches, rate=args.rate,
                                                 budget=args.budget_gb),
                   "segments": args.segments, "window_shift": 11, "keys": "raw keys",
                   "tile_cols": srv.cfg.tile_cols, "tuned": tuned},
        "clocks": clocks.summary(),
    }
    if errors:
        line["first_error"] = errors[0]
    return line


def run_serve(args):
    line = serve_run(args)
    print(json.dumps(line), flush=True)
    return 0 if not line["errors"] else 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOAD_TEXTS))
    ap.add_argument("--k", type=int, default=6, help="K-mer length (protein)")
    ap.add_argument("--proteomes", type=int, default=None,
                    help="use only the first N proteomes (small profiling cases)")
    ap.add_argument("--algorithm", default=None, choices=["window", "postings"],
                    help="restrict the tuned pair kernel to one algorithm")
    ap.add_argument("--tile-cols", type=int, default=0, choices=[0, 128, 256],
                    help="restrict the tuned window kernel to items of this many columns")
    ap.add_argument("--wshift", type=int, default=0,
                    help="window engine: key window 2^wshift ranks (default: the tuned space's)")
    ap.add_argument("--no-tune", action="store_true",
                    help="no tuning: the first configuration of the bench's space")
    ap.add_argument("--no-graph", action="store_true", help="eager launches of the pair phase")
    ap.add_argument("--no-overlap", action="store_true",
                    help="build one batch at a time instead of two in flight")
    ap.add_argument("--max-batch", type=int, default=24)
    ap.add_argument("--ref-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the per-pair ABI measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving sub-run")
    ap.add_argument("--mode", default="allpairs", choices=["allpairs", "serve"])
    ap.add_argument("--db", type=int, default=2048, help="serve: database proteomes")
    ap.add_argument("--query-batches", type=int, default=24, help="serve: arriving query batches")
    ap.add_argument("--serve-batches", type=int, default=12,
                    help="query batches of the serving sub-run of the default line")
    ap.add_argument("--rate", type=float, default=4.0, help="serve: query batches per second")
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
