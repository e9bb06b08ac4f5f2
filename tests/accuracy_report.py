"""Accuracy of the device path against the CPU oracle, per workload.

Test infrastructure (uses oracle/).  For a sample of proteomes of a workload:
  * composition vectors built on the device (batched build) vs the oracle's
    restatement of the reference rule: keys bit-exact, values max ulp distance;
  * D = (1 - C) / 2 for every pair of the sample from the all-pair engine (window
    kernel) and from the multi-pair merge kernel vs the FP64 oracle (exact
    products, double-double sum): max and p99 |dD|.

Usage (GPU):  python tests/accuracy_report.py --workload uniform256 --sample 48 --k 6
Writes a markdown section to stdout (and to --out if given).
"""
import argparse
import os
import sys
import time
from concurrent.futures import ProcessPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _oracle_cv(args):
    seq, k = args
    from oracle import oracle as O
    r = O.cv_native(seq, k)
    return r["keys"], r["values"]


def _oracle_pairs(vecs, pairs):
    import ctypes
    from oracle import oracle as O
    L = O.lib()
    u32p, f32p = ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_float)
    out = np.zeros(len(pairs))
    for n, (i, j) in enumerate(pairs):
        ki, vi = vecs[i]
        kj, vj = vecs[j]
        out[n] = L.oracle_compare_fp64(ki.ctypes.data_as(u32p), vi.ctypes.data_as(f32p), len(ki),
                                       kj.ctypes.data_as(u32p), vj.ctypes.data_as(f32p), len(kj))
    return out


def ulp_max(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return int(np.abs(a - b).max()) if len(a) else 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="uniform256")
    ap.add_argument("--sample", type=int, default=48)
    ap.add_argument("--k", type=int, default=6)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--out", default=None)
    ap.add_argument("--tile-cols", type=int, default=128, choices=[32, 64, 128, 256],
                    help="column vectors per pair-kernel work item (256: two lanes per column)")
    args = ap.parse_args()

    # CPU pool first: it must not be forked after CUDA initialises
    pool = ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 4))
    import torch
    from rocket_gb300 import synth
    from rocket_gb300.engine import BatchBuilder, EngineConfig, PairEngine

    w = synth.WORKLOADS[args.workload]
    rng = np.random.default_rng(args.seed)
    full = synth.workload(args.workload)
    ids = np.sort(rng.choice(len(full), min(args.sample, len(full)), replace=False))
    p = full.subset(ids)
    n = len(p)
    t0 = time.perf_counter()
    oracle = list(pool.map(_oracle_cv, [(p.get(i), args.k) for i in range(n)]))
    t_or = time.perf_counter() - t0

    arena = BatchBuilder("protein", args.k).build(torch.from_numpy(p.data).cuda(), p.offsets)
    torch.cuda.synchronize()
    key_ok, ulp = True, 0
    for i in range(n):
        k, v = arena.host_vector(i)
        key_ok &= bool(np.array_equal(k, oracle[i][0]))
        if len(k) == len(oracle[i][0]):
            ulp = max(ulp, ulp_max(v, oracle[i][1]))

    eng = PairEngine(arena, EngineConfig(tile_cols=args.tile_cols))
    eng.ensure_index()
    C = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    eng.run(eng.plan_triangle(), C)
    Cw = C.cpu().numpy()
    iu = np.triu_indices(n, 1)
    Cm = eng.compare_pairs_merge(iu[0], iu[1]).cpu().numpy()
    pairs = list(zip(iu[0].tolist(), iu[1].tolist()))
    exact = _oracle_pairs(oracle, pairs)
    pool.shutdown()
    dD_w = np.abs((1 - Cw[iu]) / 2 - (1 - exact) / 2)
    dD_m = np.abs((1 - Cm) / 2 - (1 - exact) / 2)
    diag = np.abs(np.diag(Cw) - 1.0)

    nnz = arena.nnz
    lines = [
        f"### {args.workload}, K={args.k}: {n} proteomes sampled (seed {args.seed}), {len(pairs)} pairs, "
        f"pair items 16 x {args.tile_cols}",
        "",
        "| check | result |",
        "|---|---|",
        f"| keys vs oracle (all {n} vectors) | {'bit-exact' if key_ok else 'MISMATCH'} |",
        f"| values vs oracle, max distance | {ulp} ulp |",
        f"| vector sizes (nnz) min / median / max | {nnz.min():,} / {int(np.median(nnz)):,} / {nnz.max():,} |",
        f"| window kernel max abs dD | {dD_w.max():.3e} |",
        f"| window kernel p99 abs dD | {np.percentile(dD_w, 99):.3e} |",
        f"| merge kernel max abs dD | {dD_m.max():.3e} |",
        f"| merge kernel p99 abs dD | {np.percentile(dD_m, 99):.3e} |",
        f"| self products max abs(C_ii - 1) | {diag.max():.3e} |",
        f"| oracle time (CPU, {min(16, os.cpu_count() or 4)} processes) | {t_or:.1f} s for the vectors |",
        "",
    ]
    text = "\n".join(lines)
    print(text)
    if args.out:
        with open(args.out, "a") as f:
            f.write(text + "\n")
    ok = key_ok and ulp <= 1 and dD_w.max() <= 1e-6 and dD_m.max() <= 1e-6
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
