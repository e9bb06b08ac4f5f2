"""Distance output and the command-line driver of the phylogenetics application.

`write_output` restates Main.writeOutput (phylogenetics_analysis/Main.java:204-251):
a JSON object with "files" (the input paths) and "distance", an n x n matrix
whose entry (i, j) is the coefficient of the pair and -1 where no pair was
computed.  Like the reference, the value stored under "distance" is the cosine
C (SequenceAnalysisContext.java:134-136 returns C); `as_distance=True` writes
D = (1 - C) / 2 instead.  The file order is the order given (the reference's is
HashMap iteration order, which is not stable across runs).

`main` mirrors the reference's `genetics` command (Main.java:43-61, 132-202):
every *.faa, *.faa.gz, *.fasta and *.fasta.gz file under the input directory is
read (ReadFasta rules), built into a composition vector and compared with every
other file and itself; the result is written with `write_output`.
"""
from __future__ import annotations

import argparse
import json
import os
from typing import List, Optional, Sequence

import numpy as np

SUFFIXES = (".faa", ".faa.gz", ".fasta", ".fasta.gz")


def write_output(path: str, files: Sequence[str], C: np.ndarray, computed: Optional[np.ndarray] = None,
                 as_distance: bool = False) -> None:
    """Writes {"files": [...], "distance": [[...]]}; entries not `computed` are -1."""
    C = np.asarray(C, dtype=np.float64)
    n = len(files)
    if C.shape != (n, n):
        raise ValueError(f"matrix shape {C.shape} does not match {n} files")
    vals = (1.0 - C) / 2.0 if as_distance else C
    if computed is None:
        computed = np.ones((n, n), dtype=bool)
    rows: List[List[float]] = []
    for i in range(n):
        rows.append([float(vals[i, j]) if computed[i, j] else -1 for j in range(n)])
    with open(path, "w", encoding="utf-8") as f:
        json.dump({"files": list(files), "distance": rows}, f, indent=1)


def scan_directory(root: str) -> List[str]:
    """Input files under `root` (relative paths, sorted), as Util.scanDirectory with
    the suffix filter of Main.java:166-172."""
    out = []
    for dirpath, _, names in os.walk(root):
        for name in names:
            if name.lower().endswith(SUFFIXES):
                out.append(os.path.relpath(os.path.join(dirpath, name), root))
    return sorted(out)


def run_directory(root: str, k: int = 6, alphabet: str = "protein", device=None):
    """Reads, builds and compares every input file under `root`; returns (files, C)."""
    import torch

    from .engine import BatchBuilder, EngineConfig, PairEngine, auto_tile_cols
    from .fasta import parse_file_bytes

    files = scan_directory(root)
    if not files:
        raise FileNotFoundError(f"no .faa/.fasta(.gz) files under {root}")
    seqs = []
    for rel in files:
        with open(os.path.join(root, rel), "rb") as f:
            seqs.append(parse_file_bytes(f.read(), rel))
    lens = np.array([len(s) for s in seqs], np.int64)
    off = np.zeros(len(seqs) + 1, np.int64)
    np.cumsum(lens, out=off[1:])
    dev = torch.device(device if device is not None else "cuda")
    data = np.frombuffer(b"".join(seqs), dtype=np.uint8)
    seq = torch.from_numpy(data.copy()).to(dev)
    arena = BatchBuilder(alphabet, k, device=dev).build(seq, off)
    engine = PairEngine(arena, EngineConfig(tile_cols=auto_tile_cols(arena.n)))
    engine.ensure_index()
    out = torch.zeros((arena.n, arena.n), dtype=torch.float64, device=dev)
    engine.run(engine.plan_triangle(), out)
    return files, out.cpu().numpy()


def main(argv: Optional[Sequence[str]] = None) -> int:
    ap = argparse.ArgumentParser(prog="python -m rocket_gb300.output",
                                 description="all-pair composition-vector comparison of a "
                                             "directory of FASTA files")
    ap.add_argument("input_dir")
    ap.add_argument("output_file")
    ap.add_argument("-k", "--k", type=int, default=6, help="length of k-mers")
    ap.add_argument("--alphabet", default="protein", choices=["protein", "DNA"])
    ap.add_argument("--as-distance", action="store_true",
                    help="write D = (1 - C) / 2 instead of the cosine C")
    args = ap.parse_args(argv)
    if not os.path.isdir(args.input_dir):
        ap.error(f"path does not exist or is not a directory: {args.input_dir}")
    files, C = run_directory(args.input_dir, args.k, args.alphabet)
    write_output(args.output_file, files, C, as_distance=args.as_distance)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
