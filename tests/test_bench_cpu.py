"""bench.py's host side on the CPU: the reference arm's JSON line, the kernel names
that key the ncu counter table, and the cost-model fit.  No GPU: the reference arm is
the Java CPU path (the oracle's C port), timed on a small bounded sample here."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from rocket_gb300.engine import EngineConfig  # noqa: E402


def test_reference_arm_line():
    """The reference arm as launched from the command line: exit 0 and exactly one
    JSON line on stdout, with the contract's keys."""
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "cpu16", "--proteomes", "4", "--steps", "1",
                        "--warmup", "0", "--ref-seconds", "0.2"],
                       capture_output=True, text=True, env=env, cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.strip()]
    assert len(lines) == 1 and lines[0].startswith("{"), r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "pairwise CV distances/s" and d["unit"] == "pairs/s"
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 0
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"].startswith("cpu16")
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert "buildCPU" in cb["sample"] and "compareCPU" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    ex = d["extrapolated"]
    assert ex["builds"] == 4 and ex["pairs"] == 6


def test_cpu_baseline_single_proteome_sample():
    """One sampled proteome compares its vector with itself (no pair among one)."""
    from rocket_gb300 import synth
    wl = synth.workload("cpu16", n=2)
    r = bench.cpu_baseline(wl, 1, 2, seconds=0.2, threads=1, k=6, n_sample=1)
    assert r["cores"] == 1 and r["value"] > 0
    assert r["extrapolated"]["sampled_builds"] == 1 and r["extrapolated"]["sampled_pairs"] >= 1


@pytest.mark.parametrize("cfg,name", [
    (dict(tile_rows=16, tile_cols=256), "k_allpairs<512,1,2>"),
    (dict(tile_rows=16, tile_cols=128), "k_allpairs<512,1,4>"),
    (dict(tile_rows=16, tile_cols=64), "k_allpairs<256,2,4>"),
    (dict(tile_rows=16, tile_cols=32), "k_allpairs<128,4,4>"),
    (dict(tile_rows=32, tile_cols=64), "k_allpairs32"),
    (dict(algorithm="postings", block=128), "k_postings<128>"),
])
def test_kernel_names(cfg, name):
    assert bench.kernel_name(EngineConfig(**cfg)) == name


def test_counter_table_keys_name_the_bench_kernel():
    """The ncu counters the bench reports as roofline.traffic are keyed by the
    kernel the bench's first tune-space entry launches, per workload, K and window
    width; every workload named exists."""
    first = EngineConfig(**{k: v for k, v in bench.BENCH_TUNE_SPACE[0].items()
                            if k in EngineConfig.__dataclass_fields__})
    for (kern, wl, k, wshift), ctr in bench.PAIR_KERNEL_COUNTERS.items():
        assert kern == bench.kernel_name(first)
        assert wshift == first.wshift
        assert wl in bench.WORKLOAD_TEXTS
        assert ctr["dram_bytes"] > 0 and ctr["smem_wavefronts"] > 0


def test_fit_cost_model():
    rng = np.random.default_rng(0)
    est = rng.uniform(1, 100, 500)
    exact = bench.fit_cost_model(3.0 * est + 7.0, est)
    assert exact["r2"] == pytest.approx(1.0) and exact["worst_ratio"] == pytest.approx(1.0)
    noisy = bench.fit_cost_model(3.0 * est * rng.uniform(0.8, 1.2, 500), est)
    assert 0.5 < noisy["r2"] < 1.0 and 1.0 < noisy["worst_ratio"] < 1.5
    assert bench.fit_cost_model(est[:2], est[:2]) == {"r2": None, "worst_ratio": None}
    assert bench.fit_cost_model(est, np.ones(500)) == {"r2": None, "worst_ratio": None}
