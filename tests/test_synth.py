"""Synthetic workload generator: deterministic, related proteomes, stated sizes."""
import hashlib

import numpy as np

from rocket_gb300 import synth



def test_deterministic():
    a = synth.workload("cpu16", n=4)
    b = synth.workload("cpu16", n=4)
    assert np.array_equal(a.data, b.data) and np.array_equal(a.offsets, b.offsets)


def test_sizes_and_format():
    p = synth.workload("cpu16")
    assert len(p) == 16
    assert np.all(p.protein_counts == 1500)
    s = p.get(3)
    assert s[0:1] == b"\n" and s.count(b"\n") == 1500
    assert set(s) <= set(b"\nACDEFGHIKLMNPQRSTVWY")
    mean_len = (len(s) - 1500) / 1500
    assert 300 < mean_len < 380  # lognormal median 300, sigma 0.5 -> mean ~340


def test_related_but_distinct():
    p = synth.workload("cpu16", n=4)
    a = np.frombuffer(p.get(0), np.uint8)
    b = np.frombuffer(p.get(1), np.uint8)
    ident = float((a == b).mean())
    assert 0.3 < ident < 0.999


def test_uneven_counts_distribution():
    c = synth.uneven_counts(1024, 2)
    assert c.min() >= 300 and c.max() <= 12000
    assert 1500 < np.median(c) < 2300
