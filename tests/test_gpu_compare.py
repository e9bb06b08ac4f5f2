"""Pair compare on the device vs the oracles: the reference test's sweep
(BindingsTest.testCompareVectors, :204-213, tolerance 1e-5 vs the Java CPU
path) and the FP64 oracle (exact products, exact sum)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rocket_gb300 import synth
from rocket_gb300.context import SequenceAnalysisContext
from rocket_gb300.kernels import CompositionVectorKernels

from gpu_helpers import build_gpu

pytestmark = pytest.mark.gpu


def compare_gpu(lk, lv, rk, rv, slot_layout=False):
    n = max(len(lk), len(rk), 1)
    ker = CompositionVectorKernels("DNA", 3, n, 1)  # as BindingsTest.compareVectorGPU (:134)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    if slot_layout:
        # [keys | values] in one buffer, as SequenceAnalysisContext lays out a cache slot
        ls = torch.from_numpy(np.concatenate([np.asarray(lk, np.int32).view(np.uint8),
                                              np.asarray(lv, np.float32).view(np.uint8)])).cuda()
        rs = torch.from_numpy(np.concatenate([np.asarray(rk, np.int32).view(np.uint8),
                                              np.asarray(rv, np.float32).view(np.uint8)])).cuda()
        lkt, lvt = ls[:4 * len(lk)], ls[4 * len(lk):]
        rkt, rvt = rs[:4 * len(rk)], rs[4 * len(rk):]
    else:
        lkt = torch.from_numpy(np.asarray(lk, np.int32).copy()).cuda()
        lvt = torch.from_numpy(np.asarray(lv, np.float32).copy()).cuda()
        rkt = torch.from_numpy(np.asarray(rk, np.int32).copy()).cuda()
        rvt = torch.from_numpy(np.asarray(rv, np.float32).copy()).cuda()
    ker.compare_vectors_gpu(lkt, lvt, len(lk), rkt, rvt, len(rk), out)
    return float(out.item())


@pytest.mark.parametrize("n", [10, 100, 1000, 10000, 100000])
@pytest.mark.parametrize("ratio", [0.0, 0.5, 1.0])
def test_bindings_compare_sweep(n, ratio):
    for seed in range(4):
        lk, lv, rk, rv, minval = O.bindings_compare_case(seed, n, ratio)
        assert not minval
        gpu = compare_gpu(lk, lv, rk, rv)
        cpu = O.java_compare(lk, lv, rk, rv)
        assert abs(cpu - gpu) <= 1e-5  # BindingsTest.java:201
        exact = O.compare_fp64(lk.view(np.uint32), lv, rk.view(np.uint32), rv)
        assert abs(gpu - exact) <= 1e-12 * max(1.0, abs(exact))


@pytest.mark.parametrize("nl,nr", [(0, 0), (0, 5), (7, 0), (1, 1), (4096, 0), (2048, 2048),
                                   (4095, 1), (12288, 4096), (3, 5000), (33333, 1),
                                   (4352, 0), (4351, 1), (8704, 4352), (2176, 2176)])
def test_edge_sizes(nl, nr):
    rng = np.random.default_rng(nl * 7919 + nr)
    universe = np.sort(rng.choice(10 * (nl + nr) + 10, size=nl + nr + 10, replace=False))
    lk = np.sort(rng.choice(universe, nl, replace=False)).astype(np.int32)
    rk = np.sort(rng.choice(universe, nr, replace=False)).astype(np.int32)
    lv = rng.random(nl, dtype=np.float32)
    rv = rng.random(nr, dtype=np.float32)
    exact = O.compare_fp64(lk.view(np.uint32), lv, rk.view(np.uint32), rv)
    for slot in (False, True):
        assert abs(compare_gpu(lk, lv, rk, rv, slot) - exact) <= 1e-12 * max(1, abs(exact))


def test_identical_and_disjoint():
    k = np.arange(0, 300000, 3, dtype=np.int32)
    v = np.random.default_rng(0).random(len(k), dtype=np.float32)
    exact = O.compare_fp64(k.view(np.uint32), v, k.view(np.uint32), v)
    assert abs(compare_gpu(k, v, k, v) - exact) <= 1e-12 * exact
    assert compare_gpu(k, v, k + 1, v) == 0.0
    # odd lengths in the slot layout misalign the value arrays (4-byte aligned only)
    assert abs(compare_gpu(k[:-1], v[:-1], k[1:], v[1:], True) -
               O.compare_fp64(k[:-1].view(np.uint32), v[:-1], k[1:].view(np.uint32), v[1:])) < 1e-9


def test_composition_vector_distances():
    p = synth.workload("uniform256", n=4, scale=0.3)
    vecs = [build_gpu(p.get(i), 6) for i in range(4)]
    for i in range(4):
        for j in range(i, 4):
            ni, ki, vi = vecs[i]
            nj, kj, vj = vecs[j]
            gpu = compare_gpu(ki[:ni].view(np.int32), vi[:ni], kj[:nj].view(np.int32), vj[:nj])
            exact = O.compare_fp64(ki[:ni], vi[:ni], kj[:nj], vj[:nj])
            assert abs(O.distance(gpu) - O.distance(exact)) <= 1e-6
            if i == j:
                assert abs(gpu - 1.0) < 1e-5


def test_application_context_flow():
    """parseFiles -> preprocessInputGPU -> correlateGPU -> postprocessOutput."""
    from rocket_gb300 import fasta
    p = synth.workload("cpu16", n=3, scale=0.1)
    files = []
    for i in range(3):
        prots = p.get(i).split(b"\n")[1:]
        files.append(fasta.write_fasta(prots))
    ctx = SequenceAnalysisContext("protein", 6, 200000, 10 ** 6)
    slots = []
    for i, f in enumerate(files):
        parsed = ctx.parse_files(f"p{i}.faa", [f])
        assert parsed == p.get(i)
        d_in = torch.frombuffer(bytearray(parsed), dtype=torch.uint8).cuda()
        slot = torch.empty(ctx.get_max_input_size(), dtype=torch.uint8, device="cuda")
        used = ctx.preprocess_input_gpu(f"p{i}", d_in, slot)
        slots.append(slot[:used])
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for i in range(3):
        for j in range(3):
            ctx.correlate_gpu(i, slots[i], j, slots[j], out)
            c = ctx.postprocess_output(i, j, out.cpu().numpy().tobytes())
            ri = O.cv_native(p.get(i), 6)
            rj = O.cv_native(p.get(j), 6)
            exact = O.compare_fp64(ri["keys"], ri["values"], rj["keys"], rj["values"])
            assert abs(ctx.distance(c) - O.distance(exact)) <= 1e-6
    ctx.destroy()
