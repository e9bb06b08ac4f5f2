"""The C-ABI library loads and exports every symbol include/phylogenetics.h
declares; host-only entry points (scratch sizing) behave like the reference's
(native.cu:705-716).  No device work runs here."""
import ctypes
import os
import re
import subprocess

import pytest

from rocket_gb300 import _native, build as nbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "phylogenetics.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"^\s*(?:long|int|void)\s+(\w+)\s*\(", text, flags=re.M)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(nbuild.LIB):
        nbuild.build()
    return _native.load()


def test_header_lists_the_boundary():
    syms = declared_symbols()
    assert syms[:3] == ["estimateScratchMemory", "buildCompositionVector",
                        "compareCompositionVectors"]
    assert sorted(syms) == sorted(_native.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", nbuild.LIB], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(\w+)$", out, flags=re.M))
    for s in declared_symbols():
        assert s in exported, s
        assert getattr(lib, s) is not None


def test_library_name_matches_jna_load():
    # Native.load("phylogenetics") resolves libphylogenetics.so (Bindings.java:15)
    assert os.path.basename(nbuild.LIB) == "libphylogenetics.so"


def test_estimate_scratch_memory(lib):
    est = lambda a, k, m: lib.estimateScratchMemory(a.encode(), k, m)
    p = [est("protein", 6, m) for m in (0, 1000, 10 ** 6, 10 ** 8)]
    assert all(x > 0 for x in p) and p == sorted(p)
    # protein k=6 needs less than the reference's dense 21^6 uint32 table (343 MB)
    assert est("protein", 6, 3 * 10 ** 6) < 21 ** 6 * 4
    # any alphabet other than "DNA" is sized as protein (native.cu:710-712)
    assert est("nonsense", 5, 1000) == est("protein", 5, 1000)
    assert est("DNA", 5, 1000) < est("protein", 5, 1000)
    # invalid k: only the compare part is sized (the build call rejects k)
    assert est("protein", 2, 1000) > 0 and est("protein", 11, 1000) > 0


def test_batch_scratch_rejects_bad_arguments(lib):
    f = lambda a, k, b, c: lib.phyloBuildBatchScratch(a.encode(), k, b, c)
    assert f("protein", 6, 4, 1000) > 0
    assert f("protein", 2, 4, 1000) == -1
    assert f("protein", 8, 4, 1000) == -1  # 21^8 keys do not fit uint32
    assert f("dna", 6, 4, 1000) == -1
    assert f("DNA", 10, 4, 1000) > 0
    assert lib.phyloBuildLaunchesPerBatch() > 0
    assert lib.phyloPairsSmemBytes(10, 16, 64) == (1024 + 1) * 80 + 2 * 256 * 32  # table + ring
    assert lib.phyloPairsSmemBytes(9, 16, 32) == (512 + 1) * 80 + 2 * 128 * 32
    assert lib.phyloPairsSmemBytes(10, 32, 64) == (1024 + 1) * 128
    assert lib.phyloPairsSmemBytes(10, 24, 64) == -1 and lib.phyloPairsSmemBytes(10, 32, 32) == -1
    assert lib.phyloPairsThreads(10, 32, 64) == 512 and lib.phyloPairsThreads(9, 32, 64) == 256
    assert lib.phyloPairsThreads(10, 16, 64) == 256 and lib.phyloPairsThreads(9, 16, 32) == 128
    assert lib.phyloPairsThreads(11, 16, 128) == 512
