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


def _prototypes():
    """(return type, name, [parameter types]) of every function the header declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = []
    for ret, name, args in re.findall(
            r"^\s*((?:unsigned\s+)?(?:long|int|void))\s+(\w+)\s*\(([^)]*)\)\s*;", text, flags=re.M):
        params = []
        for a in args.split(","):
            a = " ".join(a.split())
            if a in ("", "void"):
                continue
            params.append(re.sub(r"\s*\b\w+$", "", a).strip())
        out.append((ret, name, params))
    return out


def _ctype_ok(c_type: str, declared) -> bool:
    """Whether the ctypes declaration passes the C type with the same width and
    register class (LP64: long and pointers are 64-bit; addresses may be passed
    as uintptr_t-sized integers)."""
    if c_type == "int":
        return declared is ctypes.c_int
    if c_type == "unsigned int":
        return declared is ctypes.c_uint
    if c_type == "long":
        return declared is ctypes.c_long
    if c_type == "const char *":
        return declared is ctypes.c_char_p
    if c_type == "uintptr_t" or c_type.endswith("*"):
        return declared is ctypes.c_size_t or (
            isinstance(declared, type) and issubclass(declared, ctypes._Pointer))
    raise AssertionError(f"no rule for C type {c_type!r}")


def test_ctypes_declarations_match_the_header(lib):
    """Every prototype in include/phylogenetics.h and the ctypes declaration the
    Python side calls it through agree on the parameter count and on each
    parameter's and the result's width."""
    protos = _prototypes()
    assert sorted(n for _, n, _ in protos) == sorted(_native.EXPORTED)
    rets = {"int": ctypes.c_int, "long": ctypes.c_long, "void": None}
    for ret, name, params in protos:
        f = getattr(lib, name)
        assert f.restype is rets[ret], name
        assert len(f.argtypes) == len(params), (name, len(f.argtypes), len(params))
        for i, (c_type, declared) in enumerate(zip(params, f.argtypes)):
            assert _ctype_ok(c_type, declared), (name, i, c_type, declared)


def test_negative_sizes_refused_before_device_work(lib):
    """Every entry point that takes a count or a byte size refuses a negative one
    with cudaErrorInvalidValue before any device call (cast to an unsigned size it
    would launch grids over memory the caller never passed).  No GPU here: a call
    that got past its checks would return a CUDA error other than 1."""
    INVALID = 1
    P = b"protein"
    buf = ctypes.create_string_buffer(256)
    h = ctypes.addressof(buf)
    z = [0] * 10
    calls = {
        "build scratch": lib.buildCompositionVector(0, 0, -1, P, 6, 0, 10, 0, 0, 0, 100),
        "compare scratch": lib.compareCompositionVectors(0, 0, -1, 0, 0, 1, 0, 0, 1, 0),
        "compare left": lib.compareCompositionVectors(0, 0, 100, 0, 0, -1, 0, 0, 1, 0),
        "static right": lib.compareCompositionVectorsStatic(0, 0, 0, 1, 0, 0, -1, 0),
        "plan cand": lib.phyloBuildBatchPlan(0, 0, 100, P, 6, 2, 0, 0, -1, h, h),
        "plan scratch": lib.phyloBuildBatchPlan(0, 0, -1, P, 6, 2, 0, 0, 100, h, h),
        "plan async": lib.phyloBuildBatchPlanAsync(0, 0, 100, P, 6, 2, 0, 0, -1, h),
        "emit base": lib.phyloBuildBatchEmit(0, 0, 100, P, 6, 2, 100, 0, 0, 0, -5, 0),
        "norms cand": lib.phyloBuildBatchNorms(0, 0, 100, P, 6, 2, -1, h),
        "counts null": lib.phyloBuildBatchCounts(0, 0, 100, P, 6, 2, 100, 0, 0, 0, 0),
        "window index n": lib.phyloWindowIndex(0, 0, 0, -1, 11, 10, 100, 0),
        "window index len": lib.phyloWindowIndex(0, 0, 0, 4, 11, 10, -1, 0),
        "pairs items": lib.phyloPairsLaunch(*([0] * 9), 10, 11, 0, 0, 0, -1, 0, 0, 28, 0,
                                            16, 256, 152),
        "pairs grid": lib.phyloPairsLaunch(*([0] * 9), 10, 11, 0, 0, 0, 4, 0, 0, 28, 0,
                                           16, 256, 0),
        "reduce tiles": lib.phyloPairsReduce(0, 0, 0, -1, 1, 16, 256, 0, 0, 0, 10, 1, 1),
        "reduce segments": lib.phyloPairsReduce(0, 0, 0, 3, 0, 16, 256, 0, 0, 0, 10, 1, 1),
        "reduce ldc": lib.phyloPairsReduce(0, 0, 0, 3, 4, 16, 256, 0, 0, 0, 0, 1, 1),
        "self dot n": lib.phyloSelfDot(0, 0, 0, -1, 10, 0, 0, 10),
        "self dot ldc": lib.phyloSelfDot(0, 0, 0, 4, 10, 0, 0, 0),
        "many pairs": lib.phyloComparePairsMany(0, 0, 100, *z, -1, 10, 0),
        "many tiles": lib.phyloComparePairsMany(0, 0, 100, *z, 4, -1, 0),
        "pair async": lib.phyloComparePairAsync(0, 0, 100, 0, 0, -1, 0, 0, 1, 0),
        "ranks len": lib.phyloKeyRanks(0, 0, 10 ** 12, 21 ** 6, 0, 0, 2, -1, 0, 0, 0),
        "rank index len": lib.phyloKeyRankIndex(0, 0, 10 ** 12, 21 ** 6, 0, 0, 2, -1, 100, 0,
                                                11, 10, 0, 0),
        "postings items": lib.phyloPostingsLaunch(*([0] * 9), 10, 9, 0, 0, 0, -1,
                                                  0, 0, 0, 0, 128, 152),
        "postings tiles": lib.phyloPostingsReduce(0, 0, 0, -1, 128, 0, 0, 0, 10, 1, 1),
    }
    bad = {k: v for k, v in calls.items() if v != INVALID}
    assert not bad, bad
    assert lib.phyloSelfDotPartBytes(-1, 10) == -1 and lib.phyloSelfDotPartBytes(4, -1) == -1
    assert lib.phyloComparePairsManyScratch(-1, 10) == -1
    assert lib.phyloComparePairsManyScratch(4, -1) == -1
