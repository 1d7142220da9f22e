"""CPU tests of the device code's formula chains: the pair plan and chains of the
any-length kernel (plan_int / finish_int / finish_jaro around the runtime-W cores,
rfg_core.cuh) and the tile kernels' per-query length tables (Jaro table, normalized
chains' integer cutoff) compiled for the host behind tests/cpp/host_chain.cpp, run on the
reference-made fixtures kat.json and random.json (free, Cached and Multi forms of Levenshtein
with every weight set, Indel, LCSseq, OSA, Jaro, Jaro-Winkler and ratio, all four ops,
every code-unit width, default and explicit cutoffs), ints equal and doubles bit for bit.
The fuzz fixtures of one-byte strings go through the host-compiled fuzz scorers
(tests/cpp/host_fuzz.cpp) the same way.  No GPU."""
import ctypes
import os
import shutil
import subprocess

import pytest

import golden_lib as G
from oracle_lib import ROOT, MULTI, Params, score

CSRC = os.path.join(ROOT, "rapidfuzz-cpp_gb300", "csrc")


def _build(name, sources, extra=()):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, name)
    subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-pthread", "-ffp-contract=off", "-I" + CSRC,
                    "-o", so] + list(sources) + list(extra), check=True)
    return ctypes.CDLL(so)


@pytest.fixture(scope="module")
def chain():
    lib = _build("libhost_chain.so", [os.path.join(ROOT, "tests", "cpp", "host_chain.cpp")])
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    for f in (lib.hc_score, lib.hc_score_tab):
        f.restype = I
        f.argtypes = [I, I, I, P, I64, I, P, I64, I, ctypes.POINTER(Params), ctypes.c_uint64, ctypes.c_double,
                      ctypes.POINTER(I64), ctypes.POINTER(ctypes.c_double)]
    return lib


@pytest.mark.parametrize("fixture", ["kat.json", "random.json"])
@pytest.mark.parametrize("entry", ["hc_score", "hc_score_tab"], ids=["any_length_path", "length_tables"])
def test_chains_match_reference_fixtures(chain, fixture, entry):
    fn = getattr(chain, entry)
    n, bad = 0, []
    for c in G.load(fixture):
        if c["metric"] > 6:
            continue
        a, b = G.arrays(c)
        v = score(fn, c["metric"], c["op"], c["form"], a, b, c["cutoff"], tuple(c["weights"]), c["pw"])
        n += 1
        if not G.same(v, G.dec(c["expected"])):
            bad.append((c, v))
    assert n > 1000
    assert not bad, "%d mismatches, first: %r" % (len(bad), bad[:2])


def test_fuzz_scorers_match_reference_fixtures():
    lib = _build("libhost_fuzz.so", [os.path.join(ROOT, "tests", "cpp", "host_fuzz.cpp"),
                                     os.path.join(CSRC, "rfg_token.cpp")])
    lib.hf_score.restype = ctypes.c_int
    lib.hf_score.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                             ctypes.c_double, ctypes.c_void_p]
    got = ctypes.c_double()
    n, bad = 0, []
    for fixture in ("partial.json", "tokens.json", "tokenset.json"):
        for c in G.load(fixture):
            if c["form"] == MULTI or c["w1"] != 1 or c["w2"] != 1:
                continue
            a, b = G.arrays(c)
            cutoff = 0.0 if c["cutoff"] is None else float(c["cutoff"])
            assert lib.hf_score(c["metric"], a.ctypes.data, a.size, b.ctypes.data, b.size, cutoff,
                                ctypes.byref(got)) == 0
            n += 1
            if not G.same(got.value, G.dec(c["expected"])):
                bad.append((fixture, c, got.value))
    assert n > 500
    assert not bad, "%d mismatches, first: %r" % (len(bad), bad[:2])
