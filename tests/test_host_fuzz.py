"""CPU tests of the device path's fuzz scorers: partial_ratio_dev and token_family_dev
(rfg_core.cuh, the templates the partial / token kernels instantiate) compiled for the
host behind tests/cpp/host_fuzz.cpp, with the library's host token front end making the
part concatenations, against the oracle's free-function scores, bit for bit, on seeded
token strings (repeated, shared and disjoint tokens, lengths up to a few hundred units)
and cutoffs from 0 to above 100.  No GPU."""
import ctypes
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from oracle_lib import ROOT, Params, oracle, PARTIAL_RATIO, TOKEN_SORT_RATIO, WRATIO, SIMILARITY, FREE

CSRC = os.path.join(ROOT, "rapidfuzz-cpp_gb300", "csrc")
NAMES = {7: "partial_ratio", 8: "token_sort_ratio", 9: "partial_token_sort_ratio", 10: "QRatio",
         11: "token_set_ratio", 12: "partial_token_set_ratio", 13: "token_ratio", 14: "partial_token_ratio",
         15: "WRatio"}


@pytest.fixture(scope="module")
def libs():
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libhost_fuzz.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-pthread", "-ffp-contract=off", "-I" + CSRC,
                    "-o", so, os.path.join(ROOT, "tests", "cpp", "host_fuzz.cpp"), os.path.join(CSRC, "rfg_token.cpp")],
                   check=True)
    lib = ctypes.CDLL(so)
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    lib.hf_score.restype = I
    lib.hf_score.argtypes = [I, P, I64, P, I64, ctypes.c_double, P]
    o = oracle()
    o.rfo_score.restype = I
    o.rfo_score.argtypes = [I, I, I, P, I64, I, P, I64, I, ctypes.POINTER(Params), ctypes.c_uint64, ctypes.c_double,
                            ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)]
    return lib, o


def token_pairs(seed, n):
    rng = np.random.default_rng(seed)
    words = [bytes(rng.choice(list(b"abcdefgh"), int(rng.integers(1, 9)))) for _ in range(12)]
    out = []
    for _ in range(n):
        def sentence(k):
            ws = [words[int(rng.integers(0, len(words)))] for _ in range(k)]
            seps = [b" " * int(rng.integers(1, 3)) if rng.random() < 0.9 else b"\t" for _ in ws]
            return b"".join(w + s for w, s in zip(ws, seps)).strip(b" ") if ws else b""
        a = sentence(int(rng.integers(0, 6)))
        r = rng.random()
        if r < 0.3:
            b = sentence(int(rng.integers(0, 30)))          # long against short: partial branches
        elif r < 0.6:
            toks = a.split()
            rng.shuffle(toks)
            b = b" ".join(toks + [words[int(rng.integers(0, len(words)))]] * int(rng.integers(0, 3)))
        else:
            b = sentence(int(rng.integers(0, 6)))
        out.append((a, b) if rng.random() < 0.5 else (b, a))
    return out


def bits(x):
    return struct.pack("<d", x)


@pytest.mark.parametrize("metric", list(range(PARTIAL_RATIO, WRATIO + 1)), ids=lambda m: NAMES[m])
def test_fuzz_scorers_match_oracle(libs, metric):
    lib, o = libs
    p = Params(1, 1, 1, 0.1)
    got, want, oi = ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
    n = 0
    for a, b in token_pairs(60 + metric, 700):
        for cutoff in (0.0, 50.0, 80.0, 95.0, 100.0, 100.5):
            assert lib.hf_score(metric, a, len(a), b, len(b), cutoff, ctypes.byref(got)) == 0
            assert o.rfo_score(metric, SIMILARITY, FREE, a, len(a), 1, b, len(b), 1, ctypes.byref(p), 0, cutoff,
                               ctypes.byref(oi), ctypes.byref(want)) == 0
            assert bits(got.value) == bits(want.value), (NAMES[metric], a, b, cutoff, got.value, want.value)
            n += 1
    assert n == 700 * 6
