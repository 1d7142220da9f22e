"""CPU tests of the library's host-side token front end (rapidfuzz-cpp_gb300/csrc/rfg_token.cpp):
the sorted-split joins (common_impl.hpp:162-180, SplittedSentenceView.hpp:71-85), the
deduplicated joins (SplittedSentenceView.hpp:48-54) and the [string][S][J] part layout the
token_set_ratio family uploads, against the oracle's restatement (rfo_token_join), for every
code-unit width, with the one-byte (ASCII) and wide (Unicode) whitespace sets.  No GPU."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle_lib import ROOT, oracle

CSRC = os.path.join(ROOT, "rapidfuzz-cpp_gb300", "csrc")
DT = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}
# whitespace of both sets, and units that are whitespace only for wide strings
WS_ASCII = [0x09, 0x0A, 0x0B, 0x0C, 0x0D, 0x1C, 0x1D, 0x1E, 0x1F, 0x20]
WS_WIDE = [0x85, 0xA0, 0x1680, 0x2000, 0x2005, 0x200A, 0x2028, 0x2029, 0x202F, 0x205F, 0x3000]


@pytest.fixture(scope="module")
def host():
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libhost_tokens.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-pthread", "-I" + CSRC, "-o", so,
                    os.path.join(ROOT, "tests", "cpp", "host_tokens.cpp"), os.path.join(CSRC, "rfg_token.cpp")],
                   check=True)
    lib = ctypes.CDLL(so)
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    lib.ht_parts.restype = I64
    lib.ht_parts.argtypes = [P, P, I64, I, I, I, I, P, I64, P, P]
    lib.ht_join_set.restype = I64
    lib.ht_join_set.argtypes = [P, P, I64, I, P, I64, P]
    lib.ht_join_one.restype = I64
    lib.ht_join_one.argtypes = [P, I64, I, P, I64]
    o = oracle()
    o.rfo_token_join.restype = I
    o.rfo_token_join.argtypes = [P, I64, I, I, P, I64, ctypes.POINTER(I64)]
    return lib, o


def oracle_join(o, s, width, dedup):
    out = np.zeros(max(len(s), 1), dtype=np.uint64)
    n = ctypes.c_int64()
    assert o.rfo_token_join(s.ctypes.data, len(s), width, dedup, out.ctypes.data, out.size, ctypes.byref(n)) == 0
    return out[:n.value]


def strings(rng, width, n):
    """token strings over a few letters, with runs of mixed whitespace, repeats and empties"""
    letters = [0x61, 0x62, 0x63, 0x41]
    if width > 1:
        letters += [0xE9, 0x3B1, 0x4E00]
    if width >= 4:
        letters += [0x1F600]
    if width == 8:
        letters += [2**63 + 5]
    ws = WS_ASCII + ([u & 0xFF for u in WS_WIDE[:2]] if width == 1 else WS_WIDE)
    vocab = [np.array([letters[k] for k in rng.integers(0, len(letters), int(rng.integers(1, 5)))], dtype=np.uint64)
             for _ in range(6)]
    out = []
    for _ in range(n):
        parts = []
        for _ in range(int(rng.integers(0, 7))):
            if rng.random() < 0.5:
                parts.append(np.array(ws, dtype=np.uint64)[rng.integers(0, len(ws), int(rng.integers(1, 3)))])
            parts.append(vocab[int(rng.integers(0, len(vocab)))])
        s = np.concatenate(parts) if parts else np.zeros(0, dtype=np.uint64)
        out.append(s.astype(DT[width]))
    return out


def pack(ss, width):
    off = np.zeros(len(ss) + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(s) for s in ss])
    data = np.concatenate(ss).astype(DT[width]) if ss else np.zeros(0, DT[width])
    return np.ascontiguousarray(data), off


@pytest.mark.parametrize("width", [1, 2, 4, 8])
def test_token_joins_match_oracle(host, width):
    lib, o = host
    rng = np.random.default_rng(100 + width)
    ss = strings(rng, width, 3000)
    data, off = pack(ss, width)
    # one string at a time
    for s in ss[:300]:
        buf = np.zeros(max(len(s), 1), dtype=DT[width])
        n = lib.ht_join_one(s.ctypes.data, len(s), width, buf.ctypes.data, buf.nbytes)
        assert np.array_equal(buf[:n].astype(np.uint64), oracle_join(o, s, width, 0))
    # the packed set (over the host threads)
    buf = np.zeros(max(len(data), 1), dtype=DT[width])
    oo = np.zeros(len(ss) + 1, dtype=np.int64)
    nb = lib.ht_join_set(data.ctypes.data, off.ctypes.data, len(ss), width, buf.ctypes.data, buf.nbytes,
                         oo.ctypes.data)
    assert nb == oo[-1] * width
    for i, s in enumerate(ss):
        assert np.array_equal(buf[oo[i]:oo[i + 1]].astype(np.uint64), oracle_join(o, s, width, 0)), i


@pytest.mark.parametrize("width", [1, 2, 4, 8])
@pytest.mark.parametrize("orig,sorted_,dedup", [(1, 1, 1), (0, 1, 0), (1, 0, 0), (0, 0, 1), (1, 0, 1)])
def test_token_parts_layout(host, width, orig, sorted_, dedup):
    lib, o = host
    rng = np.random.default_rng(200 + width)
    ss = strings(rng, width, 2000)
    data, off = pack(ss, width)
    buf = np.zeros(max(3 * len(data), 1), dtype=DT[width])
    oo = np.zeros(len(ss) + 1, dtype=np.int64)
    parts = np.zeros(max(3 * len(ss), 1), dtype=np.int32)
    nb = lib.ht_parts(data.ctypes.data, off.ctypes.data, len(ss), width, orig, sorted_, dedup, buf.ctypes.data,
                      buf.nbytes, oo.ctypes.data, parts.ctypes.data)
    assert nb == oo[-1] * width
    for i, s in enumerate(ss):
        exp_o = s.astype(np.uint64) if orig else np.zeros(0, np.uint64)
        exp_s = oracle_join(o, s, width, 0) if sorted_ else np.zeros(0, np.uint64)
        exp_j = oracle_join(o, s, width, 1) if dedup else np.zeros(0, np.uint64)
        assert list(parts[3 * i:3 * i + 3]) == [len(exp_o), len(exp_s), len(exp_j)], i
        got = buf[oo[i]:oo[i + 1]].astype(np.uint64)
        assert np.array_equal(got, np.concatenate([exp_o, exp_s, exp_j])), i
