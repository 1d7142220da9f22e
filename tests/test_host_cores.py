"""CPU tests of the scorer cores themselves: rfg_core.cuh (the templates the kernels
instantiate) compiled for the host behind tests/cpp/host_cores.cpp, against the oracle's
exact values on seeded pairs -- every core the kernels pick (one-word, W-word, banded,
runtime-W and several-queries recurrences on 64- and 32-bit words; the Jaro flagging
cores), patterns of 1..700 units, cutoffs from 0 to unbounded, with the distance chain
d <= K ? d : K + 1.  No GPU."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle_lib import ROOT, oracle

CSRC = os.path.join(ROOT, "rapidfuzz-cpp_gb300", "csrc")
BIG = 2**62


@pytest.fixture(scope="module")
def libs():
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libhost_cores.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-I" + CSRC, "-o", so,
                    os.path.join(ROOT, "tests", "cpp", "host_cores.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    lib.hc_distance.restype = I64
    lib.hc_distance.argtypes = [I, I, P, I, P, I, I64]
    lib.hc_group.restype = I
    lib.hc_group.argtypes = [I, I, P, I, P, I, P, I, I64, I64, P]
    lib.hc_band32.restype = I64
    lib.hc_band32.argtypes = [I, I, P, I, P, I, I64]
    lib.hc_hist_bound.restype = I
    lib.hc_hist_bound.argtypes = [I, P, I, P, I]
    lib.hc_band_range.restype = I
    lib.hc_band_range.argtypes = [I, I, ctypes.c_uint64, ctypes.c_double, I64, I64, P, P, P]
    lib.hc_band_reject.restype = None
    lib.hc_band_reject.argtypes = [I, I, ctypes.c_uint64, P, P]
    lib.hc_band_pair.restype = None
    lib.hc_band_pair.argtypes = [I, I, ctypes.c_uint64, ctypes.c_double, I64, I64, P, P, P, P]
    lib.hc_fast.restype = I
    lib.hc_fast.argtypes = [I, I, P, P, I, P, I, I, P]
    lib.hc_jaro.restype = I
    lib.hc_jaro.argtypes = [I, P, I, P, I, P, P]
    o = oracle()
    for f in (o.rfo_lcs_exact, o.rfo_osa_exact):
        f.restype = I64
        f.argtypes = [P, I64, I, P, I64, I]
    o.rfo_levenshtein_exact.restype = I64
    o.rfo_levenshtein_exact.argtypes = [P, I64, I, P, I64, I, I64, I64, I64]
    o.rfo_jaro_counts.restype = None
    o.rfo_jaro_counts.argtypes = [P, I64, I, P, I64, I, P, P]
    return lib, o


def pairs(seed, n, lens):
    """(a, b): b is a with edits (substitutions, insertions, deletions, adjacent swaps) or
    an unrelated string; alphabets of 2, 4 and 26 letters"""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        alpha = [b"ab", b"ACGT", b"abcdefghijklmnopqrstuvwxyz"][int(rng.integers(0, 3))]
        la = int(rng.choice(lens))
        a = bytearray(alpha[int(rng.integers(0, len(alpha)))] for _ in range(la))
        if rng.random() < 0.25:
            b = bytearray(alpha[int(rng.integers(0, len(alpha)))] for _ in range(int(rng.integers(0, la + 10))))
        else:
            b = bytearray(a)
            for _ in range(int(rng.integers(0, max(2, la // 6)))):
                k, pos = rng.random(), int(rng.integers(0, len(b) + 1))
                if k < 0.3 and pos < len(b):
                    b[pos] = alpha[int(rng.integers(0, len(alpha)))]
                elif k < 0.55:
                    b.insert(pos, alpha[int(rng.integers(0, len(alpha)))])
                elif k < 0.8 and pos < len(b):
                    del b[pos]
                elif pos + 1 < len(b):
                    b[pos], b[pos + 1] = b[pos + 1], b[pos]
        out.append((bytes(a), bytes(b)))
    return out


def exact(o, fam, a, b):
    if fam == 0:
        return o.rfo_levenshtein_exact(a, len(a), 1, b, len(b), 1, 1, 1, 1)
    if fam == 1:
        return len(a) + len(b) - 2 * o.rfo_lcs_exact(a, len(a), 1, b, len(b), 1)
    return o.rfo_osa_exact(a, len(a), 1, b, len(b), 1)


def cutoffs(rng, d):
    return sorted({0, 1, 3, 8, max(0, d - 1), d, d + 1, int(rng.integers(0, 2 * d + 2)), 31, 64, 200, BIG})


@pytest.mark.parametrize("fam", [0, 1, 2], ids=["levenshtein", "indel", "osa"])
def test_cores_match_oracle(libs, fam):
    lib, o = libs
    rng = np.random.default_rng(10 + fam)
    lens = [0, 1, 2, 5, 20, 31, 32, 33, 63, 64, 65, 100, 128, 129, 200, 256, 300, 512, 513, 700]
    for a, b in pairs(20 + fam, 900, lens):
        d = exact(o, fam, a, b)
        for K in cutoffs(rng, d):
            want = d if d <= K else K + 1
            for variant in (0, 1):
                got = lib.hc_distance(fam, variant, a, len(a), b, len(b), K)
                if got == -2:
                    continue
                assert got == want, (fam, variant, a, b, K)


@pytest.mark.parametrize("fam", [0, 1, 2], ids=["levenshtein", "indel", "osa"])
@pytest.mark.parametrize("word32", [0, 1], ids=["64bit", "32bit"])
def test_several_queries_core_matches_oracle(libs, fam, word32):
    lib, o = libs
    rng = np.random.default_rng(30 + fam + 3 * word32)
    lens = [0, 1, 2, 7, 8, 9, 16, 31, 32] + ([] if word32 else [33, 48, 63, 64])
    ps = pairs(40 + fam + 3 * word32, 1200, lens)
    out = (ctypes.c_int64 * 2)()
    for k in range(0, len(ps) - 1, 2):
        (a1, b), (a2, _) = ps[k], ps[k + 1]
        d1, d2 = exact(o, fam, a1, b), exact(o, fam, a2, b)
        for K1, K2 in zip(cutoffs(rng, d1), reversed(cutoffs(rng, d2))):
            assert lib.hc_group(fam, word32, a1, len(a1), a2, len(a2), b, len(b), K1, K2, out) == 0
            assert list(out) == [d1 if d1 <= K1 else K1 + 1, d2 if d2 <= K2 else K2 + 1], (a1, a2, b, K1, K2)


@pytest.mark.parametrize("fam", [0, 1, 2], ids=["levenshtein", "indel", "osa"])
@pytest.mark.parametrize("word32", [0, 1], ids=["64bit", "32bit"])
def test_warp_tile_core_matches_oracle(libs, fam, word32):
    """fast_group: one to four patterns per text, one cutoff, int bookkeeping"""
    lib, o = libs
    rng = np.random.default_rng(50 + fam + 3 * word32)
    lens = [0, 1, 2, 7, 8, 9, 15, 16, 17, 24, 31, 32] + ([] if word32 else [33, 40, 48, 63, 64])
    ps = pairs(60 + fam + 3 * word32, 2000, lens)
    out = (ctypes.c_int * 4)()
    for k in range(0, len(ps) - 3, 4):
        qn = int(rng.integers(1, 5))
        pats = [ps[k + j][0] for j in range(qn)]
        b = ps[k][1]
        off = np.zeros(5, dtype=np.int64)
        off[1:qn + 1] = np.cumsum([len(x) for x in pats])
        packed = b"".join(pats) or b"\0"
        ds = [exact(o, fam, x, b) for x in pats]
        for K in cutoffs(rng, ds[0]):
            K = min(K, 2**31 - 1)
            assert lib.hc_fast(fam, word32, packed, off.ctypes.data, qn, b, len(b), K, out) == 0
            assert list(out)[:qn] == [d if d <= K else K + 1 for d in ds], (pats, b, K)


@pytest.mark.parametrize("lcs", [0, 1], ids=["levenshtein", "indel"])
def test_band32_core_matches_oracle(libs, lcs):
    """lev_band32<B> / lcs_band32<B>: the 32-bit banded Levenshtein and LCS (as the Indel
    distance) of the band kernel on Ukkonen's band (about K + 2 diagonals), every window
    size, against the exact distance"""
    lib, o = libs
    rng = np.random.default_rng(77 + lcs)
    lens = [40, 63, 64, 65, 100, 127, 128, 129, 200, 300, 513, 700]
    checked = 0
    for a, b in pairs(78 + lcs, 700, lens):
        d = exact(o, lcs, a, b)
        for B in ((1, 2, 3, 4, 8, 16) if lcs else (1, 2, 4, 8, 16)):
            for K in sorted({int(rng.integers(0, 32 * B)), 32 * B - 2, 32 * B - 1, max(0, d - 1), d, d + 1,
                             abs(len(a) - len(b))}):
                got = lib.hc_band32(lcs, B, a, len(a), b, len(b), K)
                if got == -2:
                    continue
                # the core gives d, or any value above K once d > K (the chain maps it to K + 1)
                assert (got == d) if d <= K else (got > K), (B, K, len(a), len(b), got, d)
                checked += 1
    assert checked > 2000


def test_count_filter_bound_never_exceeds_distance(libs):
    """the warp tiles' count filter skips a pair only when its bound exceeds the cutoff:
    the bound (hist_lower_bound) is at most the exact Levenshtein, OSA and Indel distance
    on every pair (so a skipped pair's distance exceeds K and its chain value is K + 1),
    and it is tight for anagrams-free cases such as pure insertions"""
    lib, o = libs
    checked = 0
    tight = 0
    for a, b in pairs(81, 3000, [0, 1, 2, 5, 16, 31, 32, 33, 63, 64, 100, 200, 255]):
        if len(a) > 255 or len(b) > 255:
            continue
        for fam, exact_fam in ((0, 0), (0, 2), (1, 1)):
            lb = lib.hc_hist_bound(fam, a, len(a), b, len(b))
            d = exact(o, exact_fam, a, b)
            assert 0 <= lb <= d, (fam, exact_fam, a, b, lb, d)
            tight += lb == d
            checked += 1
    assert checked > 5000 and tight > 100


# metric ids of the scorer enum (rfg_core.cuh)
LEV_M, INDEL_M, LCSSEQ_M, RATIO_M = 0, 1, 2, 6


@pytest.mark.parametrize("metric", [LEV_M, INDEL_M, LCSSEQ_M, RATIO_M], ids=["levenshtein", "indel", "lcsseq", "ratio"])
def test_band_ranges_and_rejected_values(libs, metric):
    """the band launches' split of a query's pairs: every choice length that passes the
    length filter lies in band_range's [nlo, nhi] (so a query's passing pairs are one
    run of the length-sorted choices; for unit-weight Levenshtein, whose bound is one
    value for n <= m, the interval is exactly the passing lengths), Kmax bounds every
    passing pair's K, and every pair outside the interval gets band_reject_value, for all
    four ops (ratio: its one chain) and cutoffs across their range (checked against the
    per-pair plan at every length up to maxlen)"""
    lib, _ = libs
    rng = np.random.default_rng(91 + metric)
    D, S, ND, NS = 0, 1, 2, 3
    lo, hi, km = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    ps, vi, vf, kk = ctypes.c_int(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64()
    rvi, rvf = ctypes.c_int64(), ctypes.c_double()
    cases = 0
    for _ in range(400):
        op = NS if metric == RATIO_M else int(rng.integers(0, 4))
        m = int(rng.choice([1, 2, 65, 100, 257, 300, 1000, 2000]))
        maxlen = int(rng.choice([0, 1, m // 2, m, m + 5, 2 * m, 3000]))
        if metric == RATIO_M:
            cf = float(rng.choice([0.0, 1.0, 50.0, 80.0, 85.0, 90.0, 95.0 + 1e-9, 99.0, 100.0]))
            ci = 0
        elif op in (ND, NS):
            cf = float(rng.choice([0.0, 0.01, 0.05, 0.1, 0.1 + 1e-9, 0.18, 0.3, 0.5, 0.9, 0.99, 1.0]))
            ci = 0
        else:
            ci = int(rng.choice([0, 1, 5, 30, m // 2, m, m + 3, 2 * m - 1, 2**40]))
            cf = 0.0
        ok = lib.hc_band_range(metric, op, ci, cf, m, maxlen, ctypes.byref(lo), ctypes.byref(hi), ctypes.byref(km))
        lib.hc_band_reject(metric, op, ci, ctypes.byref(rvi), ctypes.byref(rvf))
        # the band classes take patterns whose band (Kmax + 2 bits) is narrower than m
        band = ok and km.value + 2 < m
        passing = []
        for n in range(0, max(m, maxlen) + 1):
            lib.hc_band_pair(metric, op, ci, cf, m, n, ctypes.byref(ps), ctypes.byref(vi), ctypes.byref(vf),
                             ctypes.byref(kk))
            if ps.value:
                passing.append(n)
                if ok:
                    assert kk.value <= km.value, (metric, op, ci, cf, m, n, kk.value, km.value)
            elif not band or (lo.value <= n <= hi.value):
                continue
            elif metric == RATIO_M or op in (ND, NS):
                assert vf.value == rvf.value, (metric, op, cf, m, n, vf.value, rvf.value)
            else:
                assert vi.value == rvi.value, (metric, op, ci, m, n, vi.value, rvi.value)
        if not ok:
            assert not passing, (metric, op, ci, cf, m, maxlen)
            continue
        assert all(lo.value <= n <= hi.value for n in passing), (metric, op, ci, cf, m, maxlen, lo.value, hi.value)
        if metric == LEV_M:
            expect = [n for n in range(0, max(m, maxlen) + 1) if lo.value <= n <= hi.value]
            assert passing == expect, (op, ci, cf, m, maxlen, lo.value, hi.value)
        else:
            assert passing and passing[-1] == hi.value, (metric, op, ci, cf, m, maxlen, hi.value)
        cases += band
    assert cases > 60


def test_jaro_cores_match_oracle(libs):
    lib, o = libs
    c, t, ec, et = (ctypes.c_int64() for _ in range(4))
    lens = [1, 2, 3, 5, 10, 20, 40, 63, 64, 65, 100, 200, 300]
    seen = set()
    for a, b in pairs(50, 1500, lens):
        if not a or not b:
            continue
        o.rfo_jaro_counts(a, len(a), 1, b, len(b), 1, ctypes.byref(ec), ctypes.byref(et))
        for variant in (0, 1, 2, 3):
            rc = lib.hc_jaro(variant, a, len(a), b, len(b), ctypes.byref(c), ctypes.byref(t))
            if rc == -2:
                continue
            assert rc == 0 and (c.value, t.value) == (ec.value, et.value), (variant, a, b)
            seen.add(variant)
    assert seen == {0, 1, 2, 3}
