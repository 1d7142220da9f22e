"""The CPU oracle, pinned: bit-exact against fixtures the reference itself produced,
against the naive dynamic programs, and (where it was built here) against the live
reference.  CPU only."""
import ctypes
import random

import numpy as np
import pytest

import golden_lib as G
from oracle_lib import (CACHED, FREE, MULTI, LEVENSHTEIN, LCSSEQ, OSA, DISTANCE, SIMILARITY, NORM_DISTANCE,
                        NORM_SIMILARITY, JARO, JARO_WINKLER, RATIO, INDEL, as_units, oracle, reference, score,
                        result_is_int, oracle_cdist, pack_strings)


@pytest.mark.parametrize("fixture", ["kat.json", "random.json", "partial.json", "tokens.json", "tokenset.json"])
def test_oracle_matches_reference_fixtures(fixture):
    o = oracle()
    bad = []
    for c in G.load(fixture):
        a, b = G.arrays(c)
        v = score(o.rfo_score, c["metric"], c["op"], c["form"], a, b, c["cutoff"], tuple(c["weights"]), c["pw"])
        if not G.same(v, G.dec(c["expected"])):
            bad.append((c, v))
    assert not bad, "%d mismatches, first: %r" % (len(bad), bad[:2])


def _eo_arrays(c):
    dt = {1: np.uint8, 2: np.uint16, 4: np.uint32}[c["w"]]
    return np.array(c["s1"], dtype=dt), np.array(c["s2"], dtype=dt)


def test_oracle_editops_fixture():
    """editops of the DP-table restatement equal the reference's (editops.json)"""
    from oracle_lib import editops
    o = oracle()
    for c in G.load("editops.json"):
        a, b = _eo_arrays(c)
        got = editops(o.rfo_editops, c["metric"], a, b, c["hint"])
        assert got == [tuple(x) for x in c["expected"]], (c.get("cite"), c["metric"], len(a), len(b))


def test_oracle_multi_batches():
    """each element of a Multi* batch equals the single-pattern Multi chain"""
    o = oracle()
    for c in G.load("multi.json"):
        for s, exp in zip(c["strs"], c["expected"]):
            v = score(o.rfo_score, c["metric"], c["op"], MULTI, bytes(s), bytes(c["s2"]), c["cutoff"],
                      tuple(c["weights"]), c["pw"])
            assert G.same(v, G.dec(exp)), (c.get("cite"), c["metric"], c["op"], s, v, exp)


def test_reference_known_answers_literal():
    """literal values asserted by the reference's tests"""
    o = oracle()
    lev = lambda a, b, w=(1, 1, 1), c=None: score(o.rfo_score, LEVENSHTEIN, DISTANCE, FREE, a, b, c, w)
    assert lev("aaaa", "aaa") == 1 and lev("abaa", "baaa") == 2 and lev("aaaa", "bbbb") == 4
    assert lev("aaaa", "bbbb", (1, 1, 2)) == 8  # tests-Levenshtein.cpp:129
    assert lev("South Korea", "North Korea", (1, 1, 1), 0) == 1  # :153
    assert lev("aabc", "cccd", (1, 1, 2), 4) == 5  # :173
    assert score(o.rfo_score, OSA, DISTANCE, FREE, "CA", "AC") == 1  # tests-OSA.cpp:84
    assert score(o.rfo_score, OSA, DISTANCE, FREE, "aaaa", "", 1) == 2  # tests-OSA.cpp:73
    assert score(o.rfo_score, INDEL, DISTANCE, FREE, "South Korea", "North Korea") == 4  # tests-Indel.cpp:226
    assert score(o.rfo_score, LCSSEQ, SIMILARITY, FREE, "South Korea", "North Korea", 10) == 0  # tests-LCSseq.cpp:172
    assert abs(score(o.rfo_score, JARO, SIMILARITY, FREE, "0", "00") - 0.833333) < 1e-6  # tests-Jaro.cpp:178
    assert abs(score(o.rfo_score, JARO_WINKLER, SIMILARITY, FREE, "0", "00") - 0.85) < 1e-6  # tests-JaroWinkler.cpp:183
    assert abs(score(o.rfo_score, RATIO, SIMILARITY, FREE, "new york mets", "the wonderful new york mets") - 65) < 1


def _rand(rng, alpha, n):
    return [rng.choice(alpha) for _ in range(n)]


def test_bit_parallel_equals_dynamic_programs():
    o = oracle()
    rng = random.Random(11)
    for _ in range(1500):
        alpha = rng.choice([[1, 2], [65, 67, 71, 84], list(range(97, 123)), [300, 301, 70000]])
        a = as_units(_rand(rng, alpha, rng.randint(0, 150)), 4)
        b = as_units(_rand(rng, alpha, rng.randint(0, 150)), 4)
        w = rng.choice([(1, 1, 1), (1, 1, 2), (2, 3, 4), (3, 1, 2)])
        args = (a.ctypes.data, a.size, 4, b.ctypes.data, b.size, 4)
        assert o.rfo_levenshtein_exact(*args, *w) == o.rfo_dp_levenshtein(*args, *w)
        assert o.rfo_lcs_exact(*args) == o.rfo_dp_lcs(*args)
        assert o.rfo_osa_exact(*args) == o.rfo_dp_osa(*args)
        c1, t1, c2, t2 = (ctypes.c_int64() for _ in range(4))
        o.rfo_jaro_counts(*args, ctypes.byref(c1), ctypes.byref(t1))
        o.rfo_naive_jaro_counts(*args, ctypes.byref(c2), ctypes.byref(t2))
        assert (c1.value, t1.value) == (c2.value, t2.value)


def test_oracle_cdist_equals_single_calls():
    o = oracle()
    rng = random.Random(5)
    qs = [bytes(_rand(rng, b"acgt", rng.randint(0, 80))) for _ in range(7)]
    cs = [bytes(_rand(rng, b"acgt", rng.randint(0, 80))) for _ in range(9)]
    for metric, op, cut in ((LEVENSHTEIN, DISTANCE, 5), (INDEL, NORM_SIMILARITY, 0.5), (OSA, SIMILARITY, 3),
                            (JARO_WINKLER, SIMILARITY, 0.8), (RATIO, SIMILARITY, 60.0), (LCSSEQ, DISTANCE, None)):
        m = oracle_cdist(metric, op, pack_strings(qs, 1), pack_strings(cs, 1), cut, nthreads=3)
        for i, q in enumerate(qs):
            for j, c in enumerate(cs):
                assert G.same(m[i, j].item(), score(o.rfo_score, metric, op, CACHED, q, c, cut))


@pytest.mark.skipif(reference() is None, reason="reference not built here (oracle/_ref)")
def test_oracle_vs_live_reference():
    o, r = oracle(), reference()
    rng = random.Random(99)
    for _ in range(3000):
        alpha = rng.choice([[65, 67, 71, 84], list(range(97, 123)), [97, 300, 70000]])
        a = as_units(_rand(rng, alpha, rng.randint(0, 140)), 4)
        b = as_units(_rand(rng, alpha, rng.randint(0, 140)), 4)
        metric = rng.randrange(7)
        op = SIMILARITY if metric == RATIO else rng.randrange(4)
        form = rng.choice([FREE, CACHED] + ([MULTI] if a.size <= 64 else []))
        cut = (rng.choice([None, 0, 3, 8, 40]) if result_is_int(metric, op)
               else rng.choice([None, 0.0, 0.7, 0.85, 1.0]))
        if metric == RATIO and cut is not None:
            cut *= 100
        assert G.same(score(o.rfo_score, metric, op, form, a, b, cut), score(r.rfref_score, metric, op, form, a, b, cut))
