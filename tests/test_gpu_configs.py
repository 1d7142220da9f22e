"""Parity on the benchmark configurations' input shapes (seeded synthetic stand-ins):
the CUDA path against the oracle bit-exactly at sizes the oracle finishes in seconds,
and size-independent properties at the full sizes."""
import numpy as np
import pytest

from oracle_lib import oracle_cdist

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402
import workloads as WL  # noqa: E402


def _same(a, b):
    if a.dtype == np.float64:
        return np.array_equal(a.view(np.int64), b.view(np.int64))
    return np.array_equal(a, b)


def _rows(batch, idx):
    d, o, w = batch
    parts = [d[o[i]:o[i + 1]] for i in idx]
    off = np.zeros(len(idx) + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(p) for p in parts])
    return (np.concatenate(parts) if parts else d[:1], off, w)


def test_config1_shape_one_query_many_dna():
    """1 query x DNA choices len U[8,64], Levenshtein without cutoff, int64"""
    c = WL.dna_uniform(seed=1, n=100000)
    q = WL.dna_uniform(seed=2, n=1)
    got = R.cdist(R.LEVENSHTEIN, R.DISTANCE, q, c)
    sub = np.arange(0, 100000, 7)
    exp = oracle_cdist(R.LEVENSHTEIN, R.DISTANCE, q, _rows(c, sub))
    assert _same(got[:, sub], exp)
    # the Cached scorer over all choices is the same launch family
    qs = q[0][:q[1][1]]
    many = R.Cached(R.LEVENSHTEIN, qs).score_many(R.DISTANCE, c)
    assert np.array_equal(many, got[0])


def test_config2_shape_full_size():
    """4096 x 4096 a-z Zipf(1.1), Lev/Indel/OSA cutoff 8, int32: sampled rows exact,
    symmetry of the full matrices"""
    q, c = WL.cdist_zipf(seed=3)
    rows = [0, 1, 777, 2048, 4095]
    for m in (R.LEVENSHTEIN, R.INDEL, R.OSA):
        got = R.cdist(m, R.DISTANCE, q, c, 8, out_dtype=R.I32)
        exp = oracle_cdist(m, R.DISTANCE, _rows(q, rows), c, 8, out_dtype=0)
        assert _same(got[rows], exp)
        back = R.cdist(m, R.DISTANCE, c, q, 8, out_dtype=R.I32)
        assert np.array_equal(got, back.T)  # these three metrics are symmetric
    d = R.cdist(R.LEVENSHTEIN, R.DISTANCE, q, q, 8, out_dtype=R.I32)
    assert (np.diag(d) == 0).all()


def test_config3_shape_long_banded():
    """DNA lognormal(300, 0.6) in [100, 2000], mutated and unrelated choices; Levenshtein
    with the cutoff at 10 % of the longer string (normalized_distance <= 0.1)"""
    q, c = WL.dna_lognormal(seed=4, nq=24, nc=1500)
    for op, cut in ((R.NORMALIZED_DISTANCE, 0.1), (R.DISTANCE, 60), (R.DISTANCE, 200), (R.DISTANCE, None)):
        got = R.cdist(R.LEVENSHTEIN, op, q, c, cut)
        exp = oracle_cdist(R.LEVENSHTEIN, op, q, c, cut)
        assert _same(got, exp), (op, cut)


def test_config4_shape_tokens_u32():
    """uint32 token strings (26 Latin + 14 accented code points), Jaro-Winkler 0.85 and
    fuzz::ratio 85 as float64"""
    (q, ql) = WL.tokens_u32(seed=5, n=64)
    (c, _) = WL.tokens_u32(seed=6, n=20000, derive_from=ql, derive_frac=0.2)
    for m, cut in ((R.JARO_WINKLER, 0.85), (R.RATIO, 85.0), (R.JARO, 0.7)):
        got = R.cdist(m, R.SIMILARITY, q, c, cut)
        exp = oracle_cdist(m, R.SIMILARITY, q, c, cut)
        assert _same(got, exp), m
    assert (got >= 0).all()


def test_host_output_row_blocks_match_oracle():
    """Host results larger than 32 MB leave in row blocks copied while the next block
    computes; rows on both sides of every block boundary must equal the oracle"""
    q, c = WL.cdist_zipf(seed=9, nq=4096, nc=2200)
    got = R.cdist(R.LEVENSHTEIN, R.DISTANCE, q, c, 8, out_dtype=R.I32)          # 36 MB: 2 blocks
    rows = [0, 1, 2047, 2048, 2049, 4095]
    exp = oracle_cdist(R.LEVENSHTEIN, R.DISTANCE, _rows(q, rows), c, 8, out_dtype=0)
    assert _same(got[rows], exp)
    got = R.cdist(R.INDEL, R.NORMALIZED_SIMILARITY, q, c, 0.7)                    # 72 MB float64: 4 blocks
    rows = [0, 1023, 1024, 2047, 2048, 3071, 3072, 4095]
    exp = oracle_cdist(R.INDEL, R.NORMALIZED_SIMILARITY, _rows(q, rows), c, 0.7)
    assert _same(got[rows], exp)
    dev = R.cdist(R.INDEL, R.NORMALIZED_SIMILARITY, _rows(q, rows), c, 0.7)
    assert _same(dev, exp)
