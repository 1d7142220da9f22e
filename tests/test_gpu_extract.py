"""extract / extractOne over a device-resident corpus against the reference's loops
(README.md:153-214) on oracle scores: same choices, same scores (bit-identical doubles),
same order and tie rules."""
import random

import numpy as np
import pytest

from extract_lib import oracle_extract

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402


def _strings(rng, n, alpha, lo, hi, base=None):
    out = []
    for _ in range(n):
        if base and rng.random() < 0.3:
            s = list(rng.choice(base))
            for _ in range(rng.randint(0, 5)):
                if s and rng.random() < 0.5:
                    s[rng.randrange(len(s))] = rng.choice(alpha)
                else:
                    s.insert(rng.randint(0, len(s)), rng.choice(alpha))
            out.append(s)
        else:
            out.append([rng.choice(alpha) for _ in range(rng.randint(lo, hi))])
    return out


CASES = [(R.LEVENSHTEIN, R.DISTANCE, None), (R.LEVENSHTEIN, R.DISTANCE, 12), (R.INDEL, R.NORMALIZED_SIMILARITY, 0.6),
         (R.OSA, R.SIMILARITY, 5), (R.LCSSEQ, R.SIMILARITY, None), (R.JARO_WINKLER, R.SIMILARITY, 0.0),
         (R.JARO_WINKLER, R.SIMILARITY, 0.85), (R.RATIO, R.SIMILARITY, 50.0), (R.JARO, R.NORMALIZED_DISTANCE, 0.3),
         (R.PARTIAL_RATIO, R.SIMILARITY, 60.0)]


@pytest.mark.parametrize("metric,op,cut", CASES)
@pytest.mark.parametrize("limit,tie_last", [(1, True), (1, False), (10, False), (32, True)])
def test_extract_matches_reference_loop(metric, op, cut, limit, tie_last):
    rng = random.Random(hash((metric, op, limit)) & 0xffff)
    alpha = [97, 98, 99, 100]
    qs = _strings(rng, 9, alpha, 1, 90) + [[97] * 600, []]
    cs = _strings(rng, 9000, alpha, 0, 120, base=qs) + [[98] * 700]
    q = R.pack_strings([np.array(x, dtype=np.uint8) for x in qs], 1)
    c = R.pack_strings([np.array(x, dtype=np.uint8) for x in cs], 1)
    corpus = R.Corpus(c)
    idx, sc, cnt = corpus.extract(metric, op, q, limit, cut, tie_last)
    exp = oracle_extract(metric, op, q, c, limit, cut, tie_last)
    for i, (ei, es) in enumerate(exp):
        assert cnt[i] == len(ei), (i, cnt[i], len(ei))
        assert np.array_equal(idx[i, :cnt[i]], ei), (i, idx[i, :cnt[i]], ei)
        assert np.array_equal(sc[i, :cnt[i]].view(np.int64), es.view(np.int64))


TOKEN_CASES = [(R.WRATIO, 0.0), (R.WRATIO, 70.0), (R.TOKEN_SET_RATIO, 50.0), (R.TOKEN_SORT_RATIO, 60.0),
               (R.PARTIAL_TOKEN_SORT_RATIO, 0.0), (R.QRATIO, 0.0), (R.TOKEN_RATIO, 80.0),
               (R.PARTIAL_TOKEN_SET_RATIO, 0.0), (R.PARTIAL_TOKEN_RATIO, 90.0)]


@pytest.mark.parametrize("metric,cut", TOKEN_CASES)
@pytest.mark.parametrize("limit,tie_last", [(1, True), (5, False)])
def test_extract_token_scorers(metric, cut, limit, tie_last):
    """extract / extractOne with the token scorers (WRatio is rapidfuzz's default scorer):
    the corpus's token twin, the FAM_TOKEN extract kernel"""
    rng = random.Random(hash((metric, limit)) & 0xffff)
    vocab = [[rng.choice([97, 98, 99, 100]) for _ in range(rng.randint(1, 5))] for _ in range(12)]

    def mk(k):
        s = []
        for _ in range(k):
            s += list(rng.choice(vocab))
            s += [32] * rng.randint(1, 2)
        return s
    qs = [mk(rng.randint(1, 5)) for _ in range(7)] + [[], [32]]
    cs = [mk(rng.randint(0, 8)) for _ in range(3000)] + [[]]
    q = R.pack_strings([np.array(x, dtype=np.uint8) for x in qs], 1)
    c = R.pack_strings([np.array(x, dtype=np.uint8) for x in cs], 1)
    corpus = R.Corpus(c)
    idx, sc, cnt = corpus.extract(metric, R.SIMILARITY, q, limit, cut, tie_last)
    exp = oracle_extract(metric, R.SIMILARITY, q, c, limit, cut, tie_last)
    for i, (ei, es) in enumerate(exp):
        assert cnt[i] == len(ei), (i, cnt[i], len(ei))
        assert np.array_equal(idx[i, :cnt[i]], ei), (i, idx[i, :cnt[i]], ei)
        assert np.array_equal(sc[i, :cnt[i]].view(np.int64), es.view(np.int64))
