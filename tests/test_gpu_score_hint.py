"""The score-hint doubling of uniform_levenshtein_distance (Levenshtein_impl.hpp:876-897)
in the one-pair path: Levenshtein pairs of 65 to 3,000 units scored through the free
functions and the Cached scorer with hints below, at and above the distance (0, 1, half,
d - 1, d, d + 1, twice, none) under every op; the results never depend on the hint, so
each is compared with the oracle's hint-free value."""
import numpy as np
import pytest

from oracle_lib import oracle_cdist

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402


def _pairs(rng, n):
    out = []
    alpha = np.frombuffer(b"ACGT", dtype=np.uint8)
    for _ in range(n):
        m = int(rng.choice([65, 100, 300, 700, 1500, 3000]))
        a = alpha[rng.integers(0, 4, size=m)]
        b = a.copy()
        k = int(rng.integers(0, max(2, m // 5)))
        for _ in range(k):
            p = int(rng.integers(0, len(b)))
            r = rng.random()
            if r < 0.4:
                b[p] = alpha[int(rng.integers(0, 4))]
            elif r < 0.7:
                b = np.insert(b, p, alpha[int(rng.integers(0, 4))])
            elif len(b) > 1:
                b = np.delete(b, p)
        if rng.random() < 0.2:
            b = alpha[rng.integers(0, 4, size=int(rng.integers(1, m + 40)))]
        out.append((a.tobytes(), b.tobytes()))
    return out


def _oracle(op, a, b, cut):
    q = R.pack_strings([a], 1)
    c = R.pack_strings([b], 1)
    return oracle_cdist(R.LEVENSHTEIN, op, q, c, cut)[0, 0]


def test_score_hint_never_changes_results():
    rng = np.random.default_rng(611)
    checked = 0
    for a, b in _pairs(rng, 40):
        d = int(_oracle(R.DISTANCE, a, b, None))
        cached = R.Cached(R.LEVENSHTEIN, a)
        for cut in (None, d, d + 5, 2 * d + 10):
            exp = int(_oracle(R.DISTANCE, a, b, cut))
            for hint in (0, 1, d // 2, max(0, d - 1), d, d + 1, 2 * d + 3, None):
                got = R.score(R.LEVENSHTEIN, R.DISTANCE, a, b, cut, hint)
                assert got == exp, (len(a), len(b), d, cut, hint, got, exp)
                assert cached.score(R.DISTANCE, b, cut, hint) == exp
                checked += 2
        M = max(len(a), len(b))
        for op, cut, hints in ((R.SIMILARITY, max(0, M - d), (0, M, M - d, M - d // 2)),
                               (R.NORMALIZED_DISTANCE, 0.3, (0.0, 0.01, 0.1, 0.5, 1.0)),
                               (R.NORMALIZED_SIMILARITY, 0.6, (0.0, 0.5, 0.9, 0.99, 1.0))):
            exp = _oracle(op, a, b, cut)
            for hint in hints:
                got = R.score(R.LEVENSHTEIN, op, a, b, cut, hint)
                if isinstance(exp, (float, np.floating)):
                    assert np.float64(got).view(np.int64) == np.float64(exp).view(np.int64), (op, cut, hint)
                else:
                    assert got == exp, (op, cut, hint, got, exp)
                checked += 1
    assert checked > 1000
