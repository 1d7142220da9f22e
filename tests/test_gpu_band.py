"""The band classes of unit-weight Levenshtein (k_band): queries whose every passing pair
needs a diagonal band narrower than the pattern are scored on 1 to 16 32-bit words of
band.  Seeded long strings over small and full byte alphabets, cutoffs that select every
band width, all four ops, compared with the oracle element by element (integers exact,
doubles by bit pattern)."""
import numpy as np
import pytest

from oracle_lib import oracle_cdist

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402


def _same(a, b):
    if a.dtype == np.float64:
        return np.array_equal(a.view(np.int64), b.view(np.int64))
    return np.array_equal(a, b)


def _batch(rng, lens, alphabet, base=None, rate=0.0):
    out = []
    for i, n in enumerate(lens):
        if base is not None and rng.random() < 0.5:
            s = bytearray(base[int(rng.integers(0, len(base)))])
            for _ in range(int(len(s) * rate * rng.random())):
                k = int(rng.integers(0, 3))
                pos = int(rng.integers(0, max(1, len(s))))
                if k == 0 and s:
                    s[pos % len(s)] = alphabet[int(rng.integers(0, len(alphabet)))]
                elif k == 1:
                    s.insert(pos, alphabet[int(rng.integers(0, len(alphabet)))])
                elif s:
                    del s[pos % len(s)]
            out.append(bytes(s))
        else:
            out.append(bytes(np.asarray(alphabet, dtype=np.uint8)[rng.integers(0, len(alphabet), size=int(n))]))
    return out


@pytest.mark.parametrize("alphabet", ["dna", "bytes"])
def test_band_classes_match_oracle(alphabet):
    rng = np.random.default_rng(91 if alphabet == "dna" else 92)
    alpha = list(b"ACGT") if alphabet == "dna" else list(range(256))
    qlens = rng.integers(70, 2600, size=40)
    qs = _batch(rng, qlens, alpha)
    cs = _batch(rng, rng.integers(40, 2800, size=700), alpha, base=qs, rate=0.2)
    q, c = R.pack_strings(qs, 1), R.pack_strings(cs, 1)
    cases = [(R.DISTANCE, 5), (R.DISTANCE, 20), (R.DISTANCE, 47), (R.DISTANCE, 90), (R.DISTANCE, 150),
             (R.DISTANCE, 250), (R.NORMALIZED_DISTANCE, 0.05), (R.NORMALIZED_DISTANCE, 0.1),
             (R.NORMALIZED_DISTANCE, 0.18), (R.NORMALIZED_SIMILARITY, 0.9), (R.NORMALIZED_SIMILARITY, 0.85),
             (R.SIMILARITY, 2000)]
    for op, cut in cases:
        for dt in ((None,) if op >= R.NORMALIZED_DISTANCE else (R.I32, R.I64, R.F64)):
            got = R.cdist(R.LEVENSHTEIN, op, q, c, cut, out_dtype=dt)
            exp = oracle_cdist(R.LEVENSHTEIN, op, q, c, cut, out_dtype={None: None, R.I32: 0, R.I64: 1, R.F64: 2}[dt])
            assert _same(got, exp), (op, cut, dt)


@pytest.mark.parametrize("rounds", [2, 5])
def test_band_units_of_several_rounds_match_oracle(rounds):
    """band units of several 32-pair groups (the size the host picks for large classes),
    forced through the launch-shape hook on a batch small enough for the oracle"""
    lib = R.lib()
    rng = np.random.default_rng(95 + rounds)
    alpha = list(b"ACGT")
    qs = _batch(rng, rng.integers(150, 900, size=12), alpha)
    cs = _batch(rng, rng.integers(100, 1000, size=1500), alpha, base=qs, rate=0.1)
    q, c = R.pack_strings(qs, 1), R.pack_strings(cs, 1)
    try:
        assert lib.rfg_testing_band_rounds(rounds) == 0
        for op, cut in ((R.NORMALIZED_DISTANCE, 0.1), (R.DISTANCE, 40), (R.SIMILARITY, 600)):
            got = R.cdist(R.LEVENSHTEIN, op, q, c, cut)
            exp = oracle_cdist(R.LEVENSHTEIN, op, q, c, cut)
            assert _same(got, exp), (rounds, op, cut)
    finally:
        lib.rfg_testing_band_rounds(0)
