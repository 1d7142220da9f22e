"""The band classes of unit-weight Levenshtein and of the LCS families (k_band): queries
whose every passing pair needs a diagonal band narrower than the pattern are scored on 1
to 16 32-bit words of band.  Seeded long strings over small and full byte alphabets, cutoffs that select every
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
        for metric, op, cut in ((R.LEVENSHTEIN, R.NORMALIZED_DISTANCE, 0.1), (R.LEVENSHTEIN, R.DISTANCE, 40),
                                (R.LEVENSHTEIN, R.SIMILARITY, 600), (R.INDEL, R.NORMALIZED_DISTANCE, 0.1),
                                (R.LCSSEQ, R.DISTANCE, 40), (R.RATIO, R.SIMILARITY, 92.0)):
            got = R.cdist(metric, op, q, c, cut)
            exp = oracle_cdist(metric, op, q, c, cut)
            assert _same(got, exp), (rounds, metric, op, cut)
    finally:
        lib.rfg_testing_band_rounds(0)


LCS_CASES = [
    (R.INDEL, R.DISTANCE, 10), (R.INDEL, R.DISTANCE, 45), (R.INDEL, R.DISTANCE, 120), (R.INDEL, R.DISTANCE, 300),
    (R.INDEL, R.SIMILARITY, 2500), (R.INDEL, R.NORMALIZED_DISTANCE, 0.05), (R.INDEL, R.NORMALIZED_DISTANCE, 0.1),
    (R.INDEL, R.NORMALIZED_SIMILARITY, 0.88),
    (R.LCSSEQ, R.DISTANCE, 30), (R.LCSSEQ, R.DISTANCE, 140), (R.LCSSEQ, R.SIMILARITY, 1200),
    (R.LCSSEQ, R.NORMALIZED_DISTANCE, 0.06), (R.LCSSEQ, R.NORMALIZED_SIMILARITY, 0.9),
    (R.RATIO, R.SIMILARITY, 90.0), (R.RATIO, R.SIMILARITY, 95.0), (R.RATIO, R.SIMILARITY, 97.5),
]


@pytest.mark.parametrize("alphabet", ["dna", "bytes"])
def test_lcs_band_classes_match_oracle(alphabet):
    """the banded LCS families (Indel, LCSseq, ratio; lcs_blockwise's band): every op,
    cutoffs that select band widths from 1 to 16 words, every output type"""
    rng = np.random.default_rng(191 if alphabet == "dna" else 192)
    alpha = list(b"ACGT") if alphabet == "dna" else list(range(256))
    qs = _batch(rng, rng.integers(70, 2600, size=40), alpha)
    cs = _batch(rng, rng.integers(40, 2800, size=700), alpha, base=qs, rate=0.2)
    q, c = R.pack_strings(qs, 1), R.pack_strings(cs, 1)
    for metric, op, cut in LCS_CASES:
        ints = metric != R.RATIO and op < R.NORMALIZED_DISTANCE
        for dt in ((R.I32, R.I64, R.F64) if ints else (None,)):
            got = R.cdist(metric, op, q, c, cut, out_dtype=dt)
            exp = oracle_cdist(metric, op, q, c, cut, out_dtype={None: None, R.I32: 0, R.I64: 1, R.F64: 2}[dt])
            assert _same(got, exp), (metric, op, cut, dt, int((got != exp).sum()))


def test_lcs_band_batch_runs_band_kernel_and_replays():
    """a prepared Indel / ratio batch over long DNA takes the LCS band kernel
    (k_band<u8, B, true>), and its graph replays give the oracle's matrix"""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(197)
    alpha = list(b"ACGT")
    qs = _batch(rng, rng.integers(200, 1500, size=24), alpha)
    cs = _batch(rng, rng.integers(150, 1600, size=3000), alpha, base=qs, rate=0.12)
    q, c = R.pack_strings(qs, 1), R.pack_strings(cs, 1)
    dev = torch.device("cuda", 0)
    td = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (q[0], q[1], c[0], c[1])]
    qd = (td[0].data_ptr(), td[1].data_ptr(), 1, len(qs))
    cd = (td[2].data_ptr(), td[3].data_ptr(), 1, len(cs))
    stream = torch.cuda.Stream(device=dev)
    for metric, op, cut, dt, tdt in ((R.INDEL, R.NORMALIZED_DISTANCE, 0.1, R.F64, torch.float64),
                                     (R.INDEL, R.DISTANCE, 60, R.I32, torch.int32),
                                     (R.RATIO, R.SIMILARITY, 92.0, R.F64, torch.float64)):
        out = torch.empty((len(qs), len(cs)), dtype=tdt, device=dev)
        b = R.Batch(metric, op, qd, cd, out.data_ptr(), cut, out_dtype=dt, flags=R.DEVICE_INPUTS)
        names = b.kernels()
        assert any("k_band" in k and "Lb1E" in k for k in names), names
        exp = oracle_cdist(metric, op, q, c, cut, out_dtype={R.I32: 0, R.F64: 2}[dt])
        for _ in range(2):
            out.fill_(-3)
            b.launch(stream.cuda_stream, graph=True)
            b.check(stream.cuda_stream)
            assert _same(out.cpu().numpy(), exp), (metric, op, cut)
        b.close()


def test_band_mode_hook_keeps_results():
    """with the band kernels switched off (rfg_testing_band_mode) the same Indel and
    Levenshtein batches run on the unbanded multi-word cores and give the same matrices"""
    lib = R.lib()
    rng = np.random.default_rng(199)
    alpha = list(b"ACGT")
    qs = _batch(rng, rng.integers(120, 1200, size=16), alpha)
    cs = _batch(rng, rng.integers(100, 1300, size=1200), alpha, base=qs, rate=0.1)
    q, c = R.pack_strings(qs, 1), R.pack_strings(cs, 1)
    cases = ((R.INDEL, R.NORMALIZED_DISTANCE, 0.1), (R.LEVENSHTEIN, R.DISTANCE, 50), (R.LCSSEQ, R.SIMILARITY, 500))
    exp = [oracle_cdist(mt, op, q, c, cut) for mt, op, cut in cases]
    try:
        for mode in (0, 1):
            assert lib.rfg_testing_band_mode(mode) == 0
            for (mt, op, cut), e in zip(cases, exp):
                assert _same(R.cdist(mt, op, q, c, cut), e), (mode, mt, op, cut)
    finally:
        lib.rfg_testing_band_mode(1)
