"""The warp tiles' count filter (hist_lower_bound) and survivor batches at their edges,
compared with the oracle element by element: queries of 0..64 units against choices of
0..400 units (the filter covers strings of at most 255 units and is off for longer ones),
cutoffs on both sides of the 510 at which it switches off, near-duplicate choices (most
pairs survive the bound and run the recurrence) and unrelated ones (almost none
survive), one-, two- and four-byte code units, int32 / int64 / float64 results, and a
prepared batch replayed as a graph."""
import numpy as np
import pytest

from oracle_lib import oracle_cdist

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402

DT = {R.I32: 0, R.I64: 1, R.F64: 2}


def _same(a, b):
    if a.dtype == np.float64:
        return np.array_equal(a.view(np.int64), b.view(np.int64))
    return np.array_equal(a, b)


def _strings(rng, n, lo, hi, alpha, base=None, edits=0):
    out = []
    for _ in range(n):
        if base is not None and rng.random() < 0.6:
            s = list(base[int(rng.integers(0, len(base)))])
            for _ in range(int(rng.integers(0, edits + 1))):
                k = int(rng.integers(0, 3))
                p = int(rng.integers(0, max(1, len(s))))
                if k == 0 and s:
                    s[p % len(s)] = alpha[int(rng.integers(0, len(alpha)))]
                elif k == 1:
                    s.insert(p, alpha[int(rng.integers(0, len(alpha)))])
                elif s:
                    del s[p % len(s)]
            out.append(s)
        else:
            out.append([alpha[int(x)] for x in rng.integers(0, len(alpha), size=int(rng.integers(lo, hi + 1)))])
    return out


def _pack(strs, width):
    dt = {1: np.uint8, 2: np.uint16, 4: np.uint32}[width]
    off = np.zeros(len(strs) + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(s) for s in strs])
    data = np.array([c for s in strs for c in s], dtype=dt) if off[-1] else np.zeros(0, dtype=dt)
    return data, off, width


@pytest.mark.parametrize("width", [1, 2, 4])
def test_count_filter_edges_match_oracle(width):
    rng = np.random.default_rng(700 + width)
    alpha = list(range(97, 123)) if width == 1 else list(range(97, 123)) + [0xC0 + k for k in range(14)]
    # four-byte choices also hold code units above 255, which no pattern row has (the
    # queries stay below 256, so the warp tiles take them)
    calpha = alpha + [0x4E00 + k for k in range(6)] if width == 4 else alpha
    qs = _strings(rng, 120, 0, 64, alpha)
    qs[0], qs[1] = [], [alpha[0]] * 64
    cs = _strings(rng, 900, 0, 400, calpha, base=qs, edits=6)
    cs[0], cs[1] = [], [alpha[0]] * 300
    q, c = _pack(qs, width), _pack(cs, width)
    for metric in (R.LEVENSHTEIN, R.INDEL, R.OSA):
        for cut in (0, 1, 8, 100, 254, 255, 300, 509, 510, 1000):
            for dt in ((R.I32,) if cut not in (8, 509) else (R.I32, R.I64, R.F64)):
                got = R.cdist(metric, R.DISTANCE, q, c, cut, out_dtype=dt)
                exp = oracle_cdist(metric, R.DISTANCE, q, c, cut, out_dtype=DT[dt])
                assert _same(got, exp), (width, metric, cut, dt, int((got != exp).sum()))


def test_count_filter_batch_replay_matches_oracle():
    """a prepared batch over device strings, replayed as a graph twice with the result
    overwritten in between; near-duplicates, so the survivor batches are full"""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(733)
    alpha = list(range(97, 123))
    qs = _strings(rng, 300, 16, 64, alpha)
    cs = _strings(rng, 3000, 8, 72, alpha, base=qs, edits=4)
    q, c = _pack(qs, 1), _pack(cs, 1)
    dev = torch.device("cuda", 0)
    td = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (q[0], q[1], c[0], c[1])]
    qd = (td[0].data_ptr(), td[1].data_ptr(), 1, len(qs))
    cd = (td[2].data_ptr(), td[3].data_ptr(), 1, len(cs))
    stream = torch.cuda.Stream(device=dev)
    for metric in (R.LEVENSHTEIN, R.INDEL, R.OSA):
        out = torch.empty((len(qs), len(cs)), dtype=torch.int32, device=dev)
        b = R.Batch(metric, R.DISTANCE, qd, cd, out.data_ptr(), 6, out_dtype=R.I32, flags=R.DEVICE_INPUTS)
        exp = oracle_cdist(metric, R.DISTANCE, q, c, 6, out_dtype=0)
        for _ in range(2):
            out.fill_(-7)
            b.launch(stream.cuda_stream, graph=True)
            b.check(stream.cuda_stream)
            assert np.array_equal(out.cpu().numpy(), exp), metric
        b.close()
