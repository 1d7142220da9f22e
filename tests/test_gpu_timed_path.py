"""Whole-matrix parity of the paths the benchmark times, at the benchmark's full sizes.

The headline workload (4,096 x 4,096 a-z Zipf(1.1) strings, lengths U[16, 64], 20 % mutated
copies, seed 1234; Levenshtein, Indel and OSA with score_cutoff 8, int32 results) runs
through the same prepared batches as the benchmark: device-resident strings, tuned launch
shapes, CUDA-graph replay.  Every element of every matrix is compared with the oracle (the
CPU restatement of the reference's Cached* path) -- integers bit-exact -- after two graph
replays with the result buffer overwritten in between, so a replay that skips a tile cannot
pass on stale values.  The public cdist call is checked the same way into pinned and into
pageable host memory, and the other benchmark shapes over their full choice sets:
1 x 100,000 DNA (Levenshtein, no cutoff, int64), 32 x 65,536 long DNA (normalized
Levenshtein <= 0.1), 64 x 1,000,000 uint32 token strings (Jaro-Winkler 0.85 and
fuzz::ratio 85, doubles compared by bit pattern)."""
import numpy as np
import pytest

from oracle_lib import oracle_cdist

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402
import workloads as WL  # noqa: E402

CUTOFF = 8
METRICS = ((R.LEVENSHTEIN, "levenshtein"), (R.INDEL, "indel"), (R.OSA, "osa"))


def _same(a, b):
    if a.dtype == np.float64:
        return np.array_equal(a.view(np.int64), b.view(np.int64))
    return np.array_equal(a, b)


def _mismatch(a, b):
    bad = np.argwhere(a != b)
    return "%d mismatches, first at %s: got %s expected %s" % (len(bad), tuple(bad[0]), a[tuple(bad[0])],
                                                                 b[tuple(bad[0])]) if len(bad) else ""


@pytest.fixture(scope="module")
def headline():
    q, c = WL.cdist_zipf(seed=1234, nq=4096, nc=4096)
    exp = {m: oracle_cdist(m, R.DISTANCE, q, c, CUTOFF, out_dtype=0) for m, _ in METRICS}
    return q, c, exp


def test_prepared_batches_tuned_graph_replay_full_matrix(headline):
    torch = pytest.importorskip("torch")
    q, c, exp = headline
    nq, nc = len(q[1]) - 1, len(c[1]) - 1
    dev = torch.device("cuda", 0)
    qd, qo = torch.from_numpy(q[0]).to(dev), torch.from_numpy(q[1]).to(dev)
    cd, co = torch.from_numpy(c[0]).to(dev), torch.from_numpy(c[1]).to(dev)
    stream = torch.cuda.Stream(device=dev)
    for m, name in METRICS:
        out = torch.full((nq, nc), -7, dtype=torch.int32, device=dev)
        b = R.Batch(m, R.DISTANCE, (qd.data_ptr(), qo.data_ptr(), 1, nq), (cd.data_ptr(), co.data_ptr(), 1, nc),
                    out.data_ptr(), CUTOFF, out_dtype=R.I32, flags=R.DEVICE_INPUTS)
        try:
            b.tune(stream.cuda_stream)
            for rep in range(2):
                with torch.cuda.stream(stream):
                    out.fill_(-7)
                b.launch(stream.cuda_stream, graph=True)
                b.check(stream.cuda_stream)
                stream.synchronize()
                got = out.cpu().numpy()
                assert _same(got, exp[m]), "%s replay %d: %s" % (name, rep, _mismatch(got, exp[m]))
            # a plain (non-graph) launch of the same prepared batch
            with torch.cuda.stream(stream):
                out.fill_(-7)
            b.launch(stream.cuda_stream, graph=False)
            b.check(stream.cuda_stream)
            stream.synchronize()
            assert _same(out.cpu().numpy(), exp[m]), name
        finally:
            b.close()


def test_cdist_into_pinned_and_pageable_host_memory_full_matrix(headline):
    torch = pytest.importorskip("torch")
    q, c, exp = headline
    nq, nc = len(q[1]) - 1, len(c[1]) - 1
    pinned = torch.empty((nq, nc), dtype=torch.int32).pin_memory().numpy()
    for m, name in METRICS:
        pinned.fill(-7)
        R.cdist(m, R.DISTANCE, q, c, CUTOFF, out_dtype=R.I32, out=pinned)
        assert _same(pinned, exp[m]), "%s pinned: %s" % (name, _mismatch(pinned, exp[m]))
        pageable = R.cdist(m, R.DISTANCE, q, c, CUTOFF, out_dtype=R.I32)
        assert _same(pageable, exp[m]), "%s pageable: %s" % (name, _mismatch(pageable, exp[m]))


def test_config1_all_choices():
    c = WL.dna_uniform(seed=1, n=100000)
    q = WL.dna_uniform(seed=2, n=1)
    got = R.cdist(R.LEVENSHTEIN, R.DISTANCE, q, c)
    exp = oracle_cdist(R.LEVENSHTEIN, R.DISTANCE, q, c)
    assert _same(got, exp), _mismatch(got, exp)


def test_config3_all_choices():
    q, c = WL.dna_lognormal(seed=4, nq=32, nc=65536)
    got = R.cdist(R.LEVENSHTEIN, R.NORMALIZED_DISTANCE, q, c, 0.1)
    exp = oracle_cdist(R.LEVENSHTEIN, R.NORMALIZED_DISTANCE, q, c, 0.1)
    assert _same(got, exp)
    # the integer form of the same band (cutoff = 10 % of the longest string)
    got = R.cdist(R.LEVENSHTEIN, R.DISTANCE, q, c, 200)
    exp = oracle_cdist(R.LEVENSHTEIN, R.DISTANCE, q, c, 200)
    assert _same(got, exp), _mismatch(got, exp)


def test_config4_all_choices():
    (q, ql) = WL.tokens_u32(seed=14, n=64)
    c = WL.tokens_u32_mixed(seed=15, n=1_000_000, derive_from=ql, derive_count=20_000)
    for m, cut in ((R.JARO_WINKLER, 0.85), (R.RATIO, 85.0)):
        got = R.cdist(m, R.SIMILARITY, q, c, cut)
        exp = oracle_cdist(m, R.SIMILARITY, q, c, cut)
        assert _same(got, exp), m
        assert (got > 0).sum() > 1000  # the derived choices give hits above the cutoff


def test_long_dna_band_workloads_full_matrix():
    """the long-DNA band workloads exactly as the bench times them (256 x 65,536 DNA,
    seed 13): prepared batches over device strings, replayed as graphs, every element
    against the oracle -- Levenshtein (k_band) and Indel / ratio (the LCS band classes)"""
    torch = pytest.importorskip("torch")
    q, c = WL.dna_lognormal(seed=13, nq=256, nc=65536)
    dev = torch.device("cuda", 0)
    td = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (q[0], q[1], c[0], c[1])]
    qd = (td[0].data_ptr(), td[1].data_ptr(), 1, 256)
    cd = (td[2].data_ptr(), td[3].data_ptr(), 1, 65536)
    stream = torch.cuda.Stream(device=dev)
    out = torch.empty((256, 65536), dtype=torch.float64, device=dev)
    for metric, op, cut in ((R.LEVENSHTEIN, R.NORMALIZED_DISTANCE, 0.1), (R.INDEL, R.NORMALIZED_DISTANCE, 0.1),
                            (R.RATIO, R.SIMILARITY, 90.0)):
        b = R.Batch(metric, op, qd, cd, out.data_ptr(), cut, out_dtype=R.F64, flags=R.DEVICE_INPUTS)
        assert any("k_band" in k for k in b.kernels()), b.kernels()
        exp = oracle_cdist(metric, op, q, c, cut)
        for _ in range(2):
            out.fill_(-1.0)
            b.launch(stream.cuda_stream, graph=True)
            b.check(stream.cuda_stream)
            got = out.cpu().numpy()
            assert _same(got, exp), (metric, _mismatch(got, exp))
        b.close()
