"""Failure handling on the GPU path, without faulting the GPU: broken offsets of
device-resident string batches are refused before any kernel reads through them; the
server refuses a request that alone exceeds its device-memory budget and a wait runs out
on its timeout without losing the request; device allocations made to fail on the host
(rfg_testing_fail_device_allocs) surface as RFG_ERR_OUT_OF_MEMORY and leave the library
usable -- the next call gives the oracle's results."""
import ctypes

import numpy as np
import pytest

from oracle_lib import oracle_cdist

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402
from rapidfuzz_gb300._lib import Cutoff, Strings, make_params  # noqa: E402
import workloads as WL  # noqa: E402


def _dev(torch, data, off, width=1):
    d = torch.from_numpy(np.ascontiguousarray(data)).cuda()
    o = torch.from_numpy(np.ascontiguousarray(np.asarray(off, dtype=np.int64))).cuda()
    return (d, o), Strings(d.data_ptr(), o.data_ptr(), len(off) - 1, width)


def test_device_batches_with_broken_offsets_are_refused():
    torch = pytest.importorskip("torch")
    L = R.lib()
    data = np.frombuffer(b"abcdefghijklmnop", dtype=np.uint8).copy()
    kg, good = _dev(torch, data, [0, 3, 6, 9])
    p = make_params()
    cut = Cutoff(8, 0.0, 0, 0.0)
    out = torch.zeros(64, dtype=torch.int64, device="cuda")
    flags = R.DEVICE_INPUTS | R.DEVICE_OUTPUT
    for off in ([0, 3, 2, 9], [-4, 3, 6, 9], [0, 1, 2, 2 + 2**31]):
        kb, bad = _dev(torch, data, off)
        for q, c in ((bad, good), (good, bad)):
            assert L.rfg_cdist(R.LEVENSHTEIN, R.DISTANCE, R.FORM_CACHED, ctypes.byref(q), ctypes.byref(c),
                               ctypes.byref(p), cut, R.I64, out.data_ptr(), 0, flags) == 1, off
            h = ctypes.c_void_p()
            assert L.rfg_batch_create(R.INDEL, R.DISTANCE, R.FORM_CACHED, ctypes.byref(q), ctypes.byref(c),
                                      ctypes.byref(p), cut, R.I64, out.data_ptr(), 0, R.DEVICE_INPUTS,
                                      ctypes.byref(h)) == 1, off
        h = ctypes.c_void_p()
        assert L.rfg_corpus_create(ctypes.byref(bad), R.DEVICE_INPUTS, ctypes.byref(h)) == 1
    # the library still scores a good batch
    assert L.rfg_cdist(R.LEVENSHTEIN, R.DISTANCE, R.FORM_CACHED, ctypes.byref(good), ctypes.byref(good),
                       ctypes.byref(p), cut, R.I64, out.data_ptr(), 0, flags) == 0
    torch.cuda.synchronize()
    assert out[:9].cpu().numpy().reshape(3, 3).diagonal().tolist() == [0, 0, 0]


def test_server_refuses_a_request_over_its_memory_budget():
    corpus = R.Corpus(WL.dna_uniform(seed=3, n=20000))
    small = R.Server([corpus], max_inflight=2, max_batch=8, max_device_bytes=64 * 1024)
    try:
        with pytest.raises(R.RapidfuzzError) as e:
            small.submit(0, R.LEVENSHTEIN, R.DISTANCE, b"ACGTACGT", 10)
        assert e.value.status == 7 and "max_device_bytes" in str(e.value)
    finally:
        small.close()
    ok = R.Server([corpus], max_inflight=2, max_batch=8)
    try:
        t = ok.submit(0, R.LEVENSHTEIN, R.DISTANCE, b"ACGTACGT", 10)
        idx, sc, _ = ok.wait(t)
        ei, es, en = corpus.extract(R.LEVENSHTEIN, R.DISTANCE, R.pack_strings([b"ACGTACGT"], 1), 10, None, False)
        assert list(idx) == list(ei[0][:en[0]]) and list(sc) == list(es[0][:en[0]])
    finally:
        ok.close()


def test_server_wait_times_out_and_the_request_survives():
    corpus = R.Corpus(WL.dna_corpus_fast(seed=4, n=1_000_000))
    srv = R.Server([corpus], max_inflight=1, max_batch=4)
    rng = np.random.default_rng(5)
    qs = [bytes(np.frombuffer(b"ACGT", dtype=np.uint8)[rng.integers(0, 4, size=400)]) for _ in range(48)]
    try:
        tickets = [srv.submit(0, R.OSA, R.DISTANCE, q, 10) for q in qs]
        with pytest.raises(R.RapidfuzzError) as e:
            srv.wait(tickets[-1], timeout=1e-4)
        assert e.value.status == 7 and "timed out" in str(e.value)
        idx, sc, _ = srv.wait(tickets[-1])
        ei, es, en = corpus.extract(R.OSA, R.DISTANCE, R.pack_strings([qs[-1]], 1), 10, None, False)
        assert list(idx) == list(ei[0][:en[0]]) and list(sc) == list(es[0][:en[0]])
        for t in tickets[:-1]:
            srv.wait(t)
    finally:
        srv.close()


def test_injected_allocation_failure_then_recovery():
    L = R.lib()
    q, c = WL.cdist_zipf(seed=6, nq=64, nc=900)
    exp = oracle_cdist(R.INDEL, R.DISTANCE, q, c, 8)
    try:
        for after in (0, 1, 2):
            assert L.rfg_testing_fail_device_allocs(after) == 0
            with pytest.raises(R.RapidfuzzError) as e:
                R.cdist(R.INDEL, R.DISTANCE, q, c, 8)
            assert e.value.status == 4, after
    finally:
        L.rfg_testing_fail_device_allocs(-1)
    got = R.cdist(R.INDEL, R.DISTANCE, q, c, 8)
    assert np.array_equal(got, exp)
