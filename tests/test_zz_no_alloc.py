"""rfg_cdist_noalloc: all-pairs scoring for callers that cannot allocate device memory.

Such callers (code living inside another framework's memory manager, processes whose
device memory is reserved up front, services that must not grow after start-up) hold
their strings and result buffer on the device already; the entry point runs the
any-length kernel with its scratch in a fixed 32 MiB array of the library's device
image instead of allocating.  These checks call it through the C ABI twice in a row and
compare every result with rfg_cdist on the same device buffers (tolerance 0: integers
bit-exact, doubles bit-identical).  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402
from rapidfuzz_gb300._lib import Cutoff, Strings, make_params, check  # noqa: E402
from workloads import dna_lognormal, tokens_u32  # noqa: E402


def _device_batch(torch, data, offsets, width):
    d = torch.from_numpy(np.ascontiguousarray(data)).cuda()
    o = torch.from_numpy(np.ascontiguousarray(offsets)).cuda()
    return (d, o), Strings(d.data_ptr(), o.data_ptr(), offsets.size - 1, width)


def _run_both(torch, metric, op, q, c, cutoff, out_dtype, max_len, weights=(1, 1, 1)):
    keep_q, qs = _device_batch(torch, *q)
    keep_c, cs = _device_batch(torch, *c)
    nq, nc = qs.count, cs.count
    tdt = torch.int64 if out_dtype == R.I64 else (torch.int32 if out_dtype == R.I32 else torch.float64)
    out_new = torch.full((nq, nc), -1, dtype=tdt, device="cuda")
    out_ref = torch.full((nq, nc), -2, dtype=tdt, device="cuda")
    p = make_params(weights)
    is_int = out_dtype != R.F64
    cut = Cutoff(int(cutoff) if is_int else 0, 0.0 if is_int else float(cutoff), 0, 0.0)
    torch.cuda.synchronize()
    L = R.lib()
    check(L.rfg_cdist_noalloc(metric, op, R.FORM_CACHED, ctypes.byref(qs), ctypes.byref(cs), max_len,
                              ctypes.byref(p), cut, out_dtype, out_new.data_ptr(), 0, None))
    check(L.rfg_cdist(metric, op, R.FORM_CACHED, ctypes.byref(qs), ctypes.byref(cs), ctypes.byref(p), cut, out_dtype,
                      out_ref.data_ptr(), 0, R.DEVICE_INPUTS | R.DEVICE_OUTPUT))
    torch.cuda.synchronize()
    a, b = out_new.cpu().numpy(), out_ref.cpu().numpy()
    if a.dtype == np.float64:
        a, b = a.view(np.int64), b.view(np.int64)
    return a, b, keep_q, keep_c


def test_no_alloc_matches_cdist_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    # call 1: banded Levenshtein on long DNA strings (multi-word patterns)
    q, c = dna_lognormal(seed=5, nq=12, nc=300, median=300, sigma=0.5, lo=100, hi=1500)
    a, b, *_ = _run_both(torch, R.LEVENSHTEIN, R.DISTANCE, q, c, 40, R.I64, max_len=2000)
    assert np.array_equal(a, b)
    # call 2, right after: Jaro-Winkler over uint32 token strings (doubles)
    (tq, tq_list) = tokens_u32(seed=6, n=40)
    (tc, _) = tokens_u32(seed=7, n=500, derive_from=tq_list, derive_frac=0.3)
    a, b, *_ = _run_both(torch, R.JARO_WINKLER, R.SIMILARITY, tq, tc, 0.8, R.F64, max_len=64)
    assert np.array_equal(a, b)
    # and a third: weighted Levenshtein (Wagner-Fischer family) reusing the same scratch
    a, b, *_ = _run_both(torch, R.LEVENSHTEIN, R.DISTANCE, tq, tc, 2**62, R.I64, max_len=64, weights=(1, 2, 3))
    assert np.array_equal(a, b)


def test_no_alloc_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    q, c = dna_lognormal(seed=8, nq=3, nc=10, median=300, sigma=0.3, lo=200, hi=400)
    keep_q, qs = _device_batch(torch, *q)
    keep_c, cs = _device_batch(torch, *c)
    out = torch.zeros((3, 10), dtype=torch.int64, device="cuda")
    p = make_params()
    L = R.lib()
    # bound above the stated maximum (4096 code units)
    rc = L.rfg_cdist_noalloc(R.LEVENSHTEIN, R.DISTANCE, R.FORM_CACHED, ctypes.byref(qs), ctypes.byref(cs), 5000,
                             ctypes.byref(p), Cutoff(10, 0.0, 0, 0.0), R.I64, out.data_ptr(), 0, None)
    assert rc == 1 and b"4096" in L.rfg_last_error()
    # a query longer than the caller's bound
    rc = L.rfg_cdist_noalloc(R.LEVENSHTEIN, R.DISTANCE, R.FORM_CACHED, ctypes.byref(qs), ctypes.byref(cs), 100,
                             ctypes.byref(p), Cutoff(10, 0.0, 0, 0.0), R.I64, out.data_ptr(), 0, None)
    assert rc == 1 and b"max_query_len" in L.rfg_last_error()
