"""rfg_cdist_noalloc: all-pairs scoring for callers that cannot allocate device memory.

Such callers (code living inside another framework's memory manager, processes whose
device memory is reserved up front, services that must not grow after start-up) hold
their strings and result buffer on the device already; the entry point runs the
any-length kernel with its scratch in a fixed 32 MiB array of the library's device
image instead of allocating.  These checks call it through the C ABI several times in a
row and compare every result with rfg_cdist on the same device buffers and with the
oracle (the CPU restatement of the reference), tolerance 0: integers bit-exact, doubles
bit-identical.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from oracle_lib import oracle_cdist

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402
from rapidfuzz_gb300._lib import Cutoff, Strings, make_params, check  # noqa: E402
from workloads import dna_lognormal, tokens_u32  # noqa: E402


def _device_batch(torch, data, offsets, width):
    d = torch.from_numpy(np.ascontiguousarray(data)).cuda()
    o = torch.from_numpy(np.ascontiguousarray(offsets)).cuda()
    return (d, o), Strings(d.data_ptr(), o.data_ptr(), offsets.size - 1, width)


def _bits(a):
    return a.view(np.int64) if a.dtype == np.float64 else a


def _run_both(torch, metric, op, q, c, cutoff, out_dtype, max_len, weights=(1, 1, 1), form=R.FORM_CACHED,
              oracle=True):
    """(no-allocation result, rfg_cdist result, oracle result or None) as comparable arrays"""
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
    check(L.rfg_cdist_noalloc(metric, op, form, ctypes.byref(qs), ctypes.byref(cs), max_len,
                              ctypes.byref(p), cut, out_dtype, out_new.data_ptr(), 0, None))
    check(L.rfg_cdist(metric, op, form, ctypes.byref(qs), ctypes.byref(cs), ctypes.byref(p), cut, out_dtype,
                      out_ref.data_ptr(), 0, R.DEVICE_INPUTS | R.DEVICE_OUTPUT))
    torch.cuda.synchronize()
    a, b = _bits(out_new.cpu().numpy()), _bits(out_ref.cpu().numpy())
    exp = None
    if oracle:
        exp = _bits(oracle_cdist(metric, op, q, c, cutoff, weights=weights,
                                 out_dtype={R.I32: 0, R.I64: 1, R.F64: 2}[out_dtype]))
    return a, b, exp


def _check(a, b, exp):
    assert np.array_equal(a, b)
    if exp is not None:
        assert np.array_equal(a, exp)


def _long_u16(seed, n, lo, hi, alphabet):
    """n strings of 2-byte code units (including units above 255), lengths U[lo, hi]"""
    rng = np.random.default_rng(seed)
    lens = rng.integers(lo, hi + 1, size=n)
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    data = np.asarray(alphabet, dtype=np.uint16)[rng.integers(0, len(alphabet), size=int(off[-1]))]
    return data, off, 2


def test_no_alloc_matches_cdist_and_oracle_on_calls_in_a_row():
    torch = pytest.importorskip("torch")
    # call 1: banded Levenshtein on long DNA strings (multi-word patterns)
    q, c = dna_lognormal(seed=5, nq=12, nc=300, median=300, sigma=0.5, lo=100, hi=1500)
    _check(*_run_both(torch, R.LEVENSHTEIN, R.DISTANCE, q, c, 40, R.I64, max_len=2000))
    # call 2, right after: Jaro-Winkler over uint32 token strings (doubles)
    (tq, tq_list) = tokens_u32(seed=6, n=40)
    (tc, _) = tokens_u32(seed=7, n=500, derive_from=tq_list, derive_frac=0.3)
    _check(*_run_both(torch, R.JARO_WINKLER, R.SIMILARITY, tq, tc, 0.8, R.F64, max_len=64))
    # and a third: weighted Levenshtein (Wagner-Fischer family) reusing the same scratch
    _check(*_run_both(torch, R.LEVENSHTEIN, R.DISTANCE, tq, tc, 2**62, R.I64, max_len=64, weights=(1, 2, 3)))


def test_no_alloc_largest_queries_two_byte_units():
    """queries up to the 4,096-unit limit over 2-byte code units (the most scratch per
    block, hash rows for the units above 255): OSA, Indel and fuzz::ratio, twice in a row"""
    torch = pytest.importorskip("torch")
    alpha = list(range(97, 107)) + [0x3B1, 0x3B2, 0x3B3, 0x5D0, 0x5D1]
    q = _long_u16(11, 4, 3000, 4096, alpha)
    c = _long_u16(12, 60, 2800, 4096, alpha)
    _check(*_run_both(torch, R.OSA, R.DISTANCE, q, c, 2**62, R.I64, max_len=4096))
    _check(*_run_both(torch, R.INDEL, R.NORMALIZED_SIMILARITY, q, c, 0.3, R.F64, max_len=4096))
    _check(*_run_both(torch, R.RATIO, R.SIMILARITY, q, c, 20.0, R.F64, max_len=4096))
    _check(*_run_both(torch, R.OSA, R.DISTANCE, q, c, 2**62, R.I64, max_len=4096))


def test_no_alloc_multi_form_and_mixed_widths():
    torch = pytest.importorskip("torch")
    (tq, tq_list) = tokens_u32(seed=16, n=24)
    (tc, _) = tokens_u32(seed=17, n=300, derive_from=tq_list, derive_frac=0.3)
    # the experimental::Multi* chains (patterns of at most 64 units)
    for metric, op, cut, dt in ((R.LEVENSHTEIN, R.NORMALIZED_SIMILARITY, 0.6, R.F64),
                                (R.INDEL, R.DISTANCE, 10, R.I64), (R.JARO_WINKLER, R.SIMILARITY, 0.85, R.F64)):
        a, b, _ = _run_both(torch, metric, op, tq, tc, cut, dt, max_len=64, form=R.FORM_MULTI, oracle=False)
        assert np.array_equal(a, b)
    # one-byte queries against four-byte choices (choice units above 255 match nothing)
    rng = np.random.default_rng(18)
    qb = [bytes(rng.integers(97, 123, size=int(rng.integers(0, 90))).astype(np.uint8)) for _ in range(20)]
    q1 = R.pack_strings(qb, 1)
    for metric, op, cut, dt in ((R.LEVENSHTEIN, R.DISTANCE, 30, R.I32), (R.OSA, R.SIMILARITY, 5, R.I64),
                                (R.RATIO, R.SIMILARITY, 50.0, R.F64)):
        _check(*_run_both(torch, metric, op, q1, tc, cut, dt, max_len=128))


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
