"""Host-side failure handling (no GPU needed): string batches with broken offsets are
refused with RFG_ERR_INVALID_ARGUMENT -- the reference's std::invalid_argument -- before
the library touches a device, for the batch entry points that take host strings
(rfg_cdist, rfg_batch_create, rfg_corpus_create); the allocation-failure injection the
GPU failure tests use is exported.  CPU only."""
import ctypes
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def R():
    import importlib.util
    spec = importlib.util.spec_from_file_location("rfg_build", os.path.join(ROOT, "rapidfuzz-cpp_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import rapidfuzz_gb300
    return rapidfuzz_gb300


BAD_OFFSETS = {
    "decreasing": [0, 3, 2, 5],
    "negative start": [-1, 2, 4, 5],
    "longer than 2^31": [0, 1, 2, 2 + 2**31],
}


def _strings(R, off):
    from rapidfuzz_gb300._lib import Strings
    off = np.asarray(off, dtype=np.int64)
    data = np.zeros(16, dtype=np.uint8)
    s = Strings(data.ctypes.data, off.ctypes.data, off.size - 1, 1)
    s._keep = (data, off)
    return s


@pytest.mark.parametrize("which", sorted(BAD_OFFSETS))
def test_bad_offsets_are_refused_before_the_device(R, which):
    from rapidfuzz_gb300._lib import Cutoff, make_params
    L = R.lib()
    good = _strings(R, [0, 1, 2, 3])
    bad = _strings(R, BAD_OFFSETS[which])
    p = make_params()
    cut = Cutoff(8, 0.0, 0, 0.0)
    out = np.zeros(16, dtype=np.int64)
    for q, c in ((bad, good), (good, bad)):
        assert L.rfg_cdist(R.LEVENSHTEIN, R.DISTANCE, R.FORM_CACHED, ctypes.byref(q), ctypes.byref(c), ctypes.byref(p),
                           cut, R.I64, out.ctypes.data, 0, 0) == 1, which
        assert b"offsets" in L.rfg_last_error()
        h = ctypes.c_void_p()
        assert L.rfg_batch_create(R.OSA, R.DISTANCE, R.FORM_CACHED, ctypes.byref(q), ctypes.byref(c), ctypes.byref(p),
                                  cut, R.I64, out.ctypes.data, 0, 0, ctypes.byref(h)) == 1, which
        assert not h.value
    h = ctypes.c_void_p()
    assert L.rfg_corpus_create(ctypes.byref(bad), 0, ctypes.byref(h)) == 1
    assert not h.value


def test_allocation_failure_injection_is_exported(R):
    L = R.lib()
    assert L.rfg_testing_fail_device_allocs(3) == 0
    assert L.rfg_testing_fail_device_allocs(-1) == 0
