"""The C-ABI library: builds, loads, exports every symbol include/rapidfuzz_gb300.h
declares, and rejects bad arguments the way the reference throws std::invalid_argument.
No compute call runs here without a GPU.  CPU only."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _built_lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("rfg_build", os.path.join(ROOT, "rapidfuzz-cpp_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def declared_symbols():
    with open(os.path.join(ROOT, "include", "rapidfuzz_gb300.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rfg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    path = _built_lib()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 18
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_abi_version():
    import rapidfuzz_gb300 as R
    _built_lib()
    assert R.lib().rfg_abi_version() == 1


def test_invalid_arguments_are_rejected_before_the_device():
    import rapidfuzz_gb300 as R
    _built_lib()
    L = R.lib()
    a = np.frombuffer(b"abc", dtype=np.uint8)
    p = R._lib.make_params()
    r = ctypes.c_int64()
    f = ctypes.c_double()
    # ratio has no distance (fuzz.hpp:44-48)
    assert L.rfg_score_f64(R.RATIO, R.DISTANCE, a.ctypes.data, 3, 1, a.ctypes.data, 3, 1, ctypes.byref(p), 0.0,
                           0.0, ctypes.byref(f)) == 1
    # bad char width
    assert L.rfg_score_i64(R.LEVENSHTEIN, R.DISTANCE, a.ctypes.data, 3, 3, a.ctypes.data, 3, 1, ctypes.byref(p), 5,
                           5, ctypes.byref(r)) == 1
    # integer overload on a double result
    assert L.rfg_score_i64(R.JARO, R.SIMILARITY, a.ctypes.data, 3, 1, a.ctypes.data, 3, 1, ctypes.byref(p), 0, 0,
                           ctypes.byref(r)) == 1
    # MultiLevenshtein weight check (Levenshtein.hpp:338-339)
    h = ctypes.c_void_p()
    bad = R._lib.make_params((2, 1, 1))
    assert L.rfg_multi_create(R.LEVENSHTEIN, 64, 4, ctypes.byref(bad), ctypes.byref(h)) == 1
    assert b"unsupported weights" in L.rfg_last_error()
    # MaxLen must be 8/16/32/64
    assert L.rfg_multi_create(R.JARO, 12, 4, ctypes.byref(p), ctypes.byref(h)) == 1
    # out-of-bounds insert (Levenshtein.hpp:372) and short score buffer (:387-388)
    assert L.rfg_multi_create(R.OSA, 8, 1, ctypes.byref(p), ctypes.byref(h)) == 0
    assert L.rfg_multi_insert(h, a.ctypes.data, 3, 1) == 0
    assert L.rfg_multi_insert(h, a.ctypes.data, 3, 1) == 1
    assert b"out of bounds insert" in L.rfg_last_error()
    n = ctypes.c_size_t()
    assert L.rfg_multi_result_count(h, ctypes.byref(n)) == 0 and n.value == 32
    out = np.zeros(4, dtype=np.int64)
    assert L.rfg_multi_score_i64(h, R.DISTANCE, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), 4,
                                 a.ctypes.data, 3, 1, 10) == 1
    assert b"result_count" in L.rfg_last_error()
    L.rfg_multi_destroy(h)
    # cdist: double results need RFG_F64
    from rapidfuzz_gb300._lib import Strings, Cutoff
    off = np.array([0, 3], dtype=np.int64)
    s = Strings(a.ctypes.data, off.ctypes.data, 1, 1)
    o = np.zeros(1, dtype=np.int32)
    assert L.rfg_cdist(R.JARO_WINKLER, R.SIMILARITY, R.FORM_CACHED, ctypes.byref(s), ctypes.byref(s),
                       ctypes.byref(p), Cutoff(0, 0.0, 0, 0.0), R.I32, o.ctypes.data, 0, 0) == 1


def test_no_cpu_fallback_without_a_device():
    """without a GPU a valid call fails loudly instead of computing on the CPU"""
    import rapidfuzz_gb300 as R
    _built_lib()
    n = ctypes.c_int()
    cudart_has_device = False
    try:
        import torch
        cudart_has_device = torch.cuda.is_available()
    except Exception:
        pass
    if cudart_has_device:
        pytest.skip("a GPU is present")
    with pytest.raises(R.RapidfuzzError) as e:
        R.levenshtein_distance("abc", "abd")
    assert e.value.status == 5


def test_reference_names_are_mirrored():
    """every scorer name of the reference's public API has its mirror in the Python package
    (rapidfuzz/distance/*.hpp, rapidfuzz/fuzz.hpp, rapidfuzz/details/types.hpp); no call"""
    import rapidfuzz_gb300 as R
    for prefix in ("levenshtein", "indel", "lcs_seq", "osa", "jaro", "jaro_winkler"):
        for op in ("distance", "similarity", "normalized_distance", "normalized_similarity"):
            assert callable(getattr(R, "%s_%s" % (prefix, op)))
    for name in ("ratio", "partial_ratio", "token_sort_ratio", "partial_token_sort_ratio", "token_set_ratio",
                 "partial_token_set_ratio", "token_ratio", "partial_token_ratio", "WRatio", "QRatio"):
        assert callable(getattr(R, "fuzz_" + name))
    for name in ("CachedLevenshtein", "CachedIndel", "CachedLCSseq", "CachedOSA", "CachedJaro", "CachedJaroWinkler",
                 "CachedRatio", "CachedPartialRatio", "CachedTokenSortRatio", "CachedPartialTokenSortRatio",
                 "CachedTokenSetRatio", "CachedPartialTokenSetRatio", "CachedTokenRatio", "CachedPartialTokenRatio",
                 "CachedWRatio", "CachedQRatio"):
        assert isinstance(getattr(R, name), type)
    for name in ("MultiLevenshtein", "MultiIndel", "MultiLCSseq", "MultiOSA", "MultiJaro", "MultiJaroWinkler",
                 "MultiRatio", "MultiTokenSortRatio", "MultiQRatio"):
        assert isinstance(getattr(R.experimental, name), type)
    for name in ("levenshtein_editops", "indel_editops", "lcs_seq_editops"):
        assert callable(getattr(R, name))
    e = R.Editops([R.EditOp(2, 0, 0), R.EditOp(1, 3, 4)], 5, 6)
    oc = e.as_opcodes()
    assert list(oc.as_editops()) == list(e) and oc.src_len == 5 and oc.dest_len == 6
    assert "".join(e.apply("abcde", "xabcyz")[:1]) == "x"
    for name in ("slice", "remove_slice", "reverse", "inverse", "remove_subsequence"):
        assert callable(getattr(e, name))
    for name in ("slice", "reverse", "inverse"):
        assert callable(getattr(oc, name))
    assert e.inverse().inverse() == e and e.reverse().reverse() == e


@pytest.mark.parametrize("std", ["c++11", "c++17"])
def test_cpp_dropin_compiles(std):
    """the C++ drop-in header and its caller compile (run on the GPU in test_gpu_cpp_api.py)"""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("no g++")
    cmd = ["g++", "-std=" + std, "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "rapidfuzz-cpp_gb300", "include"), "-I", os.path.join(ROOT, "oracle"),
           os.path.join(ROOT, "tests", "cpp", "test_api.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
