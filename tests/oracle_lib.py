"""ctypes access to the CPU oracle (oracle/librfo.so) and, where it was built, to the
reference driver (oracle/_ref/librfref.so).  Test infrastructure: the side of
the parity tests the CUDA path is compared with, never the thing measured."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")

LEVENSHTEIN, INDEL, LCSSEQ, OSA, JARO, JARO_WINKLER, RATIO, PARTIAL_RATIO = range(8)
TOKEN_SORT_RATIO, PARTIAL_TOKEN_SORT_RATIO, QRATIO = 8, 9, 10
TOKEN_SET_RATIO, PARTIAL_TOKEN_SET_RATIO, TOKEN_RATIO, PARTIAL_TOKEN_RATIO, WRATIO = 11, 12, 13, 14, 15
FUZZ_METRICS = (RATIO, PARTIAL_RATIO, TOKEN_SORT_RATIO, PARTIAL_TOKEN_SORT_RATIO, QRATIO, TOKEN_SET_RATIO,
                PARTIAL_TOKEN_SET_RATIO, TOKEN_RATIO, PARTIAL_TOKEN_RATIO, WRATIO)
DISTANCE, SIMILARITY, NORM_DISTANCE, NORM_SIMILARITY = range(4)
FREE, CACHED, MULTI = range(3)
METRIC_NAMES = ["levenshtein", "indel", "lcsseq", "osa", "jaro", "jaro_winkler", "ratio"]


class Params(ctypes.Structure):
    _fields_ = [("insert_cost", ctypes.c_int64), ("delete_cost", ctypes.c_int64),
                ("replace_cost", ctypes.c_int64), ("prefix_weight", ctypes.c_double)]


class Strings(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("offsets", ctypes.c_void_p),
                ("count", ctypes.c_int64), ("char_width", ctypes.c_int32)]


def result_is_int(metric, op):
    if metric in (JARO, JARO_WINKLER) + FUZZ_METRICS:
        return False
    return op in (DISTANCE, SIMILARITY)


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "all"], check=True)


def _declare_score(fn):
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                   ctypes.POINTER(Params), ctypes.c_uint64, ctypes.c_double,
                   ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)]


_oracle = None
_ref = None


def oracle():
    global _oracle
    if _oracle is None:
        path = os.path.join(ORACLE_DIR, "librfo.so")
        if not os.path.exists(path):
            build_oracle()
        lib = ctypes.CDLL(path)
        _declare_score(lib.rfo_score)
        for name in ("rfo_lcs_exact", "rfo_osa_exact", "rfo_dp_lcs", "rfo_dp_osa"):
            f = getattr(lib, name)
            f.restype = ctypes.c_int64
            f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int] * 2
        for name in ("rfo_levenshtein_exact", "rfo_dp_levenshtein"):
            f = getattr(lib, name)
            f.restype = ctypes.c_int64
            f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int] * 2 + [ctypes.c_int64] * 3
        for name in ("rfo_jaro_counts", "rfo_naive_jaro_counts"):
            f = getattr(lib, name)
            f.restype = None
            f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int] * 2 + [ctypes.POINTER(ctypes.c_int64)] * 2
        lib.rfo_editops.restype = ctypes.c_int
        lib.rfo_editops.argtypes = _EDITOPS_ARGS
        lib.rfo_cdist.restype = ctypes.c_int
        lib.rfo_cdist.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(Strings), ctypes.POINTER(Strings),
                                  ctypes.POINTER(Params), ctypes.c_uint64, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_void_p, ctypes.c_int]
        _oracle = lib
    return _oracle


class EditOp(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("reserved", ctypes.c_int32), ("src_pos", ctypes.c_int64),
                ("dest_pos", ctypes.c_int64)]


_EDITOPS_ARGS = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
                 ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(EditOp), ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]


def editops(lib_fn, metric, s1, s2, score_hint=None):
    """rfo_editops / rfref_editops of one pair -> [(type, src_pos, dest_pos), ...], or None
    where the oracle leaves the pair out (the reference's Hirschberg regime)"""
    a, b = as_units(s1), as_units(s2)
    cap = a.size + b.size + 1
    ops = (EditOp * cap)()
    cnt = ctypes.c_int64()
    args = [metric, _ptr(a), a.size, a.itemsize, _ptr(b), b.size, b.itemsize,
            ctypes.c_uint64(2**64 - 1 if score_hint is None else score_hint)]
    rc = lib_fn(*args, ops, cap, ctypes.byref(cnt))
    if rc == -2:
        return None
    if rc != 0:
        raise ValueError("editops rejected (%d)" % rc)
    return [(ops[k].type, ops[k].src_pos, ops[k].dest_pos) for k in range(cnt.value)]


def reference():
    """The unmodified reference behind a C driver, or None where it was not built."""
    global _ref
    if _ref is None:
        path = os.path.join(ORACLE_DIR, "_ref", "librfref.so")
        if not os.path.exists(path):
            return None
        lib = ctypes.CDLL(path)
        _declare_score(lib.rfref_score)
        lib.rfref_multi.restype = ctypes.c_int
        lib.rfref_multi.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Strings),
                                    ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(Params),
                                    ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.POINTER(ctypes.c_int64)]
        lib.rfref_editops.restype = ctypes.c_int
        lib.rfref_editops.argtypes = _EDITOPS_ARGS
        _ref = lib
    return _ref


def as_units(s, width=None):
    """str / bytes / list of ints -> contiguous numpy array of unsigned code units."""
    if isinstance(s, np.ndarray):
        return np.ascontiguousarray(s)
    if isinstance(s, (bytes, bytearray)):
        return np.frombuffer(bytes(s), dtype=np.uint8).copy()
    if isinstance(s, str):
        cps = [ord(ch) for ch in s]
    else:
        cps = list(s)
    if width is None:
        mx = max(cps) if cps else 0
        width = 1 if mx < 256 else (2 if mx < 65536 else 4)
    return np.array(cps, dtype={1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[width])


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a.size else ctypes.c_void_p(0)


def make_params(weights=(1, 1, 1), prefix_weight=0.1):
    return Params(weights[0], weights[1], weights[2], prefix_weight)


def score(lib_fn, metric, op, form, s1, s2, cutoff=None, weights=(1, 1, 1), prefix_weight=0.1):
    """One scorer call through rfo_score / rfref_score; returns int or float (None if rejected)."""
    a, b = as_units(s1), as_units(s2)
    p = make_params(weights, prefix_weight)
    if result_is_int(metric, op):
        ci = (2**63 - 1 if op == DISTANCE else 0) if cutoff is None else int(cutoff)
        cf = 0.0
    else:
        ci = 0
        if cutoff is None:
            cf = 1.0 if op in (DISTANCE, NORM_DISTANCE) and metric not in FUZZ_METRICS else 0.0
        else:
            cf = float(cutoff)
    oi = ctypes.c_int64(0)
    of = ctypes.c_double(0.0)
    rc = lib_fn(metric, op, form, _ptr(a), a.size, a.itemsize, _ptr(b), b.size, b.itemsize,
                ctypes.byref(p), ci, cf, ctypes.byref(oi), ctypes.byref(of))
    if rc != 0:
        return None
    return oi.value if result_is_int(metric, op) else of.value


def pack_strings(strs, width=None):
    """list of code-unit arrays -> (data ndarray, offsets int64 ndarray, width)."""
    arrs = [as_units(s, width) for s in strs]
    if width is None:
        width = max([a.itemsize for a in arrs] + [1])
    dt = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[width]
    lens = np.array([a.size for a in arrs], dtype=np.int64)
    offsets = np.zeros(len(arrs) + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    data = np.concatenate([a.astype(dt) for a in arrs]) if arrs else np.zeros(0, dt)
    if data.size == 0:
        data = np.zeros(1, dt)
    return data, offsets, width


def strings_struct(data, offsets, width):
    return Strings(data.ctypes.data, offsets.ctypes.data, offsets.size - 1, width)


def oracle_cdist(metric, op, queries, choices, cutoff=None, weights=(1, 1, 1), prefix_weight=0.1,
                 out_dtype=None, nthreads=0):
    """Cached-path cdist on host threads; queries/choices are (data, offsets, width) tuples."""
    lib = oracle()
    qs = strings_struct(*queries)
    cs = strings_struct(*choices)
    p = make_params(weights, prefix_weight)
    is_int = result_is_int(metric, op)
    if out_dtype is None:
        out_dtype = 1 if is_int else 2
    nq, nc = queries[1].size - 1, choices[1].size - 1
    out = np.zeros((nq, nc), dtype={0: np.int32, 1: np.int64, 2: np.float64}[out_dtype])
    if is_int:
        ci = (2**63 - 1 if op == DISTANCE else 0) if cutoff is None else int(cutoff)
        cf = 0.0
    else:
        ci = 0
        cf = (1.0 if op in (DISTANCE, NORM_DISTANCE) else 0.0) if cutoff is None else float(cutoff)
    rc = lib.rfo_cdist(metric, op, ctypes.byref(qs), ctypes.byref(cs), ctypes.byref(p), ci, cf, out_dtype,
                       out.ctypes.data, nthreads)
    if rc != 0:
        raise ValueError("rfo_cdist rejected the arguments")
    return out
