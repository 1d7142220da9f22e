"""ctypes declarations of the C ABI and the generic entry points."""
import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
lib_path = os.path.join(PKG_DIR, "lib", "librapidfuzz_gb300.so")

(LEVENSHTEIN, INDEL, LCSSEQ, OSA, JARO, JARO_WINKLER, RATIO, PARTIAL_RATIO, TOKEN_SORT_RATIO,
 PARTIAL_TOKEN_SORT_RATIO, QRATIO) = range(11)
TOKEN_SET_RATIO, PARTIAL_TOKEN_SET_RATIO, TOKEN_RATIO, PARTIAL_TOKEN_RATIO, WRATIO = range(11, 16)
FUZZ_METRICS = (RATIO, PARTIAL_RATIO, TOKEN_SORT_RATIO, PARTIAL_TOKEN_SORT_RATIO, QRATIO, TOKEN_SET_RATIO,
                PARTIAL_TOKEN_SET_RATIO, TOKEN_RATIO, PARTIAL_TOKEN_RATIO, WRATIO)
DISTANCE, SIMILARITY, NORMALIZED_DISTANCE, NORMALIZED_SIMILARITY = range(4)
FORM_FREE, FORM_CACHED, FORM_MULTI = range(3)
I32, I64, F64 = range(3)
DEVICE_INPUTS, DEVICE_OUTPUT = 1, 2

STATUS = {0: "ok", 1: "invalid argument", 2: "out of range", 3: "CUDA error", 4: "out of memory",
          5: "no device", 6: "device check", 7: "busy"}


class RapidfuzzError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS.get(status, status), message))
        self.status = status


class InvalidArgument(RapidfuzzError, ValueError):
    """the reference throws std::invalid_argument here"""


class Params(ctypes.Structure):
    _fields_ = [("insert_cost", ctypes.c_int64), ("delete_cost", ctypes.c_int64),
                ("replace_cost", ctypes.c_int64), ("prefix_weight", ctypes.c_double)]


class Cutoff(ctypes.Structure):
    _fields_ = [("cutoff_i", ctypes.c_uint64), ("cutoff_f", ctypes.c_double),
                ("hint_i", ctypes.c_uint64), ("hint_f", ctypes.c_double)]


class Strings(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("offsets", ctypes.c_void_p),
                ("count", ctypes.c_int64), ("char_width", ctypes.c_int32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("max_inflight", ctypes.c_int32), ("max_batch", ctypes.c_int32), ("max_device_bytes", ctypes.c_int64)]


class Request(ctypes.Structure):
    _fields_ = [("corpus", ctypes.c_int32), ("metric", ctypes.c_int), ("op", ctypes.c_int), ("params", Params),
                ("cutoff", Cutoff), ("limit", ctypes.c_int32), ("tie_last_wins", ctypes.c_int32),
                ("query", ctypes.c_void_p), ("query_len", ctypes.c_int64), ("query_width", ctypes.c_int32),
                ("out_index", ctypes.c_void_p), ("out_score", ctypes.c_void_p), ("out_count", ctypes.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(lib_path):
            raise ImportError("librapidfuzz_gb300.so is not built (run __graft_entry__.build() or "
                              "python rapidfuzz-cpp_gb300/build.py); there is no CPU fallback")
        L = ctypes.CDLL(lib_path)
        vp, i64, i32, u64, f64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_uint64, ctypes.c_double
        P = ctypes.POINTER
        sig = {
            "rfg_abi_version": ([], ctypes.c_int),
            "rfg_last_error": ([], ctypes.c_char_p),
            "rfg_set_device": ([ctypes.c_int], ctypes.c_int),
            "rfg_synchronize": ([], ctypes.c_int),
            "rfg_score_i64": ([ctypes.c_int, ctypes.c_int, vp, i64, i32, vp, i64, i32, P(Params), u64, u64, P(i64)],
                              ctypes.c_int),
            "rfg_score_f64": ([ctypes.c_int, ctypes.c_int, vp, i64, i32, vp, i64, i32, P(Params), f64, f64, P(f64)],
                              ctypes.c_int),
            "rfg_cached_create": ([ctypes.c_int, vp, i64, i32, P(Params), P(vp)], ctypes.c_int),
            "rfg_cached_destroy": ([vp], ctypes.c_int),
            "rfg_cached_score_i64": ([vp, ctypes.c_int, vp, i64, i32, u64, u64, P(i64)], ctypes.c_int),
            "rfg_cached_score_f64": ([vp, ctypes.c_int, vp, i64, i32, f64, f64, P(f64)], ctypes.c_int),
            "rfg_cached_score_many": ([vp, ctypes.c_int, P(Strings), Cutoff, ctypes.c_int, vp, ctypes.c_uint32],
                                      ctypes.c_int),
            "rfg_cdist": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, P(Strings), P(Strings), P(Params), Cutoff,
                           ctypes.c_int, vp, i64, ctypes.c_uint32], ctypes.c_int),
            "rfg_multi_create": ([ctypes.c_int, i32, ctypes.c_size_t, P(Params), P(vp)], ctypes.c_int),
            "rfg_multi_destroy": ([vp], ctypes.c_int),
            "rfg_multi_insert": ([vp, vp, i64, i32], ctypes.c_int),
            "rfg_multi_result_count": ([vp, P(ctypes.c_size_t)], ctypes.c_int),
            "rfg_multi_score_i64": ([vp, ctypes.c_int, P(i64), ctypes.c_size_t, vp, i64, i32, u64], ctypes.c_int),
            "rfg_multi_score_f64": ([vp, ctypes.c_int, P(f64), ctypes.c_size_t, vp, i64, i32, f64], ctypes.c_int),
            "rfg_batch_create": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, P(Strings), P(Strings), P(Params), Cutoff,
                                  ctypes.c_int, vp, i64, ctypes.c_uint32, P(vp)], ctypes.c_int),
            "rfg_batch_launch": ([vp, vp, ctypes.c_uint32], ctypes.c_int),
            "rfg_batch_check": ([vp, vp], ctypes.c_int),
            "rfg_batch_tune": ([vp, vp, P(i32), P(i64)], ctypes.c_int),
            "rfg_batch_destroy": ([vp], ctypes.c_int),
            "rfg_batch_kernels": ([vp, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
            "rfg_get_stream": ([P(vp)], ctypes.c_int),
            "rfg_corpus_create": ([P(Strings), ctypes.c_uint32, P(vp)], ctypes.c_int),
            "rfg_corpus_destroy": ([vp], ctypes.c_int),
            "rfg_extract": ([vp, ctypes.c_int, ctypes.c_int, P(Strings), P(Params), Cutoff, i32, i32, vp, vp, vp,
                             ctypes.c_uint32], ctypes.c_int),
            "rfg_server_create": ([P(vp), i32, P(ServerConfig), P(vp)], ctypes.c_int),
            "rfg_server_submit": ([vp, P(Request), P(ctypes.c_uint64)], ctypes.c_int),
            "rfg_server_wait": ([vp, ctypes.c_uint64, ctypes.c_double, P(ctypes.c_double)], ctypes.c_int),
            "rfg_testing_fail_device_allocs": ([i64], ctypes.c_int),
            "rfg_testing_band_rounds": ([ctypes.c_int32], ctypes.c_int),
            "rfg_testing_band_mode": ([ctypes.c_int32], ctypes.c_int),
            "rfg_server_stats": ([vp, P(i64), P(i64), P(i64)], ctypes.c_int),
            "rfg_server_destroy": ([vp], ctypes.c_int),
            "rfg_cdist_noalloc": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, P(Strings), P(Strings), i64, P(Params),
                                   Cutoff, ctypes.c_int, vp, i64, vp], ctypes.c_int),
            "rfg_editops": ([ctypes.c_int, P(Strings), P(Strings), u64, vp, i64, vp, ctypes.c_uint32], ctypes.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def check(status):
    if status != 0:
        msg = lib().rfg_last_error().decode(errors="replace")
        if status == 1:
            raise InvalidArgument(status, msg)
        raise RapidfuzzError(status, msg)


def result_is_int(metric, op):
    if metric in (JARO, JARO_WINKLER) or metric in FUZZ_METRICS:
        return False
    return op in (DISTANCE, SIMILARITY)


_DT = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def as_units(s, width=None):
    """str / bytes / sequence of ints / ndarray -> contiguous unsigned code-unit array"""
    if isinstance(s, np.ndarray):
        a = np.ascontiguousarray(s)
        if a.dtype.kind == "i":
            a = a.view({1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.itemsize])
        return a
    if isinstance(s, (bytes, bytearray)):
        return np.frombuffer(bytes(s), dtype=np.uint8).copy()
    cps = [ord(ch) for ch in s] if isinstance(s, str) else list(s)
    if width is None:
        mx = max(cps) if cps else 0
        width = 1 if mx < 256 else (2 if mx < 65536 else 4)
    return np.array(cps, dtype=_DT[width])


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a.size else ctypes.c_void_p(0)


def pack_strings(strs, width=None):
    """list of strings -> (data, int64 offsets, width) for the batch entry points"""
    arrs = [as_units(s) for s in strs]
    if width is None:
        width = max([a.itemsize for a in arrs] + [1])
    dt = _DT[width]
    lens = np.fromiter((a.size for a in arrs), dtype=np.int64, count=len(arrs))
    offsets = np.zeros(len(arrs) + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    data = np.concatenate([a.astype(dt) for a in arrs]) if arrs else np.zeros(0, dt)
    if data.size == 0:
        data = np.zeros(1, dt)
    return data, offsets, width


def make_params(weights=(1, 1, 1), prefix_weight=0.1):
    return Params(int(weights[0]), int(weights[1]), int(weights[2]), float(prefix_weight))


def _default_cutoff(metric, op):
    if result_is_int(metric, op):
        return (2**63 - 1) if op == DISTANCE else 0
    return 1.0 if op in (DISTANCE, NORMALIZED_DISTANCE) and metric not in FUZZ_METRICS else 0.0


def score(metric, op, s1, s2, score_cutoff=None, score_hint=None, weights=(1, 1, 1), prefix_weight=0.1):
    """One call of the reference's free function for (metric, op)."""
    a, b = as_units(s1), as_units(s2)
    p = make_params(weights, prefix_weight)
    c = _default_cutoff(metric, op) if score_cutoff is None else score_cutoff
    if result_is_int(metric, op):
        h = c if score_hint is None else score_hint
        r = ctypes.c_int64()
        check(lib().rfg_score_i64(metric, op, _ptr(a), a.size, a.itemsize, _ptr(b), b.size, b.itemsize,
                                  ctypes.byref(p), int(c), int(h), ctypes.byref(r)))
        return r.value
    h = c if score_hint is None else score_hint
    r = ctypes.c_double()
    check(lib().rfg_score_f64(metric, op, _ptr(a), a.size, a.itemsize, _ptr(b), b.size, b.itemsize,
                              ctypes.byref(p), float(c), float(h), ctypes.byref(r)))
    return r.value


class Cached:
    """A Cached* scorer (s1 lives on the device)."""

    def __init__(self, metric, s1, weights=(1, 1, 1), prefix_weight=0.1):
        self.metric = metric
        self._h = ctypes.c_void_p()
        a = as_units(s1)
        p = make_params(weights, prefix_weight)
        check(lib().rfg_cached_create(metric, _ptr(a), a.size, a.itemsize, ctypes.byref(p), ctypes.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.rfg_cached_destroy(self._h)

    def score(self, op, s2, score_cutoff=None, score_hint=None):
        b = as_units(s2)
        c = _default_cutoff(self.metric, op) if score_cutoff is None else score_cutoff
        h = c if score_hint is None else score_hint
        if result_is_int(self.metric, op):
            r = ctypes.c_int64()
            check(lib().rfg_cached_score_i64(self._h, op, _ptr(b), b.size, b.itemsize, int(c), int(h),
                                             ctypes.byref(r)))
            return r.value
        r = ctypes.c_double()
        check(lib().rfg_cached_score_f64(self._h, op, _ptr(b), b.size, b.itemsize, float(c), float(h),
                                         ctypes.byref(r)))
        return r.value

    def score_many(self, op, choices, score_cutoff=None, out_dtype=None):
        data, offsets, width = choices if isinstance(choices, tuple) else pack_strings(choices)
        c = _default_cutoff(self.metric, op) if score_cutoff is None else score_cutoff
        is_int = result_is_int(self.metric, op)
        if out_dtype is None:
            out_dtype = I64 if is_int else F64
        out = np.empty(offsets.size - 1, dtype={I32: np.int32, I64: np.int64, F64: np.float64}[out_dtype])
        cut = Cutoff(int(c) if is_int else 0, 0.0 if is_int else float(c), 0, 0.0)
        s = Strings(data.ctypes.data, offsets.ctypes.data, offsets.size - 1, width)
        check(lib().rfg_cached_score_many(self._h, op, ctypes.byref(s), cut, out_dtype, out.ctypes.data, 0))
        return out


class Multi:
    """An experimental::Multi* scorer."""

    def __init__(self, metric, max_len, count, weights=(1, 1, 1), prefix_weight=0.1):
        self.metric = metric
        self._h = ctypes.c_void_p()
        p = make_params(weights, prefix_weight)
        check(lib().rfg_multi_create(metric, max_len, count, ctypes.byref(p), ctypes.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.rfg_multi_destroy(self._h)

    def insert(self, s):
        a = as_units(s)
        check(lib().rfg_multi_insert(self._h, _ptr(a), a.size, a.itemsize))

    def result_count(self):
        n = ctypes.c_size_t()
        check(lib().rfg_multi_result_count(self._h, ctypes.byref(n)))
        return n.value

    def score(self, op, s2, score_cutoff=None, score_count=None):
        b = as_units(s2)
        c = _default_cutoff(self.metric, op) if score_cutoff is None else score_cutoff
        n = self.result_count() if score_count is None else score_count
        if result_is_int(self.metric, op):
            out = np.zeros(max(n, 1), dtype=np.int64)
            check(lib().rfg_multi_score_i64(self._h, op, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n,
                                            _ptr(b), b.size, b.itemsize, int(c)))
        else:
            out = np.zeros(max(n, 1), dtype=np.float64)
            check(lib().rfg_multi_score_f64(self._h, op, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n,
                                            _ptr(b), b.size, b.itemsize, float(c)))
        return out[:n]


def cdist(metric, op, queries, choices, score_cutoff=None, weights=(1, 1, 1), prefix_weight=0.1,
          out_dtype=None, form=FORM_CACHED, out=None, flags=0, ld=0):
    """All pairs: out[q, c].  queries/choices: lists of strings, (data, offsets, width)
    numpy tuples, or (data_ptr, offsets_ptr, width, count) device tuples together with
    flags=DEVICE_INPUTS; out may be a device pointer (int) with flags|=DEVICE_OUTPUT."""
    q = _batch(queries)
    ch = _batch(choices)
    is_int = result_is_int(metric, op)
    if out_dtype is None:
        out_dtype = I64 if is_int else F64
    c = _default_cutoff(metric, op) if score_cutoff is None else score_cutoff
    cut = Cutoff(int(c) if is_int else 0, 0.0 if is_int else float(c), 0, 0.0)
    if out is None:
        out = np.empty((q.count, ch.count), dtype={I32: np.int32, I64: np.int64, F64: np.float64}[out_dtype])
    p = make_params(weights, prefix_weight)
    out_addr = out if isinstance(out, int) else out.ctypes.data
    check(lib().rfg_cdist(metric, op, form, ctypes.byref(q), ctypes.byref(ch), ctypes.byref(p), cut, out_dtype,
                          out_addr, ld, flags))
    return out


def _batch(b):
    if isinstance(b, tuple) and len(b) == 4:  # device pointers
        return Strings(b[0], b[1], b[3], b[2])
    data, offsets, width = b if isinstance(b, tuple) else pack_strings(b)
    s = Strings(data.ctypes.data, offsets.ctypes.data, offsets.size - 1, width)
    s._keep = (data, offsets)
    return s


LAUNCH_GRAPH = 1


class Batch:
    """A prepared cdist (rfg_batch_*): launch() only enqueues kernels on a stream."""

    def __init__(self, metric, op, queries, choices, out_ptr, score_cutoff=None, weights=(1, 1, 1),
                 prefix_weight=0.1, out_dtype=None, form=FORM_CACHED, flags=0, ld=0):
        self._h = ctypes.c_void_p()
        q, ch = _batch(queries), _batch(choices)
        self._keep = (q, ch)
        is_int = result_is_int(metric, op)
        if out_dtype is None:
            out_dtype = I64 if is_int else F64
        c = _default_cutoff(metric, op) if score_cutoff is None else score_cutoff
        cut = Cutoff(int(c) if is_int else 0, 0.0 if is_int else float(c), 0, 0.0)
        p = make_params(weights, prefix_weight)
        check(lib().rfg_batch_create(metric, op, form, ctypes.byref(q), ctypes.byref(ch), ctypes.byref(p), cut,
                                     out_dtype, out_ptr, ld, flags, ctypes.byref(self._h)))

    def launch(self, stream=0, graph=True):
        check(lib().rfg_batch_launch(self._h, stream, LAUNCH_GRAPH if graph else 0))

    def check(self, stream=0):
        check(lib().rfg_batch_check(self._h, stream))

    def tune(self, stream=0):
        b, t = ctypes.c_int32(), ctypes.c_int64()
        check(lib().rfg_batch_tune(self._h, stream, ctypes.byref(b), ctypes.byref(t)))
        return b.value, t.value

    def kernels(self):
        """names of the kernels one launch runs"""
        buf = ctypes.create_string_buffer(4096)
        check(lib().rfg_batch_kernels(self._h, buf, len(buf)))
        return [k for k in buf.value.decode().split(";") if k]

    def close(self):
        if self._h and self._h.value:
            lib().rfg_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        if _lib is not None:
            self.close()


def library_stream():
    s = ctypes.c_void_p()
    check(lib().rfg_get_stream(ctypes.byref(s)))
    return s.value or 0


class Corpus:
    """A device-resident choice list for repeated extract calls (rfg_corpus_*)."""

    def __init__(self, choices, flags=0):
        self._h = ctypes.c_void_p()
        self._b = _batch(choices)
        self.count = self._b.count
        check(lib().rfg_corpus_create(ctypes.byref(self._b), flags, ctypes.byref(self._h)))

    def extract(self, metric, op, queries, limit=5, score_cutoff=None, tie_last=False, weights=(1, 1, 1),
                prefix_weight=0.1):
        """-> (index int64 [nq, limit], score float64 [nq, limit], count int32 [nq]), best first"""
        q = _batch(queries)
        is_int = result_is_int(metric, op)
        c = _default_cutoff(metric, op) if score_cutoff is None else score_cutoff
        cut = Cutoff(int(c) if is_int else 0, 0.0 if is_int else float(c), 0, 0.0)
        idx = np.full((q.count, limit), -1, dtype=np.int64)
        sc = np.zeros((q.count, limit), dtype=np.float64)
        cnt = np.zeros(q.count, dtype=np.int32)
        p = make_params(weights, prefix_weight)
        check(lib().rfg_extract(self._h, metric, op, ctypes.byref(q), ctypes.byref(p), cut, limit, int(tie_last),
                                idx.ctypes.data, sc.ctypes.data, cnt.ctypes.data, 0))
        return idx, sc, cnt

    def close(self):
        if self._h and self._h.value:
            lib().rfg_corpus_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        if _lib is not None:
            self.close()


class Server:
    """Continuous-batching extract service (rfg_server_*)."""

    def __init__(self, corpora, max_inflight=4, max_batch=64, max_device_bytes=0):
        self._corpora = list(corpora)
        arr = (ctypes.c_void_p * len(self._corpora))(*[c._h.value for c in self._corpora])
        cfg = ServerConfig(max_inflight, max_batch, max_device_bytes)
        self._h = ctypes.c_void_p()
        check(lib().rfg_server_create(arr, len(self._corpora), ctypes.byref(cfg), ctypes.byref(self._h)))
        self._pending = {}

    def submit(self, corpus, metric, op, query, limit=1, score_cutoff=None, tie_last=None, weights=(1, 1, 1),
               prefix_weight=0.1):
        q = as_units(query)
        is_int = result_is_int(metric, op)
        c = _default_cutoff(metric, op) if score_cutoff is None else score_cutoff
        idx = np.full(limit, -1, dtype=np.int64)
        sc = np.zeros(limit, dtype=np.float64)
        cnt = np.zeros(1, dtype=np.int32)
        r = Request(corpus, metric, op, make_params(weights, prefix_weight),
                    Cutoff(int(c) if is_int else 0, 0.0 if is_int else float(c), 0, 0.0), limit,
                    int(limit == 1 if tie_last is None else tie_last), q.ctypes.data if q.size else None, q.size,
                    q.itemsize, idx.ctypes.data, sc.ctypes.data, cnt.ctypes.data)
        t = ctypes.c_uint64()
        check(lib().rfg_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)))
        self._pending[t.value] = (idx, sc, cnt)
        return t.value

    def wait(self, ticket, timeout=600.0):
        lat = ctypes.c_double()
        check(lib().rfg_server_wait(self._h, ticket, timeout, ctypes.byref(lat)))
        idx, sc, cnt = self._pending.pop(ticket)
        n = int(cnt[0])
        return idx[:n], sc[:n], lat.value

    def stats(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().rfg_server_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"completed": a.value, "batches": b.value, "batched_requests": c.value}

    def close(self):
        if self._h and self._h.value:
            lib().rfg_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        if _lib is not None:
            self.close()


EDITOP_DTYPE = np.dtype([("type", np.int32), ("reserved", np.int32), ("src_pos", np.int64), ("dest_pos", np.int64)])


class EditopsBatch:
    """the operations of many pairs: ops (structured array type / src_pos / dest_pos),
    offsets (pair i owns ops[offsets[i]:offsets[i + 1]]); indexing gives one pair's slice"""

    def __init__(self, ops, offsets):
        self.ops = ops
        self.offsets = offsets

    def __len__(self):
        return self.offsets.size - 1

    def __getitem__(self, i):
        if not -len(self) <= i < len(self):
            raise IndexError(i)
        i %= len(self)
        return self.ops[self.offsets[i]:self.offsets[i + 1]]

    def __iter__(self):
        return (self[i] for i in range(len(self)))


def editops_many(metric, s1s, s2s, score_hint=None):
    """rfg_editops: editops of the pairs (s1s[i], s2s[i]) -> EditopsBatch"""
    p1 = s1s if isinstance(s1s, tuple) else pack_strings(s1s)
    p2 = s2s if isinstance(s2s, tuple) else pack_strings(s2s)
    a, b = _batch(p1), _batch(p2)
    cap = int(p1[1][-1] - p1[1][0] + p2[1][-1] - p2[1][0])
    ops = np.zeros(max(cap, 1), dtype=EDITOP_DTYPE)
    offsets = np.zeros(a.count + 1, dtype=np.int64)
    hint = 2**64 - 1 if score_hint is None else int(score_hint)
    check(lib().rfg_editops(metric, ctypes.byref(a), ctypes.byref(b), hint, ops.ctypes.data, cap,
                            offsets.ctypes.data, 0))
    return EditopsBatch(ops[:offsets[-1]], offsets)
