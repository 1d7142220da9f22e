"""The other benchmark configurations of bench.py (--workload dna1x100k | dna256x65536 | tokens1024x1m); each
prints one JSON line like the headline workload.

dna1x100k  Levenshtein (no cutoff), 1 query x 100,000 DNA choices len U[8,64], int64: the
      batched launch (prepared batch, device-resident) against the plain per-call path
      (rfg_cached_score_i64, one H2D + launch + D2H per choice, timed on a sample) and the
      CPU port (Cached* loop, all host threads).
dna256x65536  Levenshtein normalized_distance with score_cutoff 0.1 (cutoff = 10 % of the longer
      string), 256 x 65,536 DNA strings, lengths log-normal(300, 0.6) in [100, 2000], each
      choice unrelated or a query mutated at 1-15 %: multi-word and banded kernels.
dna256x65536_indel  the same strings under Indel normalized_distance with score_cutoff 0.1
      (10 % of m + n): the banded LCS kernels, timed beside the unbanded multi-word cores.
tokens1024x1m  Jaro-Winkler (prefix_weight 0.1, cutoff 0.85) and fuzz::ratio (cutoff 85) over uint32
      code-point token strings, 1,024 x 1,000,000, dense float64 outputs kept on the device.
partial  fuzz::partial_ratio (cutoff 80) of 256 token queries against 200,000 token strings
      (uint32, as in tokens1024x1m), dense float64 out on the device (the first widening of the path).
tokens   token_sort_ratio, QRatio, WRatio and token_set_ratio (cutoff 80), 256 x 200,000 token
      strings, host inputs and host results through rfg_cdist (joins / parts on the host threads).
editops  levenshtein_editops of 200,000 DNA pairs (len U[8,64], 0-5 edits) through rfg_editops.
serving  serving: device-resident corpora of 10,000,000 DNA strings (len U[10,200]) and
      1,000,000 uint32 token strings; Poisson arrivals (--rate req/s for --duration s), each
      an extractOne (limit 1) or top-10 extract of one query of length U[5,500] with a metric
      drawn from {Levenshtein, Indel, OSA} (DNA corpus) or Jaro-Winkler (token corpus);
      continuous batching (rfg_server); p50/p99 submit-to-result latency and pairs/s, beside
      the same requests run one at a time (rfg_extract).
"""
import json
import os
import time

import numpy as np

import bench as B

METRIC = B.METRIC_NAME


def _timed_batches(torch, batches, stream, steps, warmup, flush):
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            for b in batches:
                b.launch(stream.cuda_stream, graph=True)
        for b in batches:
            b.check(stream.cuda_stream)
    torch.cuda.synchronize()
    clocks = B.ClockSampler()
    clocks.start()
    time.sleep(0.3)
    per = [0.0] * len(batches)
    total = 0.0
    with torch.cuda.stream(stream):
        for _ in range(steps):
            flush.zero_()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in batches]
            for (e0, e1), b in zip(ev, batches):
                e0.record(stream)
                b.launch(stream.cuda_stream, graph=True)
                e1.record(stream)
            stream.synchronize()
            for i, (e0, e1) in enumerate(ev):
                per[i] += e0.elapsed_time(e1)
            total += ev[0][0].elapsed_time(ev[-1][1])
    torch.cuda.synchronize()
    return total / 1e3, [p / steps for p in per], clocks.stop(torch.cuda.current_device())


def _dev(torch, batch, dev):
    d, o, w = batch
    td = torch.from_numpy(np.ascontiguousarray(d)).to(dev)
    to = torch.from_numpy(np.ascontiguousarray(o)).to(dev)
    return (td.data_ptr(), to.data_ptr(), w, o.size - 1), (td, to)


def band_steps(q, c, op, ci, cf, metric=0):
    """word steps of the band kernels on one-byte strings (librfg_count.so); metric in the
    scorer enum (0 Levenshtein, 1 Indel, 2 LCSseq, 6 ratio)"""
    import ctypes
    lib = ctypes.CDLL(os.path.join(B.ROOT, "rapidfuzz-cpp_gb300", "lib", "librfg_count.so"))
    vp, u64p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)
    lib.rfg_count_band_steps.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_double, vp, vp, ctypes.c_int64, vp,
                                         vp, ctypes.c_int64, ctypes.c_int, u64p, u64p, u64p]
    e, a, p = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    rc = lib.rfg_count_band_steps(metric, op, ci, cf, q[0].ctypes.data, q[1].ctypes.data, len(q[1]) - 1, c[0].ctypes.data,
                                  c[1].ctypes.data, len(c[1]) - 1, 0, ctypes.byref(e), ctypes.byref(a), ctypes.byref(p))
    if rc != 0:
        raise RuntimeError("band step count failed")
    return {"exec_words": float(e.value), "alg_words": float(a.value), "pairs": int(p.value)}


def _cells(q, c):
    ql = np.diff(q[1]).astype(np.float64)
    cl = np.diff(c[1]).astype(np.float64)
    return float(ql.sum()) * float(cl.sum())


def run(args, rank, world, local):
    import torch
    import rapidfuzz_gb300 as R
    import workloads as WL
    from oracle_lib import oracle_cdist
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    steps, warmup = args.steps, args.warmup
    line = {"metric": METRIC, "unit": "GCUPS", "n_gpus": 1, "steps": steps, "warmup": warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic (seeded)"}
    if args.workload == "dna1x100k":
        q = WL.dna_uniform(seed=11, n=1)
        c = WL.dna_uniform(seed=12, n=100000)
        nq, nc = 1, 100000
        cells = _cells(q, c)
        qd, kq = _dev(torch, q, dev)
        cd, kc = _dev(torch, c, dev)
        out = torch.empty((nq, nc), dtype=torch.int64, device=dev)
        b = R.Batch(R.LEVENSHTEIN, R.DISTANCE, qd, cd, out.data_ptr(), None, out_dtype=R.I64, flags=R.DEVICE_INPUTS)
        b.tune(stream.cuda_stream)
        t, per, clk = _timed_batches(torch, [b], stream, steps, warmup, flush)
        batched_pairs = nc * steps / t
        exp = oracle_cdist(R.LEVENSHTEIN, R.DISTANCE, q, c)
        assert np.array_equal(out.cpu().numpy(), exp), "dna1x100k parity"
        # plain per-call GPU path: one Cached* call per choice
        qs = q[0][:q[1][1]]
        sc = R.Cached(R.LEVENSHTEIN, qs)
        strs = [c[0][c[1][i]:c[1][i + 1]] for i in range(2000)]
        for s2 in strs[:50]:
            sc.score(R.DISTANCE, s2)
        t0 = time.perf_counter()
        vals = [sc.score(R.DISTANCE, s2) for s2 in strs]
        tp = time.perf_counter() - t0
        assert vals == exp[0, :2000].tolist()
        percall_pairs = len(strs) / tp
        # e2e of the batched path from host buffers (Cached scorer over all choices)
        for _ in range(2):
            sc.score_many(R.DISTANCE, c)
        t0 = time.perf_counter()
        for _ in range(steps):
            sc.score_many(R.DISTANCE, c)
        te = time.perf_counter() - t0
        tc0 = time.perf_counter()
        oracle_cdist(R.LEVENSHTEIN, R.DISTANCE, q, c)
        tc = time.perf_counter() - tc0
        tc1 = time.perf_counter()
        oracle_cdist(R.LEVENSHTEIN, R.DISTANCE, q, c, nthreads=1)
        tc1 = time.perf_counter() - tc1
        line.update({"value": cells * steps / t / 1e9, "ms_per_step": t / steps * 1e3, "dtype": "u64",
                     "config": {"workload": "dna1x100k: Levenshtein, 1 query x 100,000 DNA len U[8,64], no cutoff, int64",
                                "pairs_per_s_batched": batched_pairs, "pairs_per_s_per_call_gpu": percall_pairs,
                                "batched_over_per_call": batched_pairs / percall_pairs,
                                "per_call_us": tp / len(strs) * 1e6,
                                "cpu_pairs_per_s_all_cores": nc / tc, "cpu_pairs_per_s_1_core": nc / tc1},
                     "e2e": {"value": cells * steps / te / 1e9, "unit": "GCUPS",
                             "h2d_bytes_per_step": int(c[0].nbytes + c[1].nbytes), "d2h_bytes_per_step": nc * 8,
                             "pairs_per_s": nc * steps / te},
                     "cpu_baseline": {"value": cells / tc / 1e9, "unit": "GCUPS", "cores": os.cpu_count(),
                                      "kind": "port", "sample": "the full 1 x 100k workload"},
                     "gpu_launches": steps, "clocks": clk})
    elif args.workload == "dna256x65536":
        q, c = WL.dna_lognormal(seed=13, nq=256, nc=65536)
        nq, nc = 256, 65536
        cells = _cells(q, c)
        qd, kq = _dev(torch, q, dev)
        cd, kc = _dev(torch, c, dev)
        out = torch.empty((nq, nc), dtype=torch.float64, device=dev)
        b = R.Batch(R.LEVENSHTEIN, R.NORMALIZED_DISTANCE, qd, cd, out.data_ptr(), 0.1, out_dtype=R.F64,
                    flags=R.DEVICE_INPUTS)
        if not args.no_tune:
            b.tune(stream.cuda_stream)
        t, per, clk = _timed_batches(torch, [b], stream, steps, warmup, flush)
        # every element of the timed batch's result against the oracle (outside the timed region)
        exp = oracle_cdist(R.LEVENSHTEIN, R.NORMALIZED_DISTANCE, q, c, 0.1)
        assert np.array_equal(out.cpu().numpy().view(np.int64), exp.view(np.int64)), "dna256x65536 parity"
        tc0 = time.perf_counter()
        sub = 16
        qsub = (q[0][:q[1][sub]], q[1][:sub + 1].copy(), 1)
        oracle_cdist(R.LEVENSHTEIN, R.NORMALIZED_DISTANCE, qsub, c, 0.1)
        tc = time.perf_counter() - tc0
        # roofline of the band kernels: the 32-bit word steps Ukkonen's band of every pair
        # needs (counted on the host by the same core), 13 INT32 operations each (the
        # 32-bit-word form of the Levenshtein step: Levenshtein_impl.hpp:285-302)
        band = band_steps(q, c, 2, 0, 0.1)
        peak = B.int_peak_ops()
        ach = band["alg_words"] * 13 / (t / steps)
        roofline = {"bound": "int32", "achieved": ach / 1e12, "peak": peak / 1e12, "unit": "Tops/s",
                    "frac": ach / peak, "traffic": None, "kernel": ";".join(b.kernels()),
                    "peak_source": "measured: LOP3/IADD3/SHF issue-rate microbenchmark (librfg_peak.so)",
                    "ops_per_word_step_32": 13, "band_pairs": band["pairs"],
                    "alg_word_steps_32": band["alg_words"], "exec_word_steps_32": band["exec_words"]}
        line.update({"value": cells * steps / t / 1e9, "ms_per_step": t / steps * 1e3, "dtype": "u64",
                     "config": {"workload": "dna256x65536: Levenshtein normalized_distance cutoff 0.1, 256 x 65,536 DNA "
                                            "lognormal(300,0.6) in [100,2000], half mutated 1-15%",
                                "pairs_per_s": nq * nc * steps / t, "kernels": b.kernels()},
                     "cpu_baseline": {"value": _cells(qsub, c) / tc / 1e9, "unit": "GCUPS", "cores": os.cpu_count(),
                                      "kind": "port", "sample": "16 of the 256 queries x all 65,536 choices"},
                     "roofline": roofline, "e2e": None, "gpu_launches": steps * len(b.kernels()), "clocks": clk})
    elif args.workload == "dna256x65536_indel":
        q, c = WL.dna_lognormal(seed=13, nq=256, nc=65536)
        nq, nc = 256, 65536
        cells = _cells(q, c)
        qd, kq = _dev(torch, q, dev)
        cd, kc = _dev(torch, c, dev)
        out = torch.empty((nq, nc), dtype=torch.float64, device=dev)
        lib = R.lib()
        times = {}
        try:
            # the same batch with the band kernels and on the unbanded multi-word cores
            for mode in (0, 1):
                assert lib.rfg_testing_band_mode(mode) == 0
                b = R.Batch(R.INDEL, R.NORMALIZED_DISTANCE, qd, cd, out.data_ptr(), 0.1, out_dtype=R.F64,
                            flags=R.DEVICE_INPUTS)
                t, per, clk = _timed_batches(torch, [b], stream, steps, warmup, flush)
                times[mode] = (t, b.kernels(), clk)
                if mode == 0:
                    b.close()
        finally:
            lib.rfg_testing_band_mode(1)
        t, kernels, clk = times[1]
        exp = oracle_cdist(R.INDEL, R.NORMALIZED_DISTANCE, q, c, 0.1)
        assert np.array_equal(out.cpu().numpy().view(np.int64), exp.view(np.int64)), "dna256x65536 Indel parity"
        b.close()
        tc0 = time.perf_counter()
        sub = 16
        qsub = (q[0][:q[1][sub]], q[1][:sub + 1].copy(), 1)
        oracle_cdist(R.INDEL, R.NORMALIZED_DISTANCE, qsub, c, 0.1)
        tc = time.perf_counter() - tc0
        # roofline of the LCS band kernels: the 32-bit word steps Ukkonen's band of every
        # pair needs (counted on the host by the same core), 4 INT32 operations each (the
        # 32-bit-word form of the LCS step: LCSseq_impl.hpp:226-229)
        band = band_steps(q, c, 2, 0, 0.1, metric=1)
        peak = B.int_peak_ops()
        ach = band["alg_words"] * 4 / (t / steps)
        roofline = {"bound": "int32", "achieved": ach / 1e12, "peak": peak / 1e12, "unit": "Tops/s",
                    "frac": ach / peak, "traffic": None, "kernel": ";".join(kernels),
                    "peak_source": "measured: LOP3/IADD3/SHF issue-rate microbenchmark (librfg_peak.so)",
                    "ops_per_word_step_32": 4, "band_pairs": band["pairs"],
                    "alg_word_steps_32": band["alg_words"], "exec_word_steps_32": band["exec_words"]}
        line.update({"value": cells * steps / t / 1e9, "ms_per_step": t / steps * 1e3, "dtype": "u64",
                     "config": {"workload": "dna256x65536: Indel normalized_distance cutoff 0.1, 256 x 65,536 DNA "
                                            "lognormal(300,0.6) in [100,2000], half mutated 1-15%",
                                "pairs_per_s": nq * nc * steps / t, "kernels": kernels,
                                "ms_per_step_unbanded": times[0][0] / steps * 1e3,
                                "kernels_unbanded": times[0][1],
                                "band_speedup": times[0][0] / t},
                     "cpu_baseline": {"value": _cells(qsub, c) / tc / 1e9, "unit": "GCUPS", "cores": os.cpu_count(),
                                      "kind": "port", "sample": "16 of the 256 queries x all 65,536 choices"},
                     "roofline": roofline, "e2e": None, "gpu_launches": steps * len(kernels), "clocks": clk})
    elif args.workload == "serving":
        return run_serving(args, R, WL)
    elif args.workload == "tokens":
        nq = 256
        nc = args.nc if args.nc != 4096 else 200000
        (q, ql) = WL.tokens_u32(seed=43, n=nq)
        c = WL.tokens_u32_fast(seed=44, n=nc)
        per, per_fresh = {}, {}
        # the e2e contract: pinned host buffers in and out (as the cdist headline); the
        # plain R.cdist call, which allocates a fresh pageable result, is timed beside it
        def pinned(a):
            return torch.from_numpy(a).pin_memory().numpy()
        qp = (pinned(q[0]), pinned(q[1]), q[2])
        cp = (pinned(c[0]), pinned(c[1]), c[2])
        outp = torch.empty((nq, nc), dtype=torch.float64).pin_memory().numpy()
        clocks = B.ClockSampler()
        clocks.start()
        rows = [0, 100, 255]
        qrows = (np.concatenate([q[0][q[1][r]:q[1][r + 1]] for r in rows]),
                 np.concatenate([[0], np.cumsum([q[1][r + 1] - q[1][r] for r in rows])]).astype(np.int64), 4)
        for name, m in (("token_sort_ratio", R.TOKEN_SORT_RATIO), ("QRatio", R.QRATIO), ("WRatio", R.WRATIO),
                        ("token_set_ratio", R.TOKEN_SET_RATIO)):
            for _ in range(warmup):
                R.cdist(m, R.SIMILARITY, qp, cp, 80.0, out=outp)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(steps):
                R.cdist(m, R.SIMILARITY, qp, cp, 80.0, out=outp)
            per[name] = (time.perf_counter() - t0) / steps
            exp = oracle_cdist(m, R.SIMILARITY, qrows, c, 80.0)
            assert np.array_equal(outp[rows].view(np.int64), exp.view(np.int64)), name + " parity"
            for _ in range(min(warmup, 2)):
                out = R.cdist(m, R.SIMILARITY, q, c, 80.0)
            t0 = time.perf_counter()
            for _ in range(steps):
                out = R.cdist(m, R.SIMILARITY, q, c, 80.0)
            per_fresh[name] = (time.perf_counter() - t0) / steps
            assert np.array_equal(out[rows].view(np.int64), exp.view(np.int64)), name + " parity"
        clk = clocks.stop(torch.cuda.current_device())
        sub = 8
        qsub = (q[0][:q[1][sub]], q[1][:sub + 1].copy(), 4)
        tc0 = time.perf_counter()
        oracle_cdist(R.TOKEN_SORT_RATIO, R.SIMILARITY, qsub, c, 80.0)
        tc = time.perf_counter() - tc0
        t = per["token_sort_ratio"]
        h2d = int(q[0].nbytes + q[1].nbytes + c[0].nbytes + c[1].nbytes)
        line.update({"value": nq * nc / t, "unit": "pairs/s", "ms_per_step": t * 1e3, "dtype": "f64",
                     "config": {"workload": "fuzz::token_sort_ratio cutoff 80 (and QRatio, WRatio, token_set_ratio), "
                                            "256 x %d uint32 token strings (1-4 tokens of 3-12 units) from pinned "
                                            "host buffers to a pinned host float64 matrix: host sorted-split joins / "
                                            "parts, upload, device scorer, download" % nc,
                                "ms_per_call": {k: v * 1e3 for k, v in per.items()},
                                "ms_per_call_fresh_pageable_result": {k: v * 1e3 for k, v in per_fresh.items()}},
                     "cpu_baseline": {"value": sub * nc / tc, "unit": "pairs/s", "cores": os.cpu_count(),
                                      "kind": "port", "sample": "8 of the 256 queries x all %d choices" % nc},
                     "e2e": {"value": nq * nc / t, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
                             "d2h_bytes_per_step": nq * nc * 8},
                     "gpu_launches": None, "clocks": clk})
    elif args.workload == "editops":
        from oracle_lib import editops as oracle_editops, oracle
        npairs = args.nc if args.nc != 4096 else 200000
        a = WL.dna_uniform(seed=51, n=npairs)
        rng = np.random.default_rng(52)
        b_strs = []
        for i in range(npairs):
            s = bytearray(a[0][a[1][i]:a[1][i + 1]].tobytes())
            for _ in range(int(rng.integers(0, 6))):
                k = int(rng.integers(0, 3))
                pos = int(rng.integers(0, len(s) + 1))
                if k == 0 and pos < len(s):
                    s[pos] = b"ACGT"[int(rng.integers(0, 4))]
                elif k == 1:
                    s.insert(pos, b"ACGT"[int(rng.integers(0, 4))])
                elif pos < len(s):
                    del s[pos]
            b_strs.append(bytes(s))
        b = R.pack_strings(b_strs, 1)
        clocks = B.ClockSampler()
        clocks.start()
        for _ in range(warmup):
            got = R.editops_many(R.LEVENSHTEIN, a, b)
        t0 = time.perf_counter()
        for _ in range(steps):
            got = R.editops_many(R.LEVENSHTEIN, a, b)
        t = (time.perf_counter() - t0) / steps
        clk = clocks.stop(torch.cuda.current_device())
        o = oracle()
        for i in (0, 1, npairs // 2, npairs - 1):
            x = a[0][a[1][i]:a[1][i + 1]]
            y = b[0][b[1][i]:b[1][i + 1]]
            assert [tuple(int(v) for v in r) for r in got[i][["type", "src_pos", "dest_pos"]].tolist()] == \
                oracle_editops(o.rfo_editops, R.LEVENSHTEIN, x, y), "editops parity"
        sub = 2000
        tc0 = time.perf_counter()
        for i in range(sub):
            oracle_editops(o.rfo_editops, R.LEVENSHTEIN, a[0][a[1][i]:a[1][i + 1]], b[0][b[1][i]:b[1][i + 1]])
        tc = time.perf_counter() - tc0
        nops = int(got.offsets[-1])
        line.update({"value": npairs / t, "unit": "pairs/s", "ms_per_step": t * 1e3, "dtype": "u64",
                     "config": {"workload": "levenshtein_editops of %d DNA pairs, s1 len U[8,64], s2 = s1 with 0-5 "
                                            "edits, host buffers in and out through rfg_editops" % npairs,
                                "operations_per_step": nops},
                     "cpu_baseline": {"value": sub / tc, "unit": "pairs/s", "cores": 1, "kind": "port",
                                      "sample": "2,000 pairs through the oracle's DP restatement, one thread"},
                     "e2e": {"value": npairs / t, "unit": "pairs/s",
                             "h2d_bytes_per_step": int(a[0].nbytes + a[1].nbytes + b[0].nbytes + b[1].nbytes),
                             "d2h_bytes_per_step": int(nops * 24 + npairs * 8)},
                     # per call: one k_editops launch (the pairs' matrices fit one scratch
                     # budget of 256M words at this size) and one k_editops_pack
                     "gpu_launches": 2 * steps, "clocks": clk})
    elif args.workload == "partial":
        nq = 256
        nc = args.nc if args.nc != 4096 else 200000
        (q, ql) = WL.tokens_u32(seed=41, n=nq)
        c = WL.tokens_u32_fast(seed=42, n=nc)
        cells = _cells(q, c)
        qd, kq = _dev(torch, q, dev)
        cd, kc = _dev(torch, c, dev)
        out = torch.empty((nq, nc), dtype=torch.float64, device=dev)
        b = R.Batch(R.PARTIAL_RATIO, R.SIMILARITY, qd, cd, out.data_ptr(), 80.0, out_dtype=R.F64,
                    flags=R.DEVICE_INPUTS)
        if not args.no_tune:
            b.tune(stream.cuda_stream)
        t, per, clk = _timed_batches(torch, [b], stream, steps, warmup, flush)
        rows = [0, 127, 255]
        qrows = (np.concatenate([q[0][q[1][r]:q[1][r + 1]] for r in rows]),
                 np.concatenate([[0], np.cumsum([q[1][r + 1] - q[1][r] for r in rows])]).astype(np.int64), 4)
        exp = oracle_cdist(R.PARTIAL_RATIO, R.SIMILARITY, qrows, c, 80.0)
        assert np.array_equal(out[rows].cpu().numpy().view(np.int64), exp.view(np.int64)), "partial parity"
        sub = 4
        qsub = (q[0][:q[1][sub]], q[1][:sub + 1].copy(), 4)
        tc0 = time.perf_counter()
        oracle_cdist(R.PARTIAL_RATIO, R.SIMILARITY, qsub, c, 80.0)
        tc = time.perf_counter() - tc0
        line.update({"value": nq * nc * steps / t, "unit": "pairs/s", "ms_per_step": t / steps * 1e3, "dtype": "f64",
                     "config": {"workload": "fuzz::partial_ratio cutoff 80, 256 x %d uint32 token strings "
                                            "(1-4 tokens of 3-12 units), dense float64 out (on device)" % nc,
                                "gcups": cells * steps / t / 1e9, "per_kernel_ms": {"partial_ratio": per[0]}},
                     "cpu_baseline": {"value": sub * nc / tc, "unit": "pairs/s", "cores": os.cpu_count(),
                                      "kind": "port", "sample": "4 of the 256 queries x all %d choices" % nc},
                     "e2e": None, "gpu_launches": steps, "clocks": clk})
    else:
        nq = 1024
        nc = args.nc if args.nc != 4096 else 1000000
        (q, ql) = WL.tokens_u32(seed=14, n=nq)
        c = WL.tokens_u32_fast(seed=15, n=nc)
        cells = _cells(q, c)
        qd, kq = _dev(torch, q, dev)
        cd, kc = _dev(torch, c, dev)
        outs = [torch.empty((nq, nc), dtype=torch.float64, device=dev) for _ in range(2)]
        bs = [R.Batch(R.JARO_WINKLER, R.SIMILARITY, qd, cd, outs[0].data_ptr(), 0.85, out_dtype=R.F64,
                      flags=R.DEVICE_INPUTS),
              R.Batch(R.RATIO, R.SIMILARITY, qd, cd, outs[1].data_ptr(), 85.0, out_dtype=R.F64,
                      flags=R.DEVICE_INPUTS)]
        if not args.no_tune:
            for b in bs:
                b.tune(stream.cuda_stream)
        t, per, clk = _timed_batches(torch, bs, stream, steps, warmup, flush)
        rows = [0, 511, 1023]
        qrows = (np.concatenate([q[0][q[1][r]:q[1][r + 1]] for r in rows]),
                 np.concatenate([[0], np.cumsum([q[1][r + 1] - q[1][r] for r in rows])]).astype(np.int64), 4)
        for m, cut, o in ((R.JARO_WINKLER, 0.85, outs[0]), (R.RATIO, 85.0, outs[1])):
            exp = oracle_cdist(m, R.SIMILARITY, qrows, c, cut)
            assert np.array_equal(o[rows].cpu().numpy().view(np.int64), exp.view(np.int64)), "tokens1024x1m parity"
        tc0 = time.perf_counter()
        sub = 4
        qsub = (q[0][:q[1][sub]], q[1][:sub + 1].copy(), 4)
        for m, cut in ((R.JARO_WINKLER, 0.85), (R.RATIO, 85.0)):
            oracle_cdist(m, R.SIMILARITY, qsub, c, cut)
        tc = time.perf_counter() - tc0
        line.update({"value": 2 * cells * steps / t / 1e9, "ms_per_step": t / steps * 1e3, "dtype": "u64+f64",
                     "config": {"workload": "tokens1024x1m: Jaro-Winkler 0.85 + fuzz::ratio 85, 1,024 x %d uint32 "
                                            "token strings, dense float64 out (on device)" % nc,
                                "pairs_per_s": 2 * nq * nc * steps / t,
                                "per_kernel_ms": {"jaro_winkler": per[0], "ratio": per[1]},
                                "out_bytes_per_step": 2 * nq * nc * 8},
                     "cpu_baseline": {"value": 2 * _cells(qsub, c) / tc / 1e9, "unit": "GCUPS",
                                      "cores": os.cpu_count(), "kind": "port",
                                      "sample": "4 of the 1,024 queries x all %d choices" % nc},
                     "e2e": None, "gpu_launches": 2 * steps, "clocks": clk})
    print(json.dumps(line), flush=True)


def serving_corpora(R, corpus=10_000_000):
    """the two device-resident corpora of config 5 and the seconds it took to build them"""
    import workloads as WL
    t0 = time.perf_counter()
    dna = WL.dna_corpus_fast(seed=31, n=corpus)
    tok = WL.tokens_u32_fast(seed=32, n=1_000_000)
    corpora = [R.Corpus(dna), R.Corpus(tok)]
    return corpora, time.perf_counter() - t0


def serving_capacity(R, duration, rate=2000.0, corpus=10_000_000):
    """config 5 at the offered rate, then at 80 % of the completed rate that run measured
    (a load the server sustains without its queue growing): both legs' results"""
    corpora, setup = serving_corpora(R, corpus)
    over = serving_leg(R, duration, rate=rate, corpus=corpus, corpora=corpora)
    over["setup_s"] = setup
    sustained = serving_leg(R, duration, rate=0.8 * min(rate, over["completed_per_s"]), corpus=corpus,
                            corpora=corpora, seed=34)
    return {"at_offered_rate": over, "at_sustained_rate": sustained}


def serving_leg(R, duration, rate=2000.0, corpus=10_000_000, max_inflight=4, max_batch=64, seed=33, corpora=None):
    """Config 5 in short: device-resident corpora of `corpus` DNA strings (len U[10,200]) and
    1,000,000 uint32 token strings; Poisson arrivals at `rate` req/s for `duration` s, each
    an extractOne (limit 1) or top-10 extract of one query of length U[5,500] with a metric
    drawn from {Levenshtein, Indel, OSA} (DNA) or Jaro-Winkler (tokens), through the
    continuous-batching server; returns latency percentiles, completed and offered req/s,
    and the same kinds of requests one at a time (rfg_extract)"""
    import threading
    import workloads as WL
    t_setup = 0.0
    if corpora is None:
        corpora, t_setup = serving_corpora(R, corpus)
    rng = np.random.default_rng(seed)
    acgt = np.frombuffer(b"ACGT", dtype=np.uint8)
    alpha = np.array(WL.TOKEN_ALPHABET + [0x20], dtype=np.uint32)
    kinds = [(0, R.LEVENSHTEIN, R.DISTANCE), (0, R.INDEL, R.DISTANCE), (0, R.OSA, R.DISTANCE),
             (1, R.JARO_WINKLER, R.SIMILARITY)]

    def make_request():
        c, m, op = kinds[int(rng.integers(0, 4))]
        n = int(rng.integers(5, 501))
        q = acgt[rng.integers(0, 4, size=n)] if c == 0 else alpha[rng.integers(0, len(alpha), size=n)]
        limit = 1 if rng.random() < 0.5 else 10
        return c, m, op, q, limit

    # the same kinds of requests one at a time through rfg_extract
    alone = {}
    for kind in range(4):
        c, m, op = kinds[kind]
        ts = []
        for rep in range(4):
            n = int(rng.integers(5, 501))
            q = acgt[rng.integers(0, 4, size=n)] if c == 0 else alpha[rng.integers(0, len(alpha), size=n)]
            qb = R.pack_strings([q], q.itemsize)
            a = time.perf_counter()
            corpora[c].extract(m, op, qb, 10, None, False)
            ts.append(time.perf_counter() - a)
        alone[kind] = float(np.median(ts[1:]))
    sizes = [corpora[0].count, corpora[1].count]

    n_req = int(rate * duration)
    gaps = rng.exponential(1.0 / rate, size=n_req)
    arrivals = np.cumsum(gaps)
    reqs = [make_request() for _ in range(n_req)]
    server = R.Server(corpora, max_inflight=max_inflight, max_batch=max_batch)
    tickets = [None] * n_req
    clocks = B.ClockSampler()
    clocks.start()
    start = time.perf_counter()

    def submitter():
        for i, (c, m, op, q, limit) in enumerate(reqs):
            delay = start + arrivals[i] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            tickets[i] = server.submit(c, m, op, q, limit, None, limit == 1)

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    t_submitted = time.perf_counter() - start
    lat = []
    for t in tickets:
        _, _, ms = server.wait(t, timeout=3600)
        lat.append(ms)
    wall = time.perf_counter() - start
    clk = clocks.stop(0)
    st = server.stats()
    server.close()
    lat = np.array(lat)
    pairs = float(sum(sizes[c] for c, *_ in reqs))
    pairs_alone = float(np.mean([sizes[kinds[k][0]] / alone[k] for k in range(4)]))
    return {"workload": "serving: %d DNA (len U[10,200]) + 1,000,000 uint32 token strings, Poisson %.0f req/s "
                        "for %.1f s, extractOne/top-10, Lev/Indel/OSA/JW, query len U[5,500]" % (corpus, rate, duration),
            "requests": n_req, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_ms": float(lat.max()), "completed_per_s": n_req / wall, "offered_per_s": rate,
            "pairs_per_s": pairs / wall, "wall_s": wall,
            "arrivals_span_s": float(arrivals[-1]), "submit_span_s": t_submitted,
            "batches": st["batches"], "mean_batch": st["batched_requests"] / max(st["batches"], 1),
            "alone_ms": {"levenshtein": alone[0] * 1e3, "indel": alone[1] * 1e3, "osa": alone[2] * 1e3,
                         "jaro_winkler": alone[3] * 1e3},
            "pairs_per_s_one_at_a_time": pairs_alone, "setup_s": t_setup, "clocks": clk}


def run_serving(args, R, WL):
    leg = serving_leg(R, args.duration, rate=args.rate, corpus=args.corpus)
    n_req = leg["requests"]
    line = {"metric": METRIC, "value": leg["pairs_per_s"], "unit": "pairs/s", "n_gpus": 1, "steps": n_req,
            "warmup": 0, "ms_per_step": leg["wall_s"] / n_req * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64+f64", "data": "synthetic (seeded dna_corpus_fast, tokens_u32_fast)",
            "config": {"workload": leg["workload"]}, "detail": leg,
            "cpu_baseline": None, "e2e": None, "gpu_launches": None, "clocks": leg["clocks"]}
    print(json.dumps(line), flush=True)
