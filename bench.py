"""Benchmark of the GB300 scorer path on its headline workload.

Workload (default): all-pairs cdist 4,096 x 4,096 uint8 strings over a-z with Zipf(1.1)
letter frequencies, lengths U[16, 64], 20 % of the choices mutated copies of a query
(1-6 edits); Levenshtein, Indel and OSA each with score_cutoff = 8; int32 outputs.
One step = the three cdists over the whole batch.

  value : GCUPS (full-matrix cells l1*l2 per second, x1e9) with the strings resident in HBM,
          prepared batches replayed as CUDA graphs, CUDA events on the launching stream,
          L2 flushed (256 MB write) between steps.
  e2e   : the same metric through the public C ABI (rfg_cdist) with pinned host buffers:
          host->device copies of the strings and the device->host copy of the three
          int32 matrices inside the timed region.
  roofline : the dominant kernel against the measured INT32 issue rate (LOP3/IADD3/SHF
          microbenchmark): algorithmic integer ops = required word-steps (pairs that pass
          the length filter |l1-l2| <= 8, ceil(l1/64)*l2 each) x ops per word-step
          (Levenshtein 23, Indel/LCS 8, OSA 29).
  cpu_baseline : the CPU restatement of the reference's Cached* path (oracle/librfo.so),
          all host threads, on the same workload.

--impl reference times that CPU path alone and prints its own line.
Multi-GPU (torchrun, N ranks): every rank scores its own seed-shifted 4,096 x 4,096 batch
(independent shards, no collective on the data path); value = all ranks' cells / max time.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "rapidfuzz-cpp_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC_NAME = "GCUPS & pairs/s, batched vs per-call, 1 GB300, bit-exact; extract p50/p99 ms"
# dram__bytes_read.sum + dram__bytes_write.sum of one metric's launches of the several-queries
# kernels (k_tiles_mq, 64-bit and 32-bit words) on this workload, averaged over four steps of
# one `ncu --metrics` capture: the strings are read once, the 67 MB of results stay in the
# 129 MB L2 when the launch ends (written back later)
DRAM_BYTES_PER_LAUNCH = {"levenshtein": 1117056, "indel": 1151168, "osa": 1015104}
OPS_PER_WORD_STEP = {"levenshtein": 23, "indel": 8, "osa": 29}
CUTOFF = 8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape (fixed launch list)")
    ap.add_argument("--nq", type=int, default=4096)
    ap.add_argument("--nc", type=int, default=4096)
    ap.add_argument("--workload", default="cdist", choices=["cdist", "dna1x100k", "dna256x65536", "tokens1024x1m", "serving", "partial", "tokens", "editops"],
                    help="cdist: 4096x4096 Zipf a-z Lev/Indel/OSA (the headline); dna1x100k: 1 x 100k DNA per-call "
                         "vs batched; dna256x65536: 256 x 65536 long DNA banded; tokens1024x1m: 1024 x 1M uint32 JW + ratio; "
                         "serving: serving, Poisson extract/extractOne requests over 10M DNA + 1M token strings")
    ap.add_argument("--rate", type=float, default=2000.0, help="serving: request arrival rate (req/s)")
    ap.add_argument("--duration", type=float, default=2.0, help="serving: seconds of arrivals")
    ap.add_argument("--corpus", type=int, default=10_000_000, help="serving: DNA corpus size")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(rank, nq, nc):
    from workloads import cdist_zipf
    return cdist_zipf(seed=1234 + rank, nq=nq, nc=nc)


def cells_and_steps(q, c):
    """full-matrix cells and required word-steps (pairs with |l1-l2| <= CUTOFF)"""
    ql = np.diff(q[1]).astype(np.int64)
    cl = np.diff(c[1]).astype(np.int64)
    cells = float(ql.sum()) * float(cl.sum())
    words = (ql + 63) // 64
    # histogram over lengths keeps this O(L^2)
    lq = np.bincount(ql, minlength=1)
    wq = np.bincount(ql, weights=words, minlength=1)
    lc = np.bincount(cl, minlength=1)
    steps = 0.0
    pairs_pass = 0.0
    for a in np.nonzero(lq)[0]:
        for b in np.nonzero(lc)[0]:
            if abs(int(a) - int(b)) <= CUTOFF:
                steps += wq[a] * lc[b] * b
                pairs_pass += lq[a] * lc[b]
    return cells, steps, pairs_pass


class ClockSampler:
    """nvidia-smi samples during the timed region"""

    def __init__(self):
        self.rows = []
        self.proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self, device=0):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 9 and r[0] == str(device)]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_cdist(q, c, nthreads=0):
    """the three metrics on the CPU restatement; returns seconds"""
    from oracle_lib import oracle_cdist, LEVENSHTEIN, INDEL, OSA, DISTANCE
    t0 = time.perf_counter()
    for m in (LEVENSHTEIN, INDEL, OSA):
        oracle_cdist(m, DISTANCE, q, c, CUTOFF, out_dtype=0, nthreads=nthreads)
    return time.perf_counter() - t0


def run_reference(args, rank, world):
    if rank != 0:
        return
    q, c = workload(0, args.nq, args.nc)
    cells, steps, pairs_pass = cells_and_steps(q, c)
    npairs = float(len(q[1]) - 1) * float(len(c[1]) - 1) * 3
    cores = os.cpu_count() or 1
    for _ in range(min(args.warmup, 1)):
        cpu_cdist(q, c)
    times = [cpu_cdist(q, c) for _ in range(args.steps)]
    t = float(np.sum(times))
    value = cells * 3 * args.steps / t / 1e9
    line = {"impl": "reference", "metric": METRIC_NAME, "value": value, "unit": "GCUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded cdist_zipf)",
            "config": {"workload": "cdist 4096x4096 a-z Zipf(1.1) len U[16,64], 20% mutated copies; "
                                   "Levenshtein+Indel+OSA score_cutoff=8, int32 out",
                       "global_batch": int(npairs), "pairs_per_s": npairs * args.steps / t},
            "cpu_baseline": {"value": value, "unit": "GCUPS", "cores": cores, "kind": "port",
                             "sample": "the full workload, every step"},
            "e2e": {"value": value, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def executed_word_steps(metric, q, c):
    """word steps the single-word kernels execute on this workload (early exits and the
    length filter included), counted on the host by the same cores (librfg_count.so)"""
    lib = ctypes.CDLL(os.path.join(ROOT, "rapidfuzz-cpp_gb300", "lib", "librfg_count.so"))
    lib.rfg_count_word_steps.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64,
                                         ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
    out = ctypes.c_uint64()
    rc = lib.rfg_count_word_steps(metric, q[0].ctypes.data, q[1].ctypes.data, len(q[1]) - 1, c[0].ctypes.data,
                                  c[1].ctypes.data, len(c[1]) - 1, CUTOFF, 0, ctypes.byref(out))
    return float(out.value) if rc == 0 else None


def int_peak_ops():
    lib = ctypes.CDLL(os.path.join(ROOT, "rapidfuzz-cpp_gb300", "lib", "librfg_peak.so"))
    lib.rfg_peak_int_ops.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    ops = ctypes.c_double()
    ms = ctypes.c_double()
    rc = lib.rfg_peak_int_ops(20000, ctypes.byref(ops), ctypes.byref(ms))
    if rc:
        raise RuntimeError("peak microbenchmark failed (%d)" % rc)
    return ops.value


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.workload != "cdist":
        import bench_configs
        return bench_configs.run(args, rank, world, local)
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import rapidfuzz_gb300 as R
    from rapidfuzz_gb300 import sharding
    R.lib().rfg_set_device(local)

    q, c = workload(rank, args.nq, args.nc)
    nq, nc = len(q[1]) - 1, len(c[1]) - 1
    cells, req_steps, pairs_pass = cells_and_steps(q, c)
    npairs = float(nq) * nc

    dev = torch.device("cuda", local)
    # device-resident inputs and outputs
    qd = torch.from_numpy(q[0]).to(dev)
    qo = torch.from_numpy(q[1]).to(dev)
    cd = torch.from_numpy(c[0]).to(dev)
    co = torch.from_numpy(c[1]).to(dev)
    outs = [torch.empty((nq, nc), dtype=torch.int32, device=dev) for _ in range(3)]
    metrics = [("levenshtein", R.LEVENSHTEIN), ("indel", R.INDEL), ("osa", R.OSA)]
    stream = torch.cuda.Stream(device=dev)
    batches = []
    for (name, m), o in zip(metrics, outs):
        b = R.Batch(m, R.DISTANCE, (qd.data_ptr(), qo.data_ptr(), 1, nq), (cd.data_ptr(), co.data_ptr(), 1, nc),
                    o.data_ptr(), CUTOFF, out_dtype=R.I32, flags=R.DEVICE_INPUTS)
        if not args.no_tune:
            b.tune(stream.cuda_stream)
        batches.append((name, b))
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def step(events=None):
        for i, (name, b) in enumerate(batches):
            if events is not None:
                events[i][0].record(stream)
            b.launch(stream.cuda_stream, graph=True)
            if events is not None:
                events[i][1].record(stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        for _, b in batches:
            b.check(stream.cuda_stream)
    torch.cuda.synchronize()

    # parity spot check of the timed path (rows of each matrix against the oracle)
    from oracle_lib import oracle_cdist
    rows = [0, nq // 2, nq - 1]
    qsub_list = [q[0][q[1][r]:q[1][r + 1]] for r in rows]
    qs_off = np.zeros(len(rows) + 1, dtype=np.int64)
    qs_off[1:] = np.cumsum([len(x) for x in qsub_list])
    qsub = (np.concatenate(qsub_list), qs_off, 1)
    for (name, m), o in zip(metrics, outs):
        exp = oracle_cdist(m, R.DISTANCE, qsub, c, CUTOFF, out_dtype=0)
        got = o[rows].cpu().numpy()
        if not np.array_equal(got, exp):
            raise SystemExit("bench: %s result differs from the oracle" % name)

    if dist is not None:
        dist.barrier()
    clocks = ClockSampler()
    clocks.start()
    time.sleep(0.3)
    per_kernel = {name: 0.0 for name, _ in batches}
    total_ms = 0.0
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            flush.zero_()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in batches]
            step(ev)
            stream.synchronize()
            for (name, _), (e0, e1) in zip(batches, ev):
                t = e0.elapsed_time(e1)
                per_kernel[name] += t
            total_ms += ev[0][0].elapsed_time(ev[-1][1])
    torch.cuda.synchronize()
    clk = clocks.stop(local)
    t_max = sharding.max_over_ranks(total_ms / 1e3, device=dev)
    for _, b in batches:
        b.check(stream.cuda_stream)

    value = cells * 3 * args.steps * world / t_max / 1e9
    pairs_per_s = npairs * 3 * args.steps * world / t_max

    # roofline of the dominant kernel
    dom = max(per_kernel, key=per_kernel.get)
    dom_ms = per_kernel[dom] / args.steps
    metric_ids = {"levenshtein": 0, "indel": 1, "osa": 3}
    exec_steps = {name: executed_word_steps(metric_ids[name], q, c) for name, _ in batches}
    alg_ops = (exec_steps[dom] if exec_steps[dom] is not None else req_steps) * OPS_PER_WORD_STEP[dom]
    peak = int_peak_ops()
    achieved = alg_ops / (dom_ms * 1e-3)
    kern = dict((name, b.kernels()) for name, b in batches)
    dom_kernel = ";".join(kern[dom])
    traffic = (DRAM_BYTES_PER_LAUNCH.get(dom) if args.nq == 4096 and args.nc == 4096 and "k_tiles_mq" in dom_kernel
               else None)

    # e2e through the public C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        def pinned(a):
            t = torch.from_numpy(a).pin_memory()
            return t.numpy(), t
        qh = (pinned(q[0])[0], pinned(q[1])[0], 1)
        ch = (pinned(c[0])[0], pinned(c[1])[0], 1)
        ho = [torch.empty((nq, nc), dtype=torch.int32).pin_memory().numpy() for _ in range(3)]
        for _ in range(2):
            for (name, m), o in zip(metrics, ho):
                R.cdist(m, R.DISTANCE, qh, ch, CUTOFF, out_dtype=R.I32, out=o)
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for (name, m), o in zip(metrics, ho):
                R.cdist(m, R.DISTANCE, qh, ch, CUTOFF, out_dtype=R.I32, out=o)
        te = sharding.max_over_ranks(time.perf_counter() - t0, device=dev)
        h2d = 3 * (q[0].nbytes + q[1].nbytes + c[0].nbytes + c[1].nbytes)
        d2h = 3 * nq * nc * 4
        e2e = {"value": cells * 3 * args.steps * world / te / 1e9, "unit": "GCUPS", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": te / args.steps * 1e3,
               "pairs_per_s": npairs * 3 * args.steps * world / te}

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        tc = cpu_cdist(q, c)
        cpu = {"value": cells * 3 / tc / 1e9, "unit": "GCUPS", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": "the full 4096x4096 x3-metric workload, one pass", "seconds": tc}

    if rank == 0:
        line = {"metric": METRIC_NAME, "value": value, "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded cdist_zipf)",
                "config": {"workload": "cdist %dx%d a-z Zipf(1.1) len U[16,64], 20%% mutated copies; "
                                       "Levenshtein+Indel+OSA score_cutoff=8, int32 out" % (nq, nc),
                           "global_batch": int(npairs * 3 * world), "pairs_per_s": pairs_per_s,
                           "l2": "flushed between steps (256 MB write); strings are L2-resident within a step",
                           "launch": "prepared batches replayed as CUDA graphs",
                           "per_kernel_ms": {k: v / args.steps for k, v in per_kernel.items()},
                           "required_word_steps_per_metric": req_steps,
                           "executed_word_steps": exec_steps, "pairs_passing_length_filter": pairs_pass},
                "roofline": {"bound": "int32", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "Tops/s",
                             "frac": achieved / peak, "traffic": traffic, "kernel": dom_kernel,
                             "peak_source": "measured: LOP3/IADD3/SHF issue-rate microbenchmark (librfg_peak.so)",
                             "ops_per_word_step": OPS_PER_WORD_STEP[dom]},
                "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": sum(len(k) for k in kern.values()) * args.steps, "clocks": clk}
        print(json.dumps(line), flush=True)
    for _, b in batches:
        b.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
