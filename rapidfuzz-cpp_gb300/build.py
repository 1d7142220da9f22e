"""Build recipe of librapidfuzz_gb300.so: nvcc for sm_103a only, one object per
translation unit compiled in parallel, linked into lib/librapidfuzz_gb300.so."""
import concurrent.futures
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "librapidfuzz_gb300.so")
PEAK_LIB = os.path.join(LIB_DIR, "librfg_peak.so")  # INT32 issue-rate microbenchmark (bench roofline)
COUNT_LIB = os.path.join(LIB_DIR, "librfg_count.so")  # executed word steps of the kernels (bench roofline)
# the machine the libraries in lib/ were built on: a tree copied to another machine
# (an x86-64 build container, an aarch64 GPU host) rebuilds instead of reusing them
STAMP = os.path.join(LIB_DIR, "build_machine.txt")

SOURCES = ["rfg_api.cu", "rfg_k_band.cu", "rfg_k_band_lcs.cu", "rfg_k_lev.cu", "rfg_k_lcs.cu", "rfg_k_osa.cu", "rfg_k_jaro.cu", "rfg_k_generic.cu", "rfg_noalloc.cu", "rfg_server.cu",
           "rfg_k_token.cu", "rfg_k_editops.cu", "rfg_token.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "rapidfuzz_gb300.h")]


def _compile(src):
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def _stamp_matches():
    try:
        with open(STAMP) as f:
            return f.read().strip() == platform.machine()
    except OSError:
        return False


def build(force=False, verbose=False):
    """Compile the library if any source is newer than it, or if it was built on another
    kind of machine; returns the .so path."""
    if not force and _stamp_matches() and all(os.path.exists(x) for x in (LIB, PEAK_LIB, COUNT_LIB)):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return LIB
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    r = subprocess.run([nvcc()] + ARCH + ["-O3", "-Xcompiler", "-fPIC", "-shared", "-o", PEAK_LIB,
                                          os.path.join(CSRC, "rfg_peak.cu")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("peak benchmark build failed:\n%s%s" % (r.stdout, r.stderr))
    cxx = shutil.which("g++") or "g++"
    r = subprocess.run([cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-I" + CSRC,
                        "-o", COUNT_LIB, os.path.join(CSRC, "rfg_count.cpp")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("work counter build failed:\n%s%s" % (r.stdout, r.stderr))
    with open(STAMP, "w") as f:
        f.write(platform.machine() + "\n")
    if verbose:
        print("built", LIB, "on", platform.machine())
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
