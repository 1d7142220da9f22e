"""The C++ drop-in (rapidfuzz-cpp_gb300/include/rapidfuzz_gb300/rapidfuzz.hpp): compile
tests/cpp/test_api.cpp against the library and the oracle and run it on the GPU.  The
program restates the reference's known answers and sweeps every free-function and
Cached* form against the oracle bit-exactly."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("std", ["c++11", "c++17"])
def test_cpp_dropin(tmp_path, std):
    import __graft_entry__  # noqa: F401  (paths)
    lib = os.path.join(ROOT, "rapidfuzz-cpp_gb300", "lib")
    ora = os.path.join(ROOT, "oracle")
    exe = str(tmp_path / ("test_api_" + std.replace("+", "p")))
    cmd = ["g++", "-std=" + std, "-O1", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "rapidfuzz-cpp_gb300", "include"), "-I", ora,
           os.path.join(ROOT, "tests", "cpp", "test_api.cpp"), "-o", exe, "-L", lib, "-lrapidfuzz_gb300",
           "-L", ora, "-lrfo", "-Wl,-rpath," + lib + ":" + ora]
    subprocess.run(cmd, check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
