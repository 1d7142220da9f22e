"""CPU tests of the Editops / Opcodes boundary types against the reference (opcodes.json,
made by tests/golden/make_golden.py from the unmodified headers): Opcodes(Editops) and
Editops(Opcodes) (details/types.hpp:500-569), editops_apply / opcodes_apply
(distance.hpp:19-165), for the Python mirror and for the C++ drop-in header.  The editops
themselves are the reference's (editops.json); no device call."""
import json
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "rapidfuzz-cpp_gb300"))
NAMES = ("none", "replace", "insert", "delete")


@pytest.fixture(scope="module")
def cases():
    with open(os.path.join(GOLDEN, "editops.json")) as f:
        eops = json.load(f)
    with open(os.path.join(GOLDEN, "opcodes.json")) as f:
        opc = json.load(f)
    assert len(opc) >= 500
    return [(eops[c["case"]], c) for c in opc]


def test_python_mirror_matches_reference(cases):
    import rapidfuzz_gb300 as R
    for e, c in cases:
        ops = R.Editops([R.EditOp(t, s, d) for t, s, d in e["expected"]], len(e["s1"]), len(e["s2"]))
        o = ops.as_opcodes()
        assert [tuple(x) for x in o] == [(NAMES[t], sb, se, db, de) for t, sb, se, db, de in c["opcodes"]], c["case"]
        assert (o.src_len, o.dest_len) == (len(e["s1"]), len(e["s2"]))
        back = o.as_editops()
        assert [tuple(x) for x in back] == [(NAMES[t], s, d) for t, s, d in c["back"]], c["case"]
        assert ops.apply(e["s1"], e["s2"]) == c["editops_apply"], c["case"]
        assert o.apply(e["s1"], e["s2"]) == c["opcodes_apply"], c["case"]
        assert c["opcodes_apply"] == e["s2"]


def test_cpp_header_matches_reference(cases):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "opcodes_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "rapidfuzz-cpp_gb300", "include"), "-o", exe,
                    os.path.join(ROOT, "tests", "cpp", "opcodes_check.cpp")], check=True)
    words = [str(len(cases))]
    for e, _ in cases:
        words.append(str(len(e["expected"])))
        words += [str(v) for op in e["expected"] for v in op]
        words += [str(len(e["s1"]))] + [str(v) for v in e["s1"]]
        words += [str(len(e["s2"]))] + [str(v) for v in e["s2"]]
    r = subprocess.run([exe], input=" ".join(words), capture_output=True, text=True, check=True)
    lines = r.stdout.split("\n")
    for k, (e, c) in enumerate(cases):
        o, b, ea, oa = (list(map(int, lines[4 * k + j].split())) for j in range(4))
        assert o[0] == len(c["opcodes"]) and o[1:] == [v for x in c["opcodes"] for v in x], c["case"]
        assert b[0] == len(c["back"]) and b[1:] == [v for x in c["back"] for v in x], c["case"]
        assert ea[0] == len(c["editops_apply"]) and ea[1:] == c["editops_apply"], c["case"]
        assert oa[0] == len(c["opcodes_apply"]) and oa[1:] == c["opcodes_apply"], c["case"]


@pytest.fixture(scope="module")
def listops():
    with open(os.path.join(GOLDEN, "editops.json")) as f:
        eops = json.load(f)
    with open(os.path.join(GOLDEN, "listops.json")) as f:
        cases = json.load(f)
    assert len(cases) >= 1000
    return [(eops[c["case"]], c) for c in cases]


def _mirror_listop(R, e, c):
    ops = R.Editops([R.EditOp(t, s, d) for t, s, d in e["expected"]], len(e["s1"]), len(e["s2"]))
    w, a, b, st = c["which"], c["start"], c["stop"], c["step"]
    try:
        if w == 0:
            r = ops.slice(a, b, st)
        elif w == 1:
            r = R.Editops(list(ops), ops.src_len, ops.dest_len)
            r.remove_slice(a, b, st)
        elif w == 2:
            r = ops.reverse()
        elif w == 3:
            r = ops.inverse()
        elif w == 4:
            r = ops.remove_subsequence(ops.slice(a, b, st))
        elif w == 10:
            r = ops.as_opcodes().slice(a, b, st)
        elif w == 12:
            r = ops.as_opcodes().reverse()
        else:
            r = ops.as_opcodes().inverse()
    except ValueError:
        return None, None
    recs = [[NAMES.index(x[0])] + list(x[1:]) for x in r]
    return recs, [r.src_len, r.dest_len]


def test_python_list_operations_match_reference(listops):
    """Editops slice / remove_slice / reverse / inverse / remove_subsequence and Opcodes
    slice / reverse / inverse (details/types.hpp:109-161, 240-320, 420-475)"""
    import rapidfuzz_gb300 as R
    for e, c in listops:
        recs, lens = _mirror_listop(R, e, c)
        assert recs == c["result"] and lens == c["lens"], c


def test_cpp_list_operations_match_reference(listops):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "listops_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "rapidfuzz-cpp_gb300", "include"), "-o", exe,
                    os.path.join(ROOT, "tests", "cpp", "listops_check.cpp")], check=True)
    words = [str(len(listops))]
    for e, c in listops:
        words += [str(c["which"]), str(c["start"]), str(c["stop"]), str(c["step"]), str(len(e["expected"]))]
        words += [str(v) for op in e["expected"] for v in op]
        words += [str(len(e["s1"])), str(len(e["s2"]))]
    r = subprocess.run([exe], input=" ".join(words), capture_output=True, text=True, check=True)
    lines = r.stdout.split("\n")
    for k, (e, c) in enumerate(listops):
        if c["result"] is None:
            assert lines[k] == "err", c
            continue
        v = list(map(int, lines[k].split()))
        rec = 3 if c["which"] < 10 else 5
        assert v[0] == len(c["result"]), c
        assert v[1:1 + rec * v[0]] == [x for r_ in c["result"] for x in r_], c
        assert v[1 + rec * v[0]:] == c["lens"], c
