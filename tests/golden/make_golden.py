"""Generate tests/golden/*.json from the UNMODIFIED reference (oracle/_ref/librfref.so,
built by `make -C oracle ref` from the rapidfuzz-cpp v3.3.3 headers).

Fixtures:
  kat.json      the known-answer vectors of the reference's own test suite (each case cites
                the test file:line it restates), with the value the reference computes here;
  random.json   seeded random cases over every metric x op x API form x cutoff, char widths
                1/2/4/8, lengths 0..300 (word, multi-word, banded and any-length paths);
  multi.json    Multi* batches with several inserted strings;
  partial.json  fuzz::partial_ratio / CachedPartialRatio: the reference fuzz tests' inputs and
                seeded random pairs;
  tokens.json   token_sort_ratio / partial_token_sort_ratio / QRatio (free and Cached forms);
  tokenset.json token_set_ratio / partial_token_set_ratio / token_ratio / partial_token_ratio /
                WRatio (free and Cached forms);
  editops.json  levenshtein_editops / indel_editops / lcs_seq_editops;
  opcodes.json  the reference's Opcodes / Editops conversions and applies of editops.json's
                one-byte pairs;
  listops.json  the list operations of Editops / Opcodes (slice, remove_slice, reverse,
                inverse, remove_subsequence) on editops.json's operation lists.
Doubles are stored with float.hex() so the comparison is bit-exact.

Usage: python tests/golden/make_golden.py   (needs the reference checkout; run in the
build container, the fixtures are committed).
"""
import ctypes
import json
import os
import random
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import numpy as np  # noqa: E402

from oracle_lib import (DISTANCE, SIMILARITY, NORM_DISTANCE, NORM_SIMILARITY, LEVENSHTEIN, INDEL, LCSSEQ, OSA,  # noqa: E402
                        JARO, JARO_WINKLER, RATIO, PARTIAL_RATIO, TOKEN_SORT_RATIO, PARTIAL_TOKEN_SORT_RATIO, QRATIO,
                        TOKEN_SET_RATIO, PARTIAL_TOKEN_SET_RATIO, TOKEN_RATIO, PARTIAL_TOKEN_RATIO, WRATIO, FREE, CACHED, MULTI, as_units, reference, result_is_int,
                        score, make_params, pack_strings, strings_struct)

OPS = (DISTANCE, SIMILARITY, NORM_DISTANCE, NORM_SIMILARITY)
REF_ROOT = os.environ.get("RFG_REFERENCE", "/root/reference")  # the reference checkout (build container)


def enc(v):
    return v if isinstance(v, int) else float(v).hex()


def case(metric, op, form, s1, s2, cutoff=None, weights=(1, 1, 1), pw=0.1, w1=None, w2=None, cite=None):
    a = as_units(s1, w1)
    b = as_units(s2, w2)
    ref = reference()
    v = score(ref.rfref_score, metric, op, form, a, b, cutoff, weights, pw)
    if v is None:
        return None
    d = {"metric": metric, "op": op, "form": form, "s1": [int(x) for x in a], "w1": a.itemsize,
         "s2": [int(x) for x in b], "w2": b.itemsize, "cutoff": cutoff, "weights": list(weights), "pw": pw,
         "expected": enc(v)}
    if cite:
        d["cite"] = cite
    return d


def mul(s, k):
    return s * k


def kat_cases():
    """Known answers of the reference's tests (expected values re-derived by the reference)."""
    out = []
    T = "test/distance/tests-Levenshtein.cpp"
    # empty / simple / weighted (tests-Levenshtein.cpp:98-141)
    for s1, s2 in (("", ""), ("aaaa", ""), ("", "aaaa"), ("aaaa", "aaaa"), ("aaaa", "aaa"), ("abaa", "baaa"),
                   ("aaaa", "aaab"), ("aaaa", "bbbb")):
        for w in ((1, 1, 1), (1, 1, 2)):
            out.append(case(LEVENSHTEIN, DISTANCE, FREE, s1, s2, None, w, cite=T + ":108-130"))
            out.append(case(LEVENSHTEIN, NORM_SIMILARITY, FREE, s1, s2, None, w, cite=T + ":132-141"))
            out.append(case(LEVENSHTEIN, DISTANCE, CACHED, s1, s2, None, w, cite=T + ":21-96"))
    # mbleven cutoffs (tests-Levenshtein.cpp:143-179)
    for a, b in (("South Korea", "North Korea"), ("aabc", "cccd")):
        for w in ((1, 1, 1), (1, 1, 2)):
            for c in (None, 0, 1, 2, 3, 4, 5, 6):
                out.append(case(LEVENSHTEIN, DISTANCE, FREE, a, b, c, w, cite=T + ":143-179"))
                out.append(case(LEVENSHTEIN, DISTANCE, CACHED, a, b, c, w, cite=T + ":143-179"))
    # banded (tests-Levenshtein.cpp:181-232)
    banded = [
        ("kkkkbbbbfkkkkkkibfkkkafakkfekgkkkkkkkkkkbdbbddddddddddafkkkekkkhkk",
         "khddddddddkkkkdgkdikkccccckcckkkekkkkdddddddddddafkkhckkkkkdckkkcc", (None, 31)),
        ("ccddcddddddddddddddddddddddddddddddddddddddddddddddddddddaaaaaaaaaaa",
         "aaaaaaaaaaaaaadddddddddbddddddddddddddddddddddddddddddddddbddddddddd", (None, 31)),
        ("accccccccccaaaaaaaccccccccccccccccccccccccccccccacccccccccccccccccccccccccccccc"
         "ccccccccccccccccccccaaaaaaaaaaaaacccccccccccccccccccccc",
         "ccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccc"
         "ccccccccccccccccccccccccccccccccccccbcccb", (None, 25)),
        ("miiiiiiiiiiliiiiiiibghiiaaaaaaaaaaaaaaacccfccccedddaaaaaaaaaaaaaaaaaaaaaaaaaaaa"
         "aaaaaaaaaaaaa",
         "aaaaaaajaaaaaaaabghiiaaaaaaaaaaaaaaacccfccccedddaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaajjdim", (None, 27)),
        ("lllllfllllllllllllllllllllllllllllllllllllllllllllllllglllllilldcaaaaaaaaaaaaaa"
         "aaaaadbbllllllllllhllllllllllllllllllllllllllgl",
         "aaaaaaaaaaaaaadbbllllllllllllllelllllllllllllllllllllllllllllllglllllilldcaaaaa"
         "aaaaaaaaaaaaaadbbllllllllllllllellllllllllllllhlllllllllill", (None, 27, 28)),
        ("llccacaaaaaaaaaccccccccccccccccddffaccccaccecccggggclallhcccccljif",
         "bddcbllllllbcccccccccccccccccddffccccccccebcccggggclbllhcccccljifbddcccccc", (None, 27, 28)),
    ]
    for a, b, cuts in banded:
        for c in cuts:
            for form in (FREE, CACHED):
                out.append(case(LEVENSHTEIN, DISTANCE, form, a, b, c, cite=T + ":181-232"))
    # Indel (tests-Indel.cpp:204-286)
    T = "test/distance/tests-Indel.cpp"
    for op in OPS:
        out.append(case(INDEL, op, FREE, "aaaa", "aaaa", cite=T + ":208-220"))
        out.append(case(INDEL, op, FREE, "aaaa", "bbbb", cite=T + ":208-220"))
    for a, b in (("South Korea", "North Korea"), ("aabc", "cccd")):
        for c in (None, 0, 1, 2, 3, 4, 5, 6):
            out.append(case(INDEL, DISTANCE, FREE, a, b, c, cite=T + ":222-247"))
    out.append(case(INDEL, NORM_SIMILARITY, FREE, "001", "220", cite=T + ":249-256"))
    out.append(case(INDEL, NORM_SIMILARITY, CACHED, "001", "220", cite=T + ":249-256"))
    s1 = "ddccbccc"
    s2 = ("aaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaa"
          "aaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaccacccaccaaaaaaaa"
          "daaaaaaaaccccaccccccaaaaaaaccccaaacccaccccadddaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaa"
          "aaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaaccccccccacccaaaaaacccaaaaaacccacccaaaaaacccdccc"
          "cccacccccccccccccccccccccccccccccccccccccccccccccccccccccccccccccddddddaaaaaaaa"
          "aaaaaaaaaaaaaaaaaacacccaaaaaacccddddaaaaaaaaaaaaaaaaaaaaaaaaaaaaaccccaaaaaaaaaa"
          "ccccccaadddaaaaaaaaaaaaaaaaaaaaaacaaaaaa")
    for c in (None, 508, 507, 2**64 - 1):
        out.append(case(INDEL, DISTANCE, FREE, s1, s2, c, cite=T + ":258-272"))
    a = ("bbbdbbmbbbbbbbbbBbfbbbbbbbbbbbbbbbbbbbrbbbbbrbbbbbdbnbbbjbhbbbbbbbbbhbbbbbCbobb"
         "bxbbbbbkbbbAbxbbwbbbtbcbbbbebbiblbbbbqbbbbbbpbbbbbbubbbkbbDbbbhbkbCbbgbbrbbbbbb"
         "bbbbbkbyvbbsbAbbbbz")
    b = "jaaagaaqyaaaanrCfwaaxaeahtaaaCzaaaspaaBkvaaaaqDaacndaaeolwiaaauaaaaaaamA"
    out.append(case(INDEL, DISTANCE, FREE, a, b, cite=T + ":274-283"))
    # LCSseq (tests-LCSseq.cpp:148-204)
    T = "test/distance/tests-LCSseq.cpp"
    for op in OPS:
        out.append(case(LCSSEQ, op, FREE, "aaaa", "aaaa", cite=T + ":152-164"))
        out.append(case(LCSSEQ, op, FREE, "aaaa", "bbbb", cite=T + ":152-164"))
    for a, b in (("South Korea", "North Korea"), ("aabc", "cccd")):
        for c in (None, 0, 1, 2, 3, 4, 9, 10):
            out.append(case(LCSSEQ, SIMILARITY, FREE, a, b, c, cite=T + ":166-196"))
            out.append(case(LCSSEQ, DISTANCE, FREE, a, b, c, cite=T + ":166-196"))
    out.append(case(LCSSEQ, SIMILARITY, CACHED, "001", "220", cite=T + ":198-204"))
    # OSA (tests-OSA.cpp:55-97)
    T = "test/distance/tests-OSA.cpp"
    for a, b, c in (("", "", None), ("aaaa", "", None), ("", "aaaa", None), ("aaaa", "", 1), ("", "aaaa", 1),
                    ("CA", "ABC", None), ("CA", "AC", None)):
        out.append(case(OSA, DISTANCE, FREE, a, b, c, cite=T + ":59-86"))
        out.append(case(OSA, DISTANCE, CACHED, a, b, c, cite=T + ":59-86"))
    filler = "a" * 64
    out.append(case(OSA, DISTANCE, FREE, "a" + filler + "CA" + filler + "a", "b" + filler + "AC" + filler + "b",
                    cite=T + ":88-96"))
    out.append(case(OSA, DISTANCE, CACHED, "a" + filler + "CA" + filler + "a", "b" + filler + "AC" + filler + "b",
                    cite=T + ":88-96"))
    # Jaro / Jaro-Winkler names x names x cutoffs (tests-Jaro.cpp:160-170, tests-JaroWinkler.cpp:128-174)
    names = ["james", "robert", "john", "michael", "william", "david", "joseph", "thomas", "charles", "mary",
             "patricia", "jennifer", "linda", "elizabeth", "barbara", "susan", "jessica", "sarah", "karen", ""]
    cuts = (0.1, 0.5, 0.7, 0.8, 0.9, 1.0, 1.1)
    rng = random.Random(7)
    for metric, T in ((JARO, "test/distance/tests-Jaro.cpp:160-170"),
                      (JARO_WINKLER, "test/distance/tests-JaroWinkler.cpp:128-174")):
        for n1 in names:
            for n2 in names:
                c = rng.choice(cuts)
                out.append(case(metric, SIMILARITY, FREE, n1, n2, c, cite=T))
                out.append(case(metric, DISTANCE, CACHED, n1, n2, round(1.0 - c, 10), cite=T))
    # edge lengths (tests-Jaro.cpp:172-231, tests-JaroWinkler.cpp:177-216)
    edge = [("", ""), ("0", "0"), ("00", "00"), ("0", "00"), ("0" * 65, "0" * 65), ("0" * 64, "0" * 65),
            ("0" * 63, "0" * 65), ("000000001", "0000010"), ("01234567", "0" * 170 + "7654321" + "0" * 200),
            ("01", "1111100000"),
            ("1" + "0" * 62 + "20", "0" * 65),
            ("0" * 14 + "1" + "0" * 24 + "1" + "0" * 25, "0" * 78 + "1"),
            ("0" * 65, "01" + "0" * 126)]
    for metric, T in ((JARO, "test/distance/tests-Jaro.cpp:172-231"),
                      (JARO_WINKLER, "test/distance/tests-JaroWinkler.cpp:177-216")):
        for a, b in edge:
            for form in (FREE, CACHED):
                out.append(case(metric, SIMILARITY, form, a, b, cite=T))
                out.append(case(metric, SIMILARITY, form, b, a, cite=T))
    # MultiJaro fuzz regression (tests-Jaro.cpp:233-256): covered in multi.json
    # fuzz::ratio (test/tests-fuzz.cpp:52-74)
    T = "test/tests-fuzz.cpp:52-74"
    fz = ["new york mets", "new YORK mets", "the wonderful new york mets", "new york mets vs atlanta braves",
          "atlanta braves vs new york mets", "new york mets - atlanta braves", "new york city mets - atlanta braves",
          "{", "{a", "a{", "{b", "test"]
    for a in fz:
        for b in fz:
            out.append(case(RATIO, SIMILARITY, FREE, a, b, cite=T))
            out.append(case(RATIO, SIMILARITY, CACHED, a, b, 85.0, cite=T))
    return [c for c in out if c is not None]


def rand_str(rng, alpha, lo, hi):
    return [rng.choice(alpha) for _ in range(rng.randint(lo, hi))]


def mutate(rng, s, alpha, k):
    s = list(s)
    for _ in range(k):
        op = rng.randint(0, 3)
        if op == 0 and s:
            s[rng.randrange(len(s))] = rng.choice(alpha)
        elif op == 1:
            s.insert(rng.randint(0, len(s)), rng.choice(alpha))
        elif op == 2 and s:
            del s[rng.randrange(len(s))]
        elif op == 3 and len(s) > 1:
            i = rng.randrange(len(s) - 1)
            s[i], s[i + 1] = s[i + 1], s[i]
    return s


ALPHABETS = [[65, 67, 71, 84], list(range(97, 123)), [97, 98], list(range(0, 256)), [97, 98, 300, 70000],
             [1000, 1001, 1002], [0x41, 0xC0, 0xC9, 0xFF, 0x20], [2**40 + 1, 2**40 + 2, 5]]


def random_cases(n, seed=1):
    rng = random.Random(seed)
    out = []
    while len(out) < n:
        alpha = rng.choice(ALPHABETS)
        maxlen = rng.choice([4, 8, 16, 40, 63, 64, 65, 100, 128, 129, 200, 300])
        s1 = rand_str(rng, alpha, 0, maxlen)
        s2 = mutate(rng, s1, alpha, rng.randint(0, 12)) if rng.random() < 0.6 else rand_str(rng, alpha, 0, maxlen)
        if rng.random() < 0.5:
            s1, s2 = s2, s1
        mx1, mx2 = max(s1 + [0]), max(s2 + [0])
        w1 = 8 if mx1 >= 2**32 else (4 if mx1 >= 65536 else rng.choice([1, 2, 4, 8]) if mx1 < 256 else rng.choice([2, 4]) if mx1 < 65536 else 4)
        w2 = 8 if mx2 >= 2**32 else (4 if mx2 >= 65536 else rng.choice([1, 2, 4, 8]) if mx2 < 256 else rng.choice([2, 4]) if mx2 < 65536 else 4)
        metric = rng.randrange(7)
        op = SIMILARITY if metric == RATIO else rng.randrange(4)
        form = rng.choice([FREE, CACHED, MULTI])
        if form == MULTI and len(s1) > 64:
            form = CACHED
        weights = (1, 1, 1)
        if metric == LEVENSHTEIN:
            weights = rng.choice([(1, 1, 1), (1, 1, 1), (1, 1, 2), (2, 2, 2), (1, 2, 3), (3, 1, 1), (2, 2, 5),
                                  (0, 0, 1), (1, 1, 0)])
            if form == MULTI and weights not in ((1, 1, 1), (1, 1, 2), (1, 1, 0)):
                weights = (1, 1, 1)
        if result_is_int(metric, op):
            cutoff = rng.choice([None, 0, 1, 2, 3, 4, 5, 8, 10, 31, 32, 40, 64, 100, 1000])
        else:
            cutoff = rng.choice([None, 0.0, 0.1, 0.5, 0.7, 0.8, 0.85, 0.9, 0.95, 1.0, 1.1])
            if metric == RATIO and cutoff is not None:
                cutoff = cutoff * 100
        pw = rng.choice([0.1, 0.1, 0.25])
        c = case(metric, op, form, s1, s2, cutoff, weights, pw, w1, w2)
        if c is not None:
            out.append(c)
    return out


def multi_cases(seed=3):
    """Multi* batches (8-bit code units; the reference driver's Multi entry takes bytes)."""
    ref = reference()
    rng = random.Random(seed)
    out = []

    def run(metric, op, max_len, strs, s2, cutoff, weights=(1, 1, 1), pw=0.1, cite=None):
        data, offsets, width = pack_strings([as_units(bytes(s)) for s in strs], 1)
        st = strings_struct(data, offsets, width)
        b = as_units(bytes(s2))
        n = len(strs)
        oi = np.zeros(max(n, 1), dtype=np.int64)
        of = np.zeros(max(n, 1), dtype=np.float64)
        rc = ctypes.c_int64()
        p = make_params(weights, pw)
        is_int = result_is_int(metric, op)
        ci = (2**63 - 1 if op == DISTANCE else 0) if (cutoff is None or not is_int) else int(cutoff)
        cf = (1.0 if op in (DISTANCE, NORM_DISTANCE) and metric < RATIO else 0.0) if (cutoff is None or is_int) \
            else float(cutoff)
        r = ref.rfref_multi(metric, op, max_len, ctypes.byref(st), b.ctypes.data if b.size else None, b.size, 1,
                            ctypes.byref(p), ci, cf, oi.ctypes.data, of.ctypes.data, ctypes.byref(rc))
        if r != 0:
            return
        vals = [int(v) for v in oi[:n]] if is_int else [float(v).hex() for v in of[:n]]
        d = {"metric": metric, "op": op, "max_len": max_len, "strs": [list(s) for s in strs], "s2": list(s2),
             "cutoff": cutoff, "weights": list(weights), "pw": pw, "result_count": rc.value, "expected": vals}
        if cite:
            d["cite"] = cite
        out.append(d)

    # MultiJaro fuzz regression (tests-Jaro.cpp:233-256)
    s2 = b"01" * 133
    run(JARO, SIMILARITY, 8, [b"10010010"] * 32 + [b"00100100"], s2, 0.0, cite="test/distance/tests-Jaro.cpp:233-256")
    # SIMD wraparound (tests-LCSseq.cpp:207-244)
    for k in (256, 300, 512):
        run(LCSSEQ, DISTANCE, 8, [b"a", b"b", b"aa", b"bb"], b"b" * k, None,
            cite="test/distance/tests-LCSseq.cpp:207-244")
    for _ in range(120):
        metric = rng.randrange(7)
        op = SIMILARITY if metric == RATIO else rng.randrange(4)
        max_len = rng.choice([8, 16, 32, 64])
        alpha = rng.choice([[65, 67, 71, 84], list(range(97, 123)), [97, 98]])
        count = rng.randint(1, 70)
        base = rand_str(rng, alpha, 0, max_len)
        strs = [bytes(mutate(rng, base, alpha, rng.randint(0, 4))[:max_len]) if rng.random() < 0.5
                else bytes(rand_str(rng, alpha, 0, max_len)) for _ in range(count)]
        s2 = bytes(mutate(rng, base, alpha, rng.randint(0, 6)) if rng.random() < 0.6 else rand_str(rng, alpha, 0, 90))
        weights = rng.choice([(1, 1, 1), (1, 1, 2)]) if metric == LEVENSHTEIN else (1, 1, 1)
        if result_is_int(metric, op):
            cutoff = rng.choice([None, 0, 2, 5, 10])
        else:
            cutoff = rng.choice([None, 0.0, 0.5, 0.8, 0.9, 1.0])
            if metric == RATIO and cutoff is not None:
                cutoff *= 100
        run(metric, op, max_len, strs, s2, cutoff, weights, rng.choice([0.1, 0.2]))
    # MultiTokenSortRatio / MultiQRatio: whitespace-rich inserted strings (MaxLen bounds
    # the raw string, so the join fits too), empty strings on both sides
    trng = random.Random(seed + 100)
    for _ in range(60):
        metric = trng.choice([TOKEN_SORT_RATIO, QRATIO])
        max_len = trng.choice([8, 16, 32, 64])
        alpha = [97, 98, 99, 32, 32, 9]
        strs = [bytes(rand_str(trng, alpha, 0, max_len)) for _ in range(trng.randint(1, 40))]
        s2 = bytes(rand_str(trng, alpha, 0, 70)) if trng.random() < 0.85 else b""
        cutoff = trng.choice([None, 0.0, 50.0, 80.0, 100.0])
        run(metric, SIMILARITY, max_len, strs, s2, cutoff)
    return out


def fuzz_test_literals():
    """the string literals of test/tests-fuzz.cpp (adjacent literals joined as C++ does)"""
    import re
    text = open(os.path.join(REF_ROOT, "test", "tests-fuzz.cpp"), encoding="utf-8").read()
    lits, cur, last_end = [], None, -1
    for mt in re.finditer(r'"((?:[^"\\]|\\.)*)"', text):
        gap = text[last_end:mt.start()] if last_end >= 0 else "x"
        val = bytes(mt.group(1), "utf-8").decode("unicode_escape")
        if cur is not None and gap.strip() == "":
            cur += val
        else:
            if cur is not None:
                lits.append(cur)
            cur = val
        last_end = mt.end()
    if cur is not None:
        lits.append(cur)
    seen, out = set(), []
    for x in lits:
        if x not in seen and "::" not in x and "%" not in x:
            seen.add(x)
            out.append(x)
    return out


def partial_cases(seed=11):
    """fuzz::partial_ratio / CachedPartialRatio: the inputs of the reference's fuzz tests
    (test/tests-fuzz.cpp, its partial_ratio sections and issue regressions) paired
    with each other, then seeded random pairs (needle lengths 0..130, haystacks 0..300,
    every char width, cutoffs 0..101)."""
    T = "test/tests-fuzz.cpp"
    lits = fuzz_test_literals()
    out = []
    for i, a in enumerate(lits):
        for b in (lits[i], lits[(i + 1) % len(lits)], lits[(i + 3) % len(lits)]):
            out.append(case(PARTIAL_RATIO, SIMILARITY, FREE, a, b, cite=T))
            out.append(case(PARTIAL_RATIO, SIMILARITY, CACHED, b, a, 50.0, cite=T))
    rng = random.Random(seed)
    while len(out) < 3000:
        alpha = rng.choice(ALPHABETS)
        n1 = rng.choice([0, 1, 2, 3, 5, 8, 16, 31, 40, 63, 64, 65, 100, 130])
        n2 = rng.choice([0, 1, 4, 16, 40, 64, 65, 100, 200, 300])
        s1 = rand_str(rng, alpha, 0, n1)
        if rng.random() < 0.5 and len(s1) < 300:
            s2 = rand_str(rng, alpha, 0, n2)
            at = rng.randint(0, len(s2))
            s2 = s2[:at] + mutate(rng, s1, alpha, rng.randint(0, 4)) + s2[at:]
        else:
            s2 = rand_str(rng, alpha, 0, n2)
        if rng.random() < 0.3:
            s1, s2 = s2, s1
        mx1, mx2 = max(s1 + [0]), max(s2 + [0])
        w1 = 8 if mx1 >= 2**32 else (4 if mx1 >= 65536 else rng.choice([1, 2, 4]) if mx1 < 256 else 2 if mx1 < 65536 else 4)
        w2 = 8 if mx2 >= 2**32 else (4 if mx2 >= 65536 else rng.choice([1, 2, 4]) if mx2 < 256 else 2 if mx2 < 65536 else 4)
        cutoff = rng.choice([None, 0.0, 30.0, 50.0, 70.0, 85.0, 95.0, 100.0, 101.0])
        c = case(PARTIAL_RATIO, SIMILARITY, rng.choice([FREE, CACHED]), s1, s2, cutoff, w1=w1, w2=w2)
        if c is not None:
            out.append(c)
    return [c for c in out if c is not None]


def token_cases(seed=13):
    """fuzz::token_sort_ratio / partial_token_sort_ratio / QRatio and their Cached forms:
    the reference fuzz tests' inputs (test/tests-fuzz.cpp) paired with each other, then
    seeded random token strings (every char width, ASCII and, for wider units, Unicode
    whitespace between tokens, cutoffs 0..101)."""
    T = "test/tests-fuzz.cpp"
    metrics = (TOKEN_SORT_RATIO, PARTIAL_TOKEN_SORT_RATIO, QRATIO)
    lits = fuzz_test_literals()
    out = []
    for i, a in enumerate(lits):
        for b in (lits[i], lits[(i + 1) % len(lits)], lits[(i + 5) % len(lits)]):
            for m in metrics:
                out.append(case(m, SIMILARITY, FREE, a, b, cite=T))
                out.append(case(m, SIMILARITY, CACHED, b, a, 50.0, cite=T))
    rng = random.Random(seed)
    spaces = [0x20, 0x09, 0x0A, 0x0D, 0x1F, 0x85, 0xA0, 0x2000, 0x2028, 0x3000]
    while len(out) < 4000:
        w = rng.choice([1, 2, 4, 8])
        letters = [97, 98, 99, 100, 101, 0xC0, 0xFF] + ([300, 4000, 70000] if w == 4 else [300] if w == 2 else [])
        sp = [c for c in spaces if w > 1 or c < 256]

        def mk():
            s = []
            for _ in range(rng.randint(0, 7)):
                s += [rng.choice(letters) for _ in range(rng.randint(0, 9))]
                s += [rng.choice(sp) for _ in range(rng.randint(0, 2))]
            return s
        a, b = mk(), mk()
        if rng.random() < 0.3:
            b = list(a)
            rng.shuffle(b)
        cutoff = rng.choice([None, 0.0, 50.0, 80.0, 95.0, 100.0, 101.0])
        c = case(rng.choice(metrics), SIMILARITY, rng.choice([FREE, CACHED]), a, b, cutoff, w1=w, w2=w)
        if c is not None:
            out.append(c)
    return [c for c in out if c is not None]


def tokenset_cases(seed=17):
    """token_set_ratio / partial_token_set_ratio / token_ratio / partial_token_ratio / WRatio
    and their Cached forms: the reference fuzz tests' inputs (test/tests-fuzz.cpp) paired
    with each other, then seeded random strings drawn from small vocabularies (shared and
    repeated tokens), every char width, ASCII and Unicode whitespace, length ratios on
    both sides of WRatio's 1.5 and 8 thresholds, cutoffs 0..100.5."""
    T = "test/tests-fuzz.cpp"
    metrics = (TOKEN_SET_RATIO, PARTIAL_TOKEN_SET_RATIO, TOKEN_RATIO, PARTIAL_TOKEN_RATIO, WRATIO)
    lits = fuzz_test_literals()
    out = []
    for i, a in enumerate(lits):
        for b in (lits[i], lits[(i + 1) % len(lits)], lits[(i + 3) % len(lits)]):
            for m in metrics:
                out.append(case(m, SIMILARITY, FREE, a, b, cite=T))
                out.append(case(m, SIMILARITY, CACHED, b, a, 50.0, cite=T))
    rng = random.Random(seed)
    spaces = [0x20, 0x09, 0x0A, 0x1C, 0x85, 0xA0, 0x2000, 0x3000]
    while len(out) < 5000:
        w = rng.choice([1, 2, 4, 8])
        letters = [97, 98, 99, 100, 0xC0] + ([300, 4000, 70000] if w == 4 else [300] if w == 2 else [])
        sp = [c for c in spaces if w > 1 or c < 256]
        vocab = [[rng.choice(letters) for _ in range(rng.randint(1, 5))] for _ in range(rng.randint(1, 8))]

        def mk(k):
            s = []
            for _ in range(k):
                s += list(rng.choice(vocab)) if rng.random() < 0.7 else \
                    [rng.choice(letters) for _ in range(rng.randint(0, 6))]
                s += [rng.choice(sp) for _ in range(rng.randint(0, 2))]
            return s
        a = mk(rng.randint(0, 6))
        b = mk(rng.choice([rng.randint(0, 6), rng.randint(0, 25)]))
        if rng.random() < 0.2:
            b = list(a)
            rng.shuffle(b)
        if rng.random() < 0.3:
            a, b = b, a
        cutoff = rng.choice([None, 0.0, 30.0, 50.0, 80.0, 90.0, 100.0, 100.5])
        c = case(rng.choice(metrics), SIMILARITY, rng.choice([FREE, CACHED]), a, b, cutoff, w1=w, w2=w)
        if c is not None:
            out.append(c)
    return [c for c in out if c is not None]


def literals_in(path, first, last):
    """the string literals of lines first..last of a reference test file"""
    import re
    lines = open(os.path.join(REF_ROOT, path), encoding="utf-8").read().split("\n")[first - 1:last]
    return [bytes(m, "utf-8").decode("unicode_escape") for m in re.findall(r'"((?:[^"\\]|\\.)*)"', "\n".join(lines))]


def editops_cases(seed=19):
    """levenshtein_editops / indel_editops / lcs_seq_editops of the reference itself: the
    string literals of its editops tests (test/distance/tests-Levenshtein.cpp:235-320)
    paired with each other and repeated, then seeded random pairs (copies with edits,
    unrelated strings; every char width; lengths 0..600; score hints none / 0 / 50)."""
    from oracle_lib import editops as eops, oracle
    ref, o = reference(), oracle()
    T = "test/distance/tests-Levenshtein.cpp"
    out = []

    def add(metric, a, b, w, hint=None, cite=None):
        a, b = as_units(a, w), as_units(b, w)
        exp = eops(ref.rfref_editops, metric, a, b, hint)
        d = {"metric": metric, "s1": [int(x) for x in a], "s2": [int(x) for x in b], "w": int(a.itemsize),
             "hint": hint, "expected": [list(x) for x in exp]}
        if cite:
            d["cite"] = cite
        out.append(d)
    lits = literals_in(T, 235, 320)
    for i, x in enumerate(lits):
        for y in (lits[(i + 1) % len(lits)], x * 3, lits[(i + 2) % len(lits)] * 5):
            for metric in (LEVENSHTEIN, INDEL, LCSSEQ):
                add(metric, x, y, 1, cite=T + ":235-320")
    rng = random.Random(seed)
    while len(out) < 3000:
        w = rng.choice([1, 2, 4])
        alpha = rng.choice([[97, 98], [97, 98, 99, 100], list(range(97, 123))]) + ([300, 70000] if w == 4 else [])
        la = rng.choice([0, 1, 5, 20, 63, 64, 65, 130, 300, 600])
        a = [rng.choice(alpha) for _ in range(rng.randint(0, la))]
        b = list(a)
        for _ in range(rng.choice([rng.randint(0, 5), rng.randint(0, 80)])):
            k = rng.random()
            if k < 0.3 and b:
                b[rng.randrange(len(b))] = rng.choice(alpha)
            elif k < 0.6:
                b.insert(rng.randint(0, len(b)), rng.choice(alpha))
            elif b:
                del b[rng.randrange(len(b))]
        if rng.random() < 0.25:
            b = [rng.choice(alpha) for _ in range(rng.randint(0, la + 10))]
        add(rng.choice([LEVENSHTEIN, INDEL, LCSSEQ]), a, b, w, rng.choice([None, 0, 50]))
    # long Levenshtein pairs: the reference's Hirschberg recursion (Levenshtein_impl.hpp:1184-1257)
    for k in range(24):
        alpha = rng.choice([[97, 98], [97, 98, 99, 100], list(range(97, 123))])
        a = [rng.choice(alpha) for _ in range(rng.choice([1100, 1600, 2300]))]
        b = list(a)
        for _ in range(rng.choice([rng.randint(0, 20), rng.randint(0, 400)])):
            k2 = rng.random()
            if k2 < 0.3 and b:
                b[rng.randrange(len(b))] = rng.choice(alpha)
            elif k2 < 0.6:
                b.insert(rng.randint(0, len(b)), rng.choice(alpha))
            elif b:
                del b[rng.randrange(len(b))]
        add(LEVENSHTEIN, a, b, 1, [None, 0, 50][k % 3], cite="Levenshtein_impl.hpp:1184-1257 (Hirschberg)")
    return out


def opcodes_cases(limit=600):
    """Opcodes(Editops), Editops(Opcodes) and the two applies (details/types.hpp:500-569,
    distance.hpp:19-165) of the reference on the one-byte pairs of editops.json whose
    strings hold at most 300 units together; each case names its editops.json index."""
    ref = reference()
    P, I64 = ctypes.c_void_p, ctypes.c_int64
    fn = ref.rfref_opcodes
    fn.restype = ctypes.c_int
    fn.argtypes = [P, I64, P, I64, P, I64, P, I64, P, P, I64, P, P, P, P, P]
    with open(os.path.join(HERE, "editops.json")) as f:
        eops = json.load(f)
    out = []
    for i, c in enumerate(eops):
        if len(out) >= limit:
            break
        if c["w"] != 1 or len(c["s1"]) + len(c["s2"]) > 300:
            continue
        a = np.array(c["s1"], dtype=np.uint8)
        b = np.array(c["s2"], dtype=np.uint8)
        n = len(c["expected"])
        ops = np.zeros(max(n, 1), dtype=[("type", "<i4"), ("reserved", "<i4"), ("src_pos", "<i8"), ("dest_pos", "<i8")])
        for k, (t, sp, dp) in enumerate(c["expected"]):
            ops[k] = (t, 0, sp, dp)
        cap = 2 * (len(a) + len(b)) + 2
        opc = np.zeros(5 * cap, dtype=np.int64)
        back = np.zeros(cap, dtype=ops.dtype)
        ea = np.zeros(len(a) + len(b) + 1, dtype=np.uint8)
        oa = np.zeros(len(a) + len(b) + 1, dtype=np.uint8)
        cnt, bcnt, eal, oal = (ctypes.c_int64() for _ in range(4))
        assert fn(ops.ctypes.data, n, a.ctypes.data, len(a), b.ctypes.data, len(b), opc.ctypes.data, cap,
                  ctypes.byref(cnt), back.ctypes.data, cap, ctypes.byref(bcnt), ea.ctypes.data, ctypes.byref(eal),
                  oa.ctypes.data, ctypes.byref(oal)) == 0
        assert cnt.value <= cap and bcnt.value <= cap
        out.append({"case": i,
                    "opcodes": opc[:5 * cnt.value].reshape(-1, 5).tolist(),
                    "back": [[int(x["type"]), int(x["src_pos"]), int(x["dest_pos"])] for x in back[:bcnt.value]],
                    "editops_apply": ea[:eal.value].tolist(), "opcodes_apply": oa[:oal.value].tolist()})
    return out


def listops_cases(limit=300, seed=23):
    """Editops slice / remove_slice / reverse / inverse / remove_subsequence and Opcodes
    slice / reverse / inverse (details/types.hpp:109-161, 240-320, 420-475) of the
    reference on operation lists of editops.json, with seeded slice bounds (negative,
    past the end, empty) and steps 1..3 (step 0 and negative steps: the reference's
    invalid_argument, recorded as null)."""
    ref = reference()
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    fn = ref.rfref_list_op
    fn.restype = I
    fn.argtypes = [I, P, I64, I64, I64, I, I, I, P, I64, P, P]
    with open(os.path.join(HERE, "editops.json")) as f:
        eops = json.load(f)
    rng = random.Random(seed)
    picks = [i for i, c in enumerate(eops) if len(c["expected"]) <= 60]
    rng.shuffle(picks)
    out = []
    for i in picks[:limit]:
        c = eops[i]
        n = len(c["expected"])
        ops = np.zeros(max(n, 1), dtype=[("type", "<i4"), ("reserved", "<i4"), ("src_pos", "<i8"), ("dest_pos", "<i8")])
        for k, (t, sp, dp) in enumerate(c["expected"]):
            ops[k] = (t, 0, sp, dp)
        for which in (0, 1, 2, 3, 4, 10, 12, 13):
            start = rng.choice([0, 1, 2, -1, -3, n // 2, n, n + 5, -n - 5])
            stop = rng.choice([n, n - 1, 1, -1, -2, n // 2, n + 5, 0])
            step = rng.choice([1, 1, 2, 3, 0, -1]) if which in (0, 1, 4, 10) else 1
            cap = 2 * (len(c["s1"]) + len(c["s2"])) + 4
            res = np.zeros(5 * cap, dtype=np.int64)
            cnt = ctypes.c_int64()
            lens = np.zeros(2, dtype=np.int64)
            rc = fn(which, ops.ctypes.data, n, len(c["s1"]), len(c["s2"]), start, stop, step, res.ctypes.data, cap,
                    ctypes.byref(cnt), lens.ctypes.data)
            rec = 3 if which < 10 else 5
            out.append({"case": i, "which": which, "start": start, "stop": stop, "step": step,
                        "result": None if rc else res[:rec * cnt.value].reshape(-1, rec).tolist(),
                        "lens": None if rc else lens.tolist()})
    return out


def main():
    if reference() is None:
        sys.exit("oracle/_ref/librfref.so is missing: run `make -C oracle ref` where the reference checkout exists")
    which = sys.argv[1:] or ["kat.json", "random.json", "multi.json", "partial.json", "tokens.json", "tokenset.json",
                             "editops.json", "opcodes.json", "listops.json"]
    gens = {"kat.json": kat_cases, "random.json": lambda: random_cases(4000), "multi.json": multi_cases,
            "partial.json": partial_cases, "tokens.json": token_cases, "tokenset.json": tokenset_cases,
            "editops.json": editops_cases, "opcodes.json": opcodes_cases, "listops.json": listops_cases}
    for name, cases in ((n, gens[n]()) for n in which):
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(cases, f, separators=(",", ":"))
        print(name, len(cases))


if __name__ == "__main__":
    main()
