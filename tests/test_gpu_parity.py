"""Parity of the CUDA path with the reference: every result bit-exact (integers) or
bit-identical (doubles) -- tolerance 0.  Calls go through the C ABI."""
import random

import numpy as np
import pytest

import golden_lib as G
from oracle_lib import oracle, oracle_cdist, score as oscore, FREE, CACHED, MULTI

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402


def gpu_score(c, a, b):
    m, op, form = c["metric"], c["op"], c["form"]
    w, pw, cut = tuple(c["weights"]), c["pw"], c["cutoff"]
    if form == FREE:
        return R.score(m, op, a, b, cut, None, w, pw)
    if form == CACHED:
        return R.Cached(m, a, w, pw).score(op, b, cut)
    ml = 8 if a.size <= 8 else 16 if a.size <= 16 else 32 if a.size <= 32 else 64
    mu = R.Multi(m, ml, 1, w, pw)
    mu.insert(a)
    v = mu.score(op, b, cut)[0]
    return int(v) if R._lib.result_is_int(m, op) else float(v)


@pytest.mark.parametrize("fixture", ["kat.json", "random.json", "partial.json", "tokens.json", "tokenset.json"])
def test_fixtures_per_call(fixture):
    bad = []
    for c in G.load(fixture):
        a, b = G.arrays(c)
        v = gpu_score(c, a, b)
        if not G.same(v, G.dec(c["expected"])):
            bad.append((c.get("cite"), c["metric"], c["op"], c["form"], c["cutoff"], len(a), len(b), v,
                        G.dec(c["expected"])))
    assert not bad, "%d mismatches: %r" % (len(bad), bad[:5])


def test_multi_batches():
    for c in G.load("multi.json"):
        mu = R.Multi(c["metric"], c["max_len"], len(c["strs"]), tuple(c["weights"]), c["pw"])
        for s in c["strs"]:
            mu.insert(bytes(s))
        assert mu.result_count() == c["result_count"]
        out = mu.score(c["op"], bytes(c["s2"]), c["cutoff"])
        for i, exp in enumerate(c["expected"]):
            v = out[i].item()
            assert G.same(v, G.dec(exp)), (c.get("cite"), c["metric"], c["op"], i, v, exp)


def _rand(rng, alpha, lo, hi):
    return [rng.choice(alpha) for _ in range(rng.randint(lo, hi))]


def _mut(rng, s, alpha, k):
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


def _batch(rng, alpha, n, lo, hi, width, base=None):
    out = []
    for _ in range(n):
        if base and rng.random() < 0.4:
            out.append(_mut(rng, rng.choice(base), alpha, rng.randint(0, 8)))
        else:
            out.append(_rand(rng, alpha, lo, hi))
    return R.pack_strings([np.array(s, dtype={1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[width])
                           for s in out], width), out


CASES = [
    # metric, op, cutoff
    (R.LEVENSHTEIN, R.DISTANCE, None), (R.LEVENSHTEIN, R.DISTANCE, 8), (R.LEVENSHTEIN, R.SIMILARITY, 20),
    (R.LEVENSHTEIN, R.NORMALIZED_SIMILARITY, 0.7), (R.LEVENSHTEIN, R.NORMALIZED_DISTANCE, 0.2),
    (R.INDEL, R.DISTANCE, 8), (R.INDEL, R.NORMALIZED_SIMILARITY, 0.6), (R.LCSSEQ, R.SIMILARITY, 10),
    (R.LCSSEQ, R.DISTANCE, 12), (R.OSA, R.DISTANCE, 8), (R.OSA, R.NORMALIZED_SIMILARITY, 0.5),
    (R.JARO, R.SIMILARITY, 0.7), (R.JARO_WINKLER, R.SIMILARITY, 0.85), (R.JARO_WINKLER, R.NORMALIZED_DISTANCE, 0.3),
    (R.RATIO, R.SIMILARITY, 85.0), (R.RATIO, R.SIMILARITY, 0.0),
]


@pytest.mark.parametrize("metric,op,cut", CASES)
@pytest.mark.parametrize("shape", ["short", "multiword", "mixed", "wide"])
def test_cdist_matches_oracle(metric, op, cut, shape):
    rng = random.Random(hash((metric, op, shape)) & 0xffff)
    if shape == "short":
        alpha, qlo, qhi, clo, chi, w = list(range(97, 123)), 0, 64, 0, 80, 1
    elif shape == "multiword":
        alpha, qlo, qhi, clo, chi, w = [65, 67, 71, 84], 65, 512, 50, 600, 1
    elif shape == "mixed":
        alpha, qlo, qhi, clo, chi, w = [97, 98, 99], 0, 700, 0, 700, 1
    else:
        alpha, qlo, qhi, clo, chi, w = [0x41, 0xC0, 0xFF, 0x20, 300, 70000, 1000], 0, 140, 0, 140, 4
    (qd, qo, qw), qs = _batch(rng, alpha, 23, qlo, qhi, w)
    (cd, co, cw), _ = _batch(rng, alpha, 57, clo, chi, w, base=qs)
    weights = (1, 1, 1)
    got = R.cdist(metric, op, (qd, qo, qw), (cd, co, cw), cut, weights)
    exp = oracle_cdist(metric, op, (qd, qo, qw), (cd, co, cw), cut, weights)
    assert got.dtype == exp.dtype
    bad = np.argwhere(got.view(np.int64) != exp.view(np.int64)) if got.dtype == np.float64 else np.argwhere(got != exp)
    assert bad.size == 0, "mismatch at %r: got %r exp %r" % (bad[0], got[tuple(bad[0])], exp[tuple(bad[0])])


@pytest.mark.parametrize("weights", [(1, 1, 1), (1, 1, 2), (2, 2, 2), (1, 2, 3), (3, 1, 1), (0, 0, 5)])
def test_cdist_weighted_levenshtein(weights):
    rng = random.Random(sum(weights))
    (qd, qo, qw), qs = _batch(rng, list(range(97, 110)), 9, 0, 150, 1)
    (cd, co, cw), _ = _batch(rng, list(range(97, 110)), 17, 0, 150, 1, base=qs)
    for op, cut in ((R.DISTANCE, None), (R.DISTANCE, 9), (R.SIMILARITY, 30), (R.NORMALIZED_SIMILARITY, 0.6)):
        got = R.cdist(R.LEVENSHTEIN, op, (qd, qo, qw), (cd, co, cw), cut, weights)
        exp = oracle_cdist(R.LEVENSHTEIN, op, (qd, qo, qw), (cd, co, cw), cut, weights)
        assert np.array_equal(got.view(np.int64), exp.view(np.int64)), (weights, op, cut)


def test_cdist_int32_output_and_ld():
    rng = random.Random(3)
    (qd, qo, qw), qs = _batch(rng, list(range(97, 123)), 11, 16, 64, 1)
    (cd, co, cw), _ = _batch(rng, list(range(97, 123)), 31, 16, 64, 1, base=qs)
    out = np.full((11, 40), -7, dtype=np.int32)
    R.cdist(R.OSA, R.DISTANCE, (qd, qo, qw), (cd, co, cw), 8, out_dtype=R.I32, out=out, ld=40)
    exp = oracle_cdist(R.OSA, R.DISTANCE, (qd, qo, qw), (cd, co, cw), 8, out_dtype=0)
    assert np.array_equal(out[:, :31], exp)
    assert (out[:, 31:] == -7).all()


def test_empty_batches_and_strings():
    assert R.cdist(R.LEVENSHTEIN, R.DISTANCE, [], ["abc"]).shape == (0, 1)
    assert R.cdist(R.LEVENSHTEIN, R.DISTANCE, ["abc"], []).shape == (1, 0)
    m = R.cdist(R.JARO_WINKLER, R.SIMILARITY, ["", "a", ""], ["", "a", "b"])
    o = oracle()
    for i, q in enumerate(["", "a", ""]):
        for j, c in enumerate(["", "a", "b"]):
            assert G.same(m[i, j].item(), oscore(o.rfo_score, R.JARO_WINKLER, R.SIMILARITY, CACHED, q, c))


def test_cached_score_many():
    rng = random.Random(8)
    q = bytes(_rand(rng, b"acgt", 100, 100))
    cs = [bytes(_mut(rng, q, b"acgt", rng.randint(0, 30))) for _ in range(300)]
    sc = R.Cached(R.LEVENSHTEIN, q)
    got = sc.score_many(R.DISTANCE, cs, 10)
    o = oracle()
    for j, c in enumerate(cs):
        assert got[j] == oscore(o.rfo_score, R.LEVENSHTEIN, R.DISTANCE, CACHED, q, c, 10)


def test_long_strings_any_length_kernel():
    """pattern > 512 code units: the any-length (scratch) kernel"""
    rng = random.Random(21)
    alpha = b"acgt"
    q = bytes(_rand(rng, alpha, 3000, 3000))
    cs = [bytes(_mut(rng, q, alpha, k)) for k in (0, 5, 50, 400)] + [bytes(_rand(rng, alpha, 2500, 3500))]
    o = oracle()
    for metric, op, cut in ((R.LEVENSHTEIN, R.DISTANCE, None), (R.LEVENSHTEIN, R.DISTANCE, 60),
                            (R.INDEL, R.DISTANCE, None), (R.OSA, R.DISTANCE, None), (R.LCSSEQ, R.SIMILARITY, 2000),
                            (R.JARO_WINKLER, R.SIMILARITY, 0.0), (R.JARO, R.SIMILARITY, 0.6)):
        got = R.cdist(metric, op, [q], cs, cut)
        for j, c in enumerate(cs):
            assert G.same(got[0, j].item(), oscore(o.rfo_score, metric, op, CACHED, q, c, cut)), (metric, op, j)


@pytest.mark.parametrize("metric", [R.LEVENSHTEIN, R.INDEL, R.OSA])
@pytest.mark.parametrize("width", [1, 2, 4])
def test_cdist_several_queries_per_thread(metric, width):
    """One-word unit-weight distances run several queries per thread: partial query
    groups, empty strings, choices holding code units the queries lack (>= 256), every
    output type"""
    rng = random.Random(1000 + metric * 10 + width)
    qalpha = list(range(97, 105))
    calpha = qalpha + ([300, 4000] if width > 1 else [200, 250])
    for nq in (1, 3, 4, 6, 9):
        qs = [_rand(rng, qalpha, 0, 64) for _ in range(nq)] + [[]]
        cs = [_mut(rng, rng.choice(qs), calpha, rng.randint(0, 6)) if rng.random() < 0.5 else _rand(rng, calpha, 0, 70)
              for _ in range(300)] + [[]]
        dt = {1: np.uint8, 2: np.uint16, 4: np.uint32}[width]
        q = R.pack_strings([np.array(s, dtype=dt) for s in qs], width)
        c = R.pack_strings([np.array(s, dtype=dt) for s in cs], width)
        for cut in (None, 0, 3, 8, 64):
            exp = oracle_cdist(metric, R.DISTANCE, q, c, cut)
            for out_dtype in (R.I32, R.I64):
                got = R.cdist(metric, R.DISTANCE, q, c, cut, out_dtype=out_dtype)
                assert np.array_equal(got.astype(np.int64), exp), (nq, cut, out_dtype)


@pytest.mark.parametrize("shape", ["short", "long", "wide"])
def test_cdist_partial_ratio_matches_oracle(shape):
    """fuzz::partial_ratio over batches: needles shorter, longer and equal to the
    haystacks, embedded near-copies, several cutoffs, the CachedPartialRatio form"""
    rng = random.Random({"short": 31, "long": 32, "wide": 33}[shape])
    if shape == "short":
        alpha, qlo, qhi, clo, chi, w = list(range(97, 103)), 0, 20, 0, 60, 1
    elif shape == "long":
        alpha, qlo, qhi, clo, chi, w = [65, 67, 71, 84], 30, 150, 0, 260, 1
    else:
        alpha, qlo, qhi, clo, chi, w = [0x41, 0xC0, 300, 70000, 0x20], 0, 40, 0, 90, 4
    qs = [_rand(rng, alpha, qlo, qhi) for _ in range(13)] + [[]]
    cs = []
    for _ in range(61):
        r = rng.random()
        if r < 0.4 and qs:
            base = rng.choice(qs)
            pre, post = _rand(rng, alpha, 0, 20), _rand(rng, alpha, 0, 20)
            cs.append(pre + _mut(rng, base, alpha, rng.randint(0, 3)) + post)
        elif r < 0.5:
            cs.append(list(rng.choice(qs)))
        else:
            cs.append(_rand(rng, alpha, clo, chi))
    cs.append([])
    dt = {1: np.uint8, 4: np.uint32}[w]
    q = R.pack_strings([np.array(s, dtype=dt) for s in qs], w)
    c = R.pack_strings([np.array(s, dtype=dt) for s in cs], w)
    for cut in (0.0, 50.0, 80.0, 100.0, 100.5):
        got = R.cdist(R.PARTIAL_RATIO, R.SIMILARITY, q, c, cut)
        exp = oracle_cdist(R.PARTIAL_RATIO, R.SIMILARITY, q, c, cut)
        bad = np.argwhere(got.view(np.int64) != exp.view(np.int64))
        assert bad.size == 0, "cut %r mismatch at %r: got %r exp %r" % (cut, bad[0], got[tuple(bad[0])],
                                                                        exp[tuple(bad[0])])


def test_partial_ratio_api_names():
    """the reference's names: fuzz::partial_ratio and CachedPartialRatio"""
    o = oracle()
    for a, b in (("001", "220222"), ("physics 2 vid", "study physics physics 2 video"), ("", ""), ("abc", "")):
        exp = oscore(o.rfo_score, R.PARTIAL_RATIO, R.SIMILARITY, FREE, a.encode(), b.encode(), 0.0)
        assert G.same(R.fuzz_partial_ratio(a, b), exp)
        assert G.same(R.CachedPartialRatio(a).similarity(b), exp)


def _token_str(rng, w):
    letters = [97, 98, 99, 100, 0xC0] + ([300, 70000] if w == 4 else [])
    spaces = [0x20, 0x09, 0x0A] + ([0xA0, 0x2000, 0x3000] if w == 4 else [])
    s = []
    for _ in range(rng.randint(0, 6)):
        s += [rng.choice(letters) for _ in range(rng.randint(0, 8))]
        s += [rng.choice(spaces) for _ in range(rng.randint(0, 2))]
    return s


def _token_batches(seed, w):
    """queries and choices for the token scorers: empty and all-whitespace strings,
    choices that are the queries' tokens reordered with other whitespace"""
    rng = random.Random(seed)
    qs = [_token_str(rng, w) for _ in range(17)] + [[], [0x20, 0x09]]
    cs = []
    for _ in range(70):
        if rng.random() < 0.35:
            toks = [t for t in "".join(chr(x) for x in rng.choice(qs)).split() if t]
            rng.shuffle(toks)
            cs.append([ord(ch) for ch in rng.choice([" ", "  ", "\t"]).join(toks)])
        else:
            cs.append(_token_str(rng, w))
    cs += [[], [0x20]]
    dt = {1: np.uint8, 4: np.uint32}[w]
    return (R.pack_strings([np.array(x, dtype=dt) for x in qs], w),
            R.pack_strings([np.array(x, dtype=dt) for x in cs], w))


@pytest.mark.parametrize("metric", ["TOKEN_SORT_RATIO", "PARTIAL_TOKEN_SORT_RATIO", "QRATIO"])
@pytest.mark.parametrize("width", [1, 4])
def test_cdist_token_scorers_match_oracle(metric, width):
    """token_sort_ratio, partial_token_sort_ratio and QRatio over batches (host joins,
    the ratio / partial_ratio kernels, QRatio's empty-string rule), free and cached forms"""
    m = getattr(R, metric)
    q, c = _token_batches(41 + width, width)
    for cut in (0.0, 60.0, 100.0, 101.0):
        exp = oracle_cdist(m, R.SIMILARITY, q, c, cut)
        for form in (R.FORM_FREE, R.FORM_CACHED):
            got = R.cdist(m, R.SIMILARITY, q, c, cut, form=form)
            bad = np.argwhere(got.view(np.int64) != exp.view(np.int64))
            assert bad.size == 0, "cut %r form %d mismatch at %r: got %r exp %r" % (
                cut, form, bad[0], got[tuple(bad[0])], exp[tuple(bad[0])])
    # CachedX.score_many (rfg_cached_score_many) for one query
    data, off, w = q
    s1 = data[off[3]:off[4]]
    got = R.Cached(m, s1).score_many(R.SIMILARITY, c, 50.0)
    exp = oracle_cdist(m, R.SIMILARITY, R.pack_strings([s1], w), c, 50.0)[0]
    assert np.array_equal(got.view(np.int64), exp.view(np.int64))


@pytest.mark.parametrize("metric", ["TOKEN_SORT_RATIO", "QRATIO"])
def test_cdist_token_scorers_device_buffers(metric):
    """device inputs (downloaded for the joins) and a device result with ld > choices
    (QRatio's zero fix-up runs as a kernel there)"""
    import ctypes
    import torch
    from rapidfuzz_gb300._lib import Cutoff, Strings, make_params, check
    m = getattr(R, metric)
    q, c = _token_batches(77, 1)
    exp = oracle_cdist(m, R.SIMILARITY, q, c, 0.0)
    dq = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in q[:2]]
    dc = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in c[:2]]
    nq, nc = q[1].size - 1, c[1].size - 1
    ld = nc + 5
    out = torch.full((nq, ld), -7.0, dtype=torch.float64, device="cuda")
    qs = Strings(dq[0].data_ptr(), dq[1].data_ptr(), nq, 1)
    cs = Strings(dc[0].data_ptr(), dc[1].data_ptr(), nc, 1)
    p = make_params()
    torch.cuda.synchronize()
    check(R.lib().rfg_cdist(m, R.SIMILARITY, R.FORM_CACHED, ctypes.byref(qs), ctypes.byref(cs), ctypes.byref(p),
                            Cutoff(0, 0.0, 0, 0.0), R.F64, out.data_ptr(), ld, R.DEVICE_INPUTS | R.DEVICE_OUTPUT))
    check(R.lib().rfg_synchronize())
    got = out.cpu().numpy()
    assert np.array_equal(got[:, :nc].view(np.int64), exp.view(np.int64))
    assert (got[:, nc:] == -7.0).all()


def test_token_scorer_api_names():
    """the reference's names (fuzz.hpp): token_sort_ratio, partial_token_sort_ratio,
    QRatio, their Cached classes, MultiTokenSortRatio and MultiQRatio"""
    o = oracle()
    pairs = (("new york mets", "new york mets"), ("new york mets vs atlanta braves", "atlanta braves vs new york mets"),
             ("", ""), ("abc", ""), ("  ", "a"), ("fuzzy wuzzy was a bear", "wuzzy fuzzy was a bear"))
    for a, b in pairs:
        for m, free, cached in ((R.TOKEN_SORT_RATIO, R.fuzz_token_sort_ratio, R.CachedTokenSortRatio),
                                (R.PARTIAL_TOKEN_SORT_RATIO, R.fuzz_partial_token_sort_ratio,
                                 R.CachedPartialTokenSortRatio),
                                (R.QRATIO, R.fuzz_QRatio, R.CachedQRatio)):
            exp = oscore(o.rfo_score, m, R.SIMILARITY, FREE, a.encode(), b.encode(), 0.0)
            assert G.same(free(a, b), exp), (m, a, b)
            assert G.same(cached(a).similarity(b), exp), (m, a, b)
    assert R.fuzz_token_sort_ratio("", "") == 100.0 and R.fuzz_QRatio("", "") == 0.0
    mt = R.experimental.MultiTokenSortRatio(16, 2)
    mt.insert("  c     b   a        ")
    mt.insert("b a")
    r = mt.similarity("a b c")
    assert r[0] == 100.0 and r[1] == 75.0
    mq = R.experimental.MultiQRatio(8, 2)
    mq.insert("")
    mq.insert("ab")
    assert list(mq.similarity("ab")[:2]) == [0.0, 100.0]
    assert list(mq.similarity("")[:2]) == [0.0, 0.0]
    with pytest.raises(ValueError):
        R.Multi(R.PARTIAL_TOKEN_SORT_RATIO, 8, 1)
    with pytest.raises(ValueError):
        R.score(R.TOKEN_SORT_RATIO, R.DISTANCE, "a", "b")


def _vocab_batches(seed, w, nq=23, nc=90):
    """strings drawn from a small vocabulary (shared and repeated tokens), some long
    choices, empty and all-whitespace strings"""
    rng = random.Random(seed)
    letters = [97, 98, 99, 100, 0xC0] + ([300, 70000] if w == 4 else [])
    spaces = [0x20, 0x09, 0x0A] + ([0xA0, 0x3000] if w == 4 else [])
    vocab = [[rng.choice(letters) for _ in range(rng.randint(1, 5))] for _ in range(10)]

    def mk(k):
        s = []
        for _ in range(k):
            s += list(rng.choice(vocab)) if rng.random() < 0.75 else [rng.choice(letters)
                                                                       for _ in range(rng.randint(1, 6))]
            s += [rng.choice(spaces) for _ in range(rng.randint(1, 2))]
        return s
    qs = [mk(rng.randint(0, 7)) for _ in range(nq - 2)] + [[], [0x20]]
    cs = [mk(rng.choice([rng.randint(0, 7), rng.randint(0, 40)])) for _ in range(nc - 2)] + [[], [0x09, 0x20]]
    dt = {1: np.uint8, 4: np.uint32}[w]
    return (R.pack_strings([np.array(x, dtype=dt) for x in qs], w),
            R.pack_strings([np.array(x, dtype=dt) for x in cs], w))


@pytest.mark.parametrize("metric", ["TOKEN_SET_RATIO", "PARTIAL_TOKEN_SET_RATIO", "TOKEN_RATIO",
                                    "PARTIAL_TOKEN_RATIO", "WRATIO"])
@pytest.mark.parametrize("width", [1, 4])
def test_cdist_token_set_family_matches_oracle(metric, width):
    """token_set_ratio, partial_token_set_ratio, token_ratio, partial_token_ratio and WRatio
    over batches (host parts, the FAM_TOKEN kernel), free and cached forms, several cutoffs"""
    m = getattr(R, metric)
    q, c = _vocab_batches(61 + width, width)
    for cut in (0.0, 50.0, 85.0, 100.0, 100.5):
        exp = oracle_cdist(m, R.SIMILARITY, q, c, cut)
        for form in (R.FORM_FREE, R.FORM_CACHED):
            got = R.cdist(m, R.SIMILARITY, q, c, cut, form=form)
            bad = np.argwhere(got.view(np.int64) != exp.view(np.int64))
            assert bad.size == 0, "cut %r form %d mismatch at %r: got %r exp %r" % (
                cut, form, bad[0], got[tuple(bad[0])], exp[tuple(bad[0])])
    data, off, w = q
    s1 = data[off[2]:off[3]]
    got = R.Cached(m, s1).score_many(R.SIMILARITY, c, 30.0)
    exp = oracle_cdist(m, R.SIMILARITY, R.pack_strings([s1], w), c, 30.0)[0]
    assert np.array_equal(got.view(np.int64), exp.view(np.int64))


def test_cdist_wratio_device_buffers():
    """WRatio with device inputs (downloaded for the parts) and a device result with ld"""
    import ctypes
    import torch
    from rapidfuzz_gb300._lib import Cutoff, Strings, make_params, check
    q, c = _vocab_batches(5, 1, 9, 40)
    exp = oracle_cdist(R.WRATIO, R.SIMILARITY, q, c, 40.0)
    dq = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in q[:2]]
    dc = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in c[:2]]
    nq, nc = q[1].size - 1, c[1].size - 1
    ld = nc + 3
    out = torch.full((nq, ld), -7.0, dtype=torch.float64, device="cuda")
    qs = Strings(dq[0].data_ptr(), dq[1].data_ptr(), nq, 1)
    cs = Strings(dc[0].data_ptr(), dc[1].data_ptr(), nc, 1)
    torch.cuda.synchronize()
    check(R.lib().rfg_cdist(R.WRATIO, R.SIMILARITY, R.FORM_CACHED, ctypes.byref(qs), ctypes.byref(cs),
                            ctypes.byref(make_params()), Cutoff(0, 40.0, 0, 0.0), R.F64, out.data_ptr(), ld,
                            R.DEVICE_INPUTS | R.DEVICE_OUTPUT))
    check(R.lib().rfg_synchronize())
    got = out.cpu().numpy()
    assert np.array_equal(got[:, :nc].view(np.int64), exp.view(np.int64))
    assert (got[:, nc:] == -7.0).all()


def test_token_set_family_api_names():
    """the reference's names and known answers (tests-fuzz.cpp:48-137)"""
    s1, s3 = "new york mets", "the wonderful new york mets"
    s4, s5 = "new york mets vs atlanta braves", "atlanta braves vs new york mets"
    s7 = "new york city mets - atlanta braves"
    assert R.fuzz_token_set_ratio(s4, s5) == 100.0
    assert R.fuzz_token_set_ratio("{", "{") == 100.0 and R.fuzz_token_set_ratio("{a", "{a") == 100.0
    assert R.fuzz_token_set_ratio("a{", "{b") == 50.0
    assert R.fuzz_partial_token_set_ratio(s4, s7) == 100.0
    assert R.fuzz_WRatio(s1, s1) == 100.0
    assert abs(R.fuzz_WRatio(s1, s3) - 90.0) < 1e-6
    assert abs(R.fuzz_WRatio(s4, s5) - 95.0) < 1e-6
    assert abs(R.fuzz_WRatio("hello", "hello" + "abcde" * 7) - 90.0) < 1e-6
    assert R.fuzz_token_set_ratio("", "") == 0.0 and R.fuzz_partial_token_set_ratio("", "") == 0.0
    assert R.fuzz_token_ratio("", "") == 100.0 and R.fuzz_partial_token_ratio("", "") == 100.0
    assert R.fuzz_WRatio("", "") == 0.0
    o = oracle()
    for a, b in ((s1, s3), (s4, s5), (s4, s7), ("", "a"), ("a a a", "a"), ("fuzzy was a bear", "fuzzy fuzzy was a bear")):
        for m, free, cached in ((R.TOKEN_SET_RATIO, R.fuzz_token_set_ratio, R.CachedTokenSetRatio),
                                (R.PARTIAL_TOKEN_SET_RATIO, R.fuzz_partial_token_set_ratio,
                                 R.CachedPartialTokenSetRatio),
                                (R.TOKEN_RATIO, R.fuzz_token_ratio, R.CachedTokenRatio),
                                (R.PARTIAL_TOKEN_RATIO, R.fuzz_partial_token_ratio, R.CachedPartialTokenRatio),
                                (R.WRATIO, R.fuzz_WRatio, R.CachedWRatio)):
            exp = oscore(o.rfo_score, m, R.SIMILARITY, FREE, a.encode(), b.encode(), 0.0)
            assert G.same(free(a, b), exp), (m, a, b)
            assert G.same(cached(a).similarity(b), exp), (m, a, b)
    with pytest.raises(ValueError):
        R.Multi(R.WRATIO, 8, 1)


@pytest.mark.parametrize("metric,op,cut,dt", [("LEVENSHTEIN", "DISTANCE", 8, "I32"), ("INDEL", "NORMALIZED_SIMILARITY", 0.5, "F64"),
                                              ("JARO_WINKLER", "SIMILARITY", 0.8, "F64"), ("WRATIO", "SIMILARITY", 50.0, "F64")])
def test_cdist_into_pinned_host_memory(metric, op, cut, dt):
    """results in pinned host memory: the kernels store them over the host link directly
    (rows with ld > choices; the padding stays untouched)"""
    import torch
    m, o, d = getattr(R, metric), getattr(R, op), getattr(R, dt)
    rng = random.Random(91)
    qs = [bytes(_rand(rng, b"abcd ", 0, 70)) for _ in range(37)]
    cs = [bytes(_rand(rng, b"abcd ", 0, 70)) for _ in range(1500)]
    q, c = R.pack_strings(qs, 1), R.pack_strings(cs, 1)
    nc = len(cs)
    tdt = {R.I32: torch.int32, R.F64: torch.float64}[d]
    ld = nc + 7
    host = torch.full((len(qs), ld), -3, dtype=tdt).pin_memory()
    got = R.cdist(m, o, q, c, cut, out_dtype=d, out=host.numpy(), ld=ld)
    exp = oracle_cdist(m, o, q, c, cut, out_dtype=d)
    a = got[:, :nc]
    if a.dtype == np.float64:
        a, exp = a.view(np.int64), exp.view(np.int64)
    assert np.array_equal(a, exp)
    assert (got[:, nc:] == -3).all()



def test_editops_fixture_batched():
    """levenshtein_editops / indel_editops / lcs_seq_editops of every fixture pair, the
    pairs of one metric, width and score hint in one rfg_editops call (one thread per pair;
    the long Levenshtein pairs through the Hirschberg kernel)"""
    groups = {}
    for c in G.load("editops.json"):
        groups.setdefault((c["metric"], c["w"], c["hint"]), []).append(c)
    for (metric, w, hint), cs in groups.items():
        dt = {1: np.uint8, 2: np.uint16, 4: np.uint32}[w]
        a = R.pack_strings([np.array(c["s1"], dtype=dt) for c in cs], w)
        b = R.pack_strings([np.array(c["s2"], dtype=dt) for c in cs], w)
        got = R.editops_many(metric, a, b, hint)
        for c, g in zip(cs, got):
            assert [tuple(int(v) for v in x) for x in g[["type", "src_pos", "dest_pos"]].tolist()] == \
                [tuple(x) for x in c["expected"]], (metric, w, hint, c.get("cite"), len(c["s1"]), len(c["s2"]))


def test_editops_api_names():
    """levenshtein_editops (with a score hint), indel_editops, lcs_seq_editops; the
    Hirschberg regime is refused"""
    from oracle_lib import editops
    o = oracle()
    for a, b in (("Lorem ipsum.", "XYZLorem ABC iPsum"), ("", "abc"), ("abc", ""), ("", ""), ("aa", "abb"),
                 ("kitten", "sitting"), ("a" * 70 + "xyz", "b" + "a" * 70 + "xz")):
        for metric, fn in ((R.LEVENSHTEIN, R.levenshtein_editops), (R.INDEL, R.indel_editops),
                           (R.LCSSEQ, R.lcs_seq_editops)):
            exp = editops(o.rfo_editops, metric, a.encode(), b.encode())
            e = fn(a, b)
            assert [(["none", "replace", "insert", "delete"].index(x.type), x.src_pos, x.dest_pos) for x in e] == exp
            assert e.get_src_len() == len(a) and e.get_dest_len() == len(b)
    assert len(R.levenshtein_editops("kitten", "sitting", 5)) == 3
    for a, b in (("Lorem ipsum.", "XYZLorem ABC iPsum"), ("kitten", "sitting"), ("", "abc"), ("abc", "")):
        e = R.levenshtein_editops(a, b)
        assert "".join(e.apply(a, b)) == b
        oc = e.as_opcodes()
        assert "".join(oc.apply(a, b)) == b and list(oc.as_editops()) == list(e)
    a, b = "ab" * 1100, "ba" * 1100  # the reference's Hirschberg regime
    e = R.levenshtein_editops(a, b)
    assert [(["none", "replace", "insert", "delete"].index(x.type), x.src_pos, x.dest_pos) for x in e] == \
        editops(o.rfo_editops, R.LEVENSHTEIN, a.encode(), b.encode())
    assert "".join(e.apply(a, b)) == b
    assert len(R.indel_editops(a, b)) == 2
