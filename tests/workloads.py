"""Seeded synthetic workloads shaped like the benchmark configurations of the
rapidfuzz-cpp path (no public dataset is named; these generators stand in for it).

cdist_zipf:   N x M strings over a-z with Zipf(s) letter frequencies, lengths U[lo, hi],
              a fraction of the choices being copies of a query with 1..6 random
              substitutions / insertions / deletions / adjacent transpositions.
dna_uniform:  1 x N uint8 strings over {A,C,G,T}, lengths U[lo, hi].
dna_lognormal: N x M DNA strings, lengths log-normal (median, sigma) clipped, choices either
              unrelated or a query mutated at an edit rate drawn from [lo_rate, hi_rate].
tokens_u32:   uint32 code-point strings of 1-4 space-joined tokens of 3-12 characters
              from 40 code points (26 Latin + 14 accented in U+00C0-U+00FF).
"""
import numpy as np


def _pack(arrs, dtype):
    lens = np.fromiter((len(a) for a in arrs), dtype=np.int64, count=len(arrs))
    off = np.zeros(len(arrs) + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    data = np.concatenate([np.asarray(a, dtype=dtype) for a in arrs]) if arrs else np.zeros(0, dtype)
    if data.size == 0:
        data = np.zeros(1, dtype)
    return data, off


def _random_strings(rng, n, lo, hi, alphabet, p=None, dtype=np.uint8):
    lens = rng.integers(lo, hi + 1, size=n)
    flat = rng.choice(np.asarray(alphabet), size=int(lens.sum()), p=p).astype(dtype)
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    return flat, off


def mutate(rng, s, alphabet, k):
    s = list(s)
    for _ in range(k):
        op = int(rng.integers(0, 4))
        if op == 0 and s:
            s[int(rng.integers(0, len(s)))] = alphabet[int(rng.integers(0, len(alphabet)))]
        elif op == 1:
            s.insert(int(rng.integers(0, len(s) + 1)), alphabet[int(rng.integers(0, len(alphabet)))])
        elif op == 2 and s:
            del s[int(rng.integers(0, len(s)))]
        elif op == 3 and len(s) > 1:
            i = int(rng.integers(0, len(s) - 1))
            s[i], s[i + 1] = s[i + 1], s[i]
    return s


def zipf_probs(k, s):
    w = 1.0 / np.arange(1, k + 1) ** s
    return w / w.sum()


def cdist_zipf(seed=0, nq=4096, nc=4096, lo=16, hi=64, s=1.1, copy_frac=0.2):
    """queries, choices as (data uint8, offsets int64, width 1)"""
    rng = np.random.default_rng(seed)
    alpha = list(range(97, 123))
    p = zipf_probs(26, s)
    qd, qo = _random_strings(rng, nq, lo, hi, alpha, p)
    cd, co = _random_strings(rng, nc, lo, hi, alpha, p)
    choices = [cd[co[i]:co[i + 1]].tolist() for i in range(nc)]
    ncopy = int(round(copy_frac * nc))
    for i in rng.choice(nc, size=ncopy, replace=False):
        qi = int(rng.integers(0, nq))
        base = qd[qo[qi]:qo[qi + 1]].tolist()
        choices[i] = mutate(rng, base, alpha, int(rng.integers(1, 7)))
    cd2, co2 = _pack(choices, np.uint8)
    return (qd, qo, 1), (cd2, co2, 1)


def dna_uniform(seed=0, n=100000, lo=8, hi=64):
    rng = np.random.default_rng(seed)
    d, o = _random_strings(rng, n, lo, hi, [65, 67, 71, 84])
    return d, o, 1


def dna_lognormal(seed=0, nq=256, nc=65536, median=300, sigma=0.6, lo=100, hi=2000, rel_frac=0.5,
                  rate_lo=0.01, rate_hi=0.15):
    rng = np.random.default_rng(seed)
    alpha = [65, 67, 71, 84]

    def lens(n):
        x = np.exp(np.log(median) + sigma * rng.standard_normal(n))
        return np.clip(np.round(x), lo, hi).astype(np.int64)

    ql = lens(nq)
    queries = [rng.choice(alpha, size=int(l)).astype(np.uint8) for l in ql]
    choices = []
    for _ in range(nc):
        if rng.random() < rel_frac:
            base = queries[int(rng.integers(0, nq))]
            k = int(round(len(base) * rng.uniform(rate_lo, rate_hi)))
            choices.append(mutate(rng, base.tolist(), alpha, k))
        else:
            choices.append(rng.choice(alpha, size=int(lens(1)[0])).astype(np.uint8))
    qd, qo = _pack(queries, np.uint8)
    cd, co = _pack(choices, np.uint8)
    return (qd, qo, 1), (cd, co, 1)


TOKEN_ALPHABET = list(range(97, 123)) + [0xC0, 0xC1, 0xC7, 0xC8, 0xC9, 0xCD, 0xD1, 0xD3, 0xD6, 0xDA, 0xDC, 0xE0,
                                           0xE9, 0xF1]


def tokens_u32(seed=0, n=1000, derive_from=None, derive_frac=0.0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        if derive_from is not None and rng.random() < derive_frac:
            base = derive_from[int(rng.integers(0, len(derive_from)))]
            out.append(mutate(rng, list(base), TOKEN_ALPHABET, int(rng.integers(0, 4))))
            continue
        toks = []
        for _ in range(int(rng.integers(1, 5))):
            toks.append(rng.choice(TOKEN_ALPHABET, size=int(rng.integers(3, 13))).tolist())
        s = toks[0]
        for t in toks[1:]:
            s = s + [0x20] + t
        out.append(s)
    d, o = _pack(out, np.uint32)
    return (d, o, 4), out


def dna_corpus_fast(seed=0, n=10_000_000, lo=10, hi=200):
    """n uint8 DNA strings, lengths U[lo, hi] (vectorised; ~1 GB at the serving size)"""
    rng = np.random.default_rng(seed)
    lens = rng.integers(lo, hi + 1, size=n)
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    codes = np.frombuffer(b"ACGT", dtype=np.uint8)
    data = codes[rng.integers(0, 4, size=int(off[-1]), dtype=np.uint8)]
    return data, off, 1


def tokens_u32_fast(seed=0, n=1_000_000):
    """n uint32 strings of 1-4 space-joined tokens of 3-12 code points from TOKEN_ALPHABET"""
    rng = np.random.default_rng(seed)
    ntok = rng.integers(1, 5, size=n)
    tot = int(ntok.sum())
    tlen = rng.integers(3, 13, size=tot)
    owner = np.repeat(np.arange(n), ntok)
    slen = np.bincount(owner, weights=tlen, minlength=n).astype(np.int64) + (ntok - 1)
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(slen, out=off[1:])
    alpha = np.array(TOKEN_ALPHABET, dtype=np.uint32)
    data = alpha[rng.integers(0, len(alpha), size=int(off[-1]))]
    # a space after every token except the last of its string
    tok_end = np.cumsum(tlen + 1) - 1  # position of the separator in a space-after-every-token layout
    first_tok = np.zeros(n, dtype=np.int64)
    np.cumsum(ntok[:-1], out=first_tok[1:])
    is_last = np.zeros(tot, dtype=bool)
    is_last[first_tok + ntok - 1] = True
    # separator position inside its string = (start of the string in the all-separators layout)
    start_all = np.zeros(tot, dtype=np.int64)
    np.cumsum((tlen + 1)[:-1], out=start_all[1:])
    str_start_all = start_all[first_tok][owner]
    sep_pos = off[owner] + (tok_end - str_start_all)
    data[sep_pos[~is_last]] = 0x20
    return data, off, 4


def tokens_u32_mixed(seed=0, n=1_000_000, derive_from=None, derive_count=0):
    """tokens_u32_fast strings with derive_count of them (at seeded positions) replaced by
    copies of derive_from strings with 0-3 random edits, so that hits above a cutoff exist"""
    data, off, w = tokens_u32_fast(seed=seed, n=n)
    if not derive_from or derive_count <= 0:
        return data, off, w
    rng = np.random.default_rng(seed + 7919)
    pos = set(int(x) for x in rng.choice(n, size=derive_count, replace=False))
    out = []
    for i in range(n):
        if i in pos:
            base = derive_from[int(rng.integers(0, len(derive_from)))]
            out.append(np.asarray(mutate(rng, list(base), TOKEN_ALPHABET, int(rng.integers(0, 4))), dtype=np.uint32))
        else:
            out.append(data[off[i]:off[i + 1]])
    d, o = _pack(out, np.uint32)
    return d, o, 4
