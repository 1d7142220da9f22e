"""The continuous-batching service: requests of different metrics, limits and query
lengths submitted together (batched and overlapping on the device) give exactly the
result of the same request run alone, and the reference's extract loop's result."""
import random
import threading

import numpy as np
import pytest

from extract_lib import oracle_extract

pytestmark = pytest.mark.gpu

import rapidfuzz_gb300 as R  # noqa: E402
import workloads as WL  # noqa: E402


def _dna(rng, n):
    return np.array([rng.choice(b"ACGT") for _ in range(n)], dtype=np.uint8)


def test_results_alone_and_in_the_mix():
    rng = random.Random(17)
    dna = WL.dna_uniform(seed=21, n=30000, lo=10, hi=200)
    (tok, tok_list) = WL.tokens_u32(seed=22, n=20000)
    corpora = [R.Corpus(dna), R.Corpus(tok)]
    server = R.Server(corpora, max_inflight=3, max_batch=8)
    reqs = []
    for i in range(48):
        metric = rng.choice([R.LEVENSHTEIN, R.INDEL, R.OSA, R.JARO_WINKLER])
        limit = rng.choice([1, 10])
        if metric == R.JARO_WINKLER:
            base = list(rng.choice(tok_list))
            q = np.array(base[:rng.randint(1, len(base))] + [rng.choice(WL.TOKEN_ALPHABET)
                                                            for _ in range(rng.randint(0, 6))], dtype=np.uint32)
            reqs.append((1, metric, R.SIMILARITY, q, limit, rng.choice([None, 0.8])))
        else:
            reqs.append((0, metric, R.DISTANCE, _dna(rng, rng.randint(5, 300)), limit, rng.choice([None, 40])))
    tickets = [None] * len(reqs)

    def submit(lo, hi):
        for i in range(lo, hi):
            c, m, op, q, limit, cut = reqs[i]
            tickets[i] = server.submit(c, m, op, q, limit, cut)

    threads = [threading.Thread(target=submit, args=(k * 12, k * 12 + 12)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    got = [server.wait(t) for t in tickets]
    st = server.stats()
    assert st["completed"] == len(reqs)
    assert st["batches"] < len(reqs)  # requests were batched
    server.close()
    for i, (c, m, op, q, limit, cut) in enumerate(reqs):
        qb = R.pack_strings([q], q.itemsize)
        idx, sc, cnt = corpora[c].extract(m, op, qb, limit, cut, tie_last=(limit == 1))
        gi, gs, _ = got[i]
        assert np.array_equal(gi, idx[0, :cnt[0]]), i
        assert np.array_equal(gs.view(np.int64), sc[0, :cnt[0]].view(np.int64)), i
        if i % 6 == 0:
            ei, es = oracle_extract(m, op, qb, dna if c == 0 else tok, limit, cut, limit == 1)[0]
            assert np.array_equal(gi, ei), i
            assert np.array_equal(gs.view(np.int64), es.view(np.int64)), i
