"""Multi-rank host logic on CPU: two gloo ranks each score their shard of the choices
with the oracle, gather and merge the extract results, and agree on the slowest time.
The merged result must equal extract over the whole list (README.md:153-214 order)."""
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "rapidfuzz-cpp_gb300"))

from rapidfuzz_gb300 import sharding  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _cases():
    from oracle_lib import LEVENSHTEIN, INDEL, JARO_WINKLER, DISTANCE, SIMILARITY, NORM_SIMILARITY
    return [(LEVENSHTEIN, DISTANCE, 5, 4, False), (INDEL, SIMILARITY, 3, 6, False),
            (JARO_WINKLER, NORM_SIMILARITY, 4, 0.7, True), (LEVENSHTEIN, DISTANCE, 1, 10, True)]


def _strings(seed, n, lo, hi):
    rng = np.random.default_rng(seed)
    alpha = np.frombuffer(b"abcde", dtype=np.uint8)
    out = [alpha[rng.integers(0, 5, size=int(rng.integers(lo, hi + 1)))].tobytes() for _ in range(n)]
    return out


def _rank_main(rank, world, port, outdir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    from extract_lib import oracle_extract, better_high
    from oracle_lib import pack_strings
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        queries = _strings(1, 7, 0, 12)
        choices = _strings(2, 53, 0, 12)
        a, b = sharding.shard_of(len(choices), rank, world)
        res = []
        for metric, op, limit, cut, tie_last in _cases():
            local = oracle_extract(metric, op, pack_strings(queries, 1), pack_strings(choices[a:b], 1), limit, cut,
                                   tie_last)
            li = np.full((len(queries), limit), -1, dtype=np.int64)
            ls = np.zeros((len(queries), limit))
            lc = np.zeros(len(queries), dtype=np.int32)
            for q, (i, s) in enumerate(local):
                li[q, :len(i)] = i
                ls[q, :len(s)] = s
                lc[q] = len(i)
            res.append(sharding.gather_extract((li, ls, lc), a, limit, better_high(op), tie_last))
        t = sharding.max_over_ranks(0.25 + rank)
        np.save(os.path.join(outdir, "t%d.npy" % rank), np.array([t]))
        for k, (i, s, c) in enumerate(res):
            np.savez(os.path.join(outdir, "r%d_%d.npz" % (rank, k)), i=i, s=s, c=c)
    finally:
        dist.destroy_process_group()


def test_shard_bounds_cover_everything():
    for n in (0, 1, 5, 53, 4096):
        for world in (1, 2, 3, 8):
            b = sharding.shard_bounds(n, world)
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[r][1] == b[r + 1][0] for r in range(world - 1))
            sizes = [y - x for x, y in b]
            assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_merge_equals_whole_list(tmp_path):
    import torch.multiprocessing as mp
    from extract_lib import oracle_extract
    from oracle_lib import pack_strings
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    queries = _strings(1, 7, 0, 12)
    choices = _strings(2, 53, 0, 12)
    for rank in range(world):
        assert float(np.load(tmp_path / ("t%d.npy" % rank))[0]) == 1.25
    for k, (metric, op, limit, cut, tie_last) in enumerate(_cases()):
        exp = oracle_extract(metric, op, pack_strings(queries, 1), pack_strings(choices, 1), limit, cut, tie_last)
        for rank in range(world):
            r = np.load(tmp_path / ("r%d_%d.npz" % (rank, k)))
            for q, (i, s) in enumerate(exp):
                assert r["c"][q] == len(i)
                assert np.array_equal(r["i"][q, :len(i)], i), (k, q)
                assert np.array_equal(r["s"][q, :len(s)].view(np.int64), np.asarray(s, np.float64).view(np.int64))
