"""The reference's extract / extractOne loops (README.md:153-214) over an oracle cdist
matrix: results passing the cutoff, best first, ties by choice index."""
import numpy as np

from oracle_lib import DISTANCE, NORM_DISTANCE, oracle_cdist


def better_high(op):
    return op not in (DISTANCE, NORM_DISTANCE)


def oracle_extract(metric, op, queries, choices, limit, cutoff, tie_last, weights=(1, 1, 1), pw=0.1):
    m = oracle_cdist(metric, op, queries, choices, cutoff, weights, pw)
    res = []
    for row in m:
        row = row.astype(np.float64)
        if cutoff is None:
            ok = np.ones(row.size, dtype=bool)
        else:
            ok = row >= cutoff if better_high(op) else row <= cutoff
        idx = np.nonzero(ok)[0]
        sc = row[idx]
        key = -sc if better_high(op) else sc
        tie = -idx if tie_last else idx
        order = np.lexsort((tie, key))[:limit]
        res.append((idx[order], sc[order]))
    return res
