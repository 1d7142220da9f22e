"""Loading of the golden fixtures (tests/golden/*.json, written by make_golden.py from
the reference itself)."""
import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_DT = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def load(name):
    with open(os.path.join(HERE, name)) as f:
        return json.load(f)


def dec(v):
    return v if isinstance(v, int) else float.fromhex(v)


def arrays(c):
    return np.array(c["s1"], dtype=_DT[c["w1"]]), np.array(c["s2"], dtype=_DT[c["w2"]])


def same(a, b):
    """bit-exact equality for ints and doubles"""
    if isinstance(a, float) or isinstance(b, float):
        return np.float64(a).tobytes() == np.float64(b).tobytes()
    return a == b
