"""Python binding of librapidfuzz_gb300 (ctypes over the C ABI in include/rapidfuzz_gb300.h).

Names mirror rapidfuzz-cpp: levenshtein_distance(...), CachedLevenshtein(s1).distance(s2),
experimental.MultiLevenshtein(max_len, count), fuzz_ratio(...), plus cdist() for the
batched all-pairs path.  Strings are str, bytes, or numpy arrays of unsigned code units.
There is no CPU fallback: importing fails when the CUDA library has not been built.
"""
from ._lib import (DISTANCE, SIMILARITY, NORMALIZED_DISTANCE, NORMALIZED_SIMILARITY,  # noqa: F401
                   LEVENSHTEIN, INDEL, LCSSEQ, OSA, JARO, JARO_WINKLER, RATIO, PARTIAL_RATIO,
                   TOKEN_SORT_RATIO, PARTIAL_TOKEN_SORT_RATIO, QRATIO, TOKEN_SET_RATIO,
                   PARTIAL_TOKEN_SET_RATIO, TOKEN_RATIO, PARTIAL_TOKEN_RATIO, WRATIO,
                   FORM_FREE, FORM_CACHED, FORM_MULTI, I32, I64, F64,
                   DEVICE_INPUTS, DEVICE_OUTPUT, RapidfuzzError, lib, lib_path,
                   as_units, pack_strings, score, Cached, Multi, cdist, Batch, library_stream, Corpus, Server,
                   editops_many, EDITOP_DTYPE)
from ._api import *  # noqa: F401,F403
