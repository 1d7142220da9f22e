/*
 * rfo.h -- CPU oracle for the bit-parallel string scorers (TEST INFRASTRUCTURE ONLY).
 *
 * This is a restatement, in plain C-style C++, of rapidfuzz-cpp v3.3.3's scorers
 * (Levenshtein / Indel / LCSseq / OSA / Jaro / Jaro-Winkler / fuzz::ratio) and of
 * the formula chains of its metric bases (rapidfuzz/details/distance.hpp).  It is
 * what the CUDA path is compared with, and the CPU baseline timed beside it.  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark may load it;
 * the product library never links or calls it.
 *
 * Parity of this oracle is pinned against the reference itself: the recipe in
 * oracle/Makefile compiles a driver over the reference headers into
 * oracle/_ref/librfref.so (where the reference sources are present), and
 * tests/golden/make_golden.py uses it to write the fixtures under tests/golden/
 * that the oracle is checked against.
 */
#ifndef RFO_H
#define RFO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* metric ids -- the same numbering as the product C-ABI (include/rapidfuzz_gb300.h) */
enum {
    RFO_LEVENSHTEIN = 0,
    RFO_INDEL = 1,
    RFO_LCSSEQ = 2,
    RFO_OSA = 3,
    RFO_JARO = 4,
    RFO_JARO_WINKLER = 5,
    RFO_RATIO = 6,
    RFO_PARTIAL_RATIO = 7,
    RFO_TOKEN_SORT_RATIO = 8,
    RFO_PARTIAL_TOKEN_SORT_RATIO = 9,
    RFO_QRATIO = 10,
    RFO_TOKEN_SET_RATIO = 11,
    RFO_PARTIAL_TOKEN_SET_RATIO = 12,
    RFO_TOKEN_RATIO = 13,
    RFO_PARTIAL_TOKEN_RATIO = 14,
    RFO_WRATIO = 15
};

/* operations */
enum { RFO_DISTANCE = 0, RFO_SIMILARITY = 1, RFO_NORM_DISTANCE = 2, RFO_NORM_SIMILARITY = 3 };

/* which reference API form the formula chain follows */
enum { RFO_FORM_FREE = 0, RFO_FORM_CACHED = 1, RFO_FORM_MULTI = 2 };

typedef struct {
    int64_t insert_cost, delete_cost, replace_cost; /* Levenshtein weights */
    double prefix_weight;                           /* Jaro-Winkler */
} rfo_params;

typedef struct {
    const void* data;       /* packed code units */
    const int64_t* offsets; /* count+1 offsets, in code units */
    int64_t count;
    int32_t char_width;     /* 1, 2, 4 or 8 */
} rfo_strings;

/* ---- exact core quantities, bit-parallel restatements ---- */
int64_t rfo_levenshtein_exact(const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2, int cw2,
                              int64_t ins, int64_t del, int64_t rep);
int64_t rfo_lcs_exact(const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2, int cw2);
int64_t rfo_osa_exact(const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2, int cw2);
/* Jaro common characters and (unhalved) transposition count, P = s1, T = s2 */
void rfo_jaro_counts(const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2, int cw2,
                     int64_t* common, int64_t* transpositions);

/* ---- naive O(N*M) dynamic programs (the rapidfuzz_reference headers, restated) ---- */
int64_t rfo_dp_levenshtein(const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2, int cw2,
                           int64_t ins, int64_t del, int64_t rep);
int64_t rfo_dp_lcs(const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2, int cw2);
int64_t rfo_dp_osa(const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2, int cw2);
void rfo_naive_jaro_counts(const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2, int cw2,
                           int64_t* common, int64_t* transpositions);

/* ---- one reference API call: metric x op x form, returns 0 or -1 (invalid argument) ----
 * Integer results go to *out_i, double results to *out_f.  cutoff_i / cutoff_f: the
 * score_cutoff of the integer / double overloads. */
int rfo_score(int metric, int op, int form, const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2,
              int cw2, const rfo_params* p, uint64_t cutoff_i, double cutoff_f, int64_t* out_i, double* out_f);

/* ---- batched scoring on host threads (CPU baseline): out[q*choices+c] ----
 * Follows the Cached* per-call path of the reference: the pattern of each query is
 * built once, then every choice is scored through the cached dispatch.
 * out_dtype: 0 = int32, 1 = int64, 2 = float64.  nthreads <= 0: all cores. */
int rfo_cdist(int metric, int op, const rfo_strings* queries, const rfo_strings* choices, const rfo_params* p,
              uint64_t cutoff_i, double cutoff_f, int out_dtype, void* out, int nthreads);

/* ---- editops (rapidfuzz/details/types.hpp:28-56 EditType / EditOp) ----
 * levenshtein_editops (with the reference's score_hint handling and its Hirschberg
 * recursion for long pairs), indel_editops / lcs_seq_editops (metric RFO_INDEL or
 * RFO_LCSSEQ; hint unused).  Writes up to cap operations, *count = the number of
 * operations; returns 0 or -1 (invalid). */
typedef struct {
    int32_t type; /* 0 none, 1 replace, 2 insert, 3 delete */
    int32_t reserved;
    int64_t src_pos;
    int64_t dest_pos;
} rfo_editop;

int rfo_editops(int metric, const void* s1, int64_t l1, int cw1, const void* s2, int64_t l2, int cw2, uint64_t hint,
                rfo_editop* ops, int64_t cap, int64_t* count);

/* the joins the token scorers score: sorted_split(s).join() (dedup = 0; common_impl.hpp
 * 162-180, SplittedSentenceView.hpp:71-85) or the join of the sorted tokens without
 * adjacent duplicates (dedup = 1; SplittedSentenceView::dedupe, SplittedSentenceView.hpp
 * 48-54).  Code units are widened to uint64; writes up to cap units, *out_len = the
 * join's length; returns 0. */
int rfo_token_join(const void* s, int64_t len, int cw, int dedup, uint64_t* out, int64_t cap, int64_t* out_len);

#ifdef __cplusplus
}
#endif

#endif
