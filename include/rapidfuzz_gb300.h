/*
 * rapidfuzz_gb300.h -- C ABI of the GB300 bit-parallel string scorers.
 *
 * One shared library (librapidfuzz_gb300.so) with plain pointers and sizes in every
 * signature.  Each entry point replaces a rapidfuzz-cpp v3.3.3 interface (paths are
 * relative to that project); the C++ mirror in rapidfuzz-cpp_gb300/include/rapidfuzz_gb300/
 * binds these entry points behind the reference's own class and function names.
 *
 * Results are those of the reference on the same inputs: integers bit-exact, doubles
 * bit-identical (the formula chains of rapidfuzz/details/distance.hpp are replayed on
 * the device with round-to-nearest double operations).
 *
 * Errors: every call returns an rfg_status.  RFG_ERR_INVALID_ARGUMENT corresponds to
 * the reference throwing std::invalid_argument, RFG_ERR_OUT_OF_RANGE to
 * std::out_of_range; rfg_last_error() gives the message of the calling thread's last
 * failure.  Nothing throws across the ABI.
 *
 * Strings are sequences of unsigned code units of 1, 2, 4 or 8 bytes.  Batches are
 * packed code units plus count+1 int64 offsets (in code units).
 *
 * Threading: handles may be shared between host threads for const calls (score*);
 * every call synchronises with its own stream before returning host results.
 */
#ifndef RAPIDFUZZ_GB300_H
#define RAPIDFUZZ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RFG_ABI_VERSION 1

typedef enum {
    RFG_OK = 0,
    RFG_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument in the reference */
    RFG_ERR_OUT_OF_RANGE = 2,     /* std::out_of_range in the reference */
    RFG_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    RFG_ERR_OUT_OF_MEMORY = 4,    /* device or pinned host allocation failed */
    RFG_ERR_NO_DEVICE = 5,        /* no CUDA device: the library has no CPU path */
    RFG_ERR_DEVICE_CHECK = 6,     /* a kernel's own bounds/timeout check fired */
    RFG_ERR_BUSY = 7              /* serving: admission refused (no slot / no memory) */
} rfg_status;

/* metrics (the scorer families of rapidfuzz/distance/ and fuzz::ratio) */
typedef enum {
    RFG_LEVENSHTEIN = 0,
    RFG_INDEL = 1,
    RFG_LCSSEQ = 2,
    RFG_OSA = 3,
    RFG_JARO = 4,
    RFG_JARO_WINKLER = 5,
    RFG_RATIO = 6,        /* fuzz::ratio; only RFG_SIMILARITY */
    RFG_PARTIAL_RATIO = 7, /* fuzz::partial_ratio / CachedPartialRatio (fuzz.hpp:128-183,
                              fuzz_impl.hpp:49-293); only RFG_SIMILARITY, no Multi form */
    /* token scorers over the ratio / partial_ratio engine: both strings are split on
     * whitespace, the tokens sorted by code unit (compared unsigned) and joined with
     * U+0020 on the host (fuzz.hpp:203-373, fuzz_impl.hpp:297-366); QRatio is ratio with
     * 0 where either string is empty (fuzz.hpp:692-804, fuzz_impl.hpp:891-929).  Only
     * RFG_SIMILARITY and RFG_F64, through rfg_score_f64, rfg_cached_*, rfg_cdist, rfg_extract
     * and (token sort and QRatio) rfg_multi_*; not in a prepared batch, the server or the
     * no-allocation entry. */
    RFG_TOKEN_SORT_RATIO = 8,
    RFG_PARTIAL_TOKEN_SORT_RATIO = 9,
    RFG_QRATIO = 10,
    /* the token_set_ratio family (fuzz.hpp:375-690, fuzz_impl.hpp:372-889): token_set_ratio,
     * partial_token_set_ratio, token_ratio, partial_token_ratio and WRatio with their
     * Cached forms, scored on the device from the strings, their sorted-split joins and
     * the joins of their distinct tokens (made on the host).  Only RFG_SIMILARITY and
     * RFG_F64, through rfg_score_f64, rfg_cached_*, rfg_cdist and rfg_extract; no Multi form. */
    RFG_TOKEN_SET_RATIO = 11,
    RFG_PARTIAL_TOKEN_SET_RATIO = 12,
    RFG_TOKEN_RATIO = 13,
    RFG_PARTIAL_TOKEN_RATIO = 14,
    RFG_WRATIO = 15
} rfg_metric;

/* the four result kinds of every metric (rapidfuzz/details/distance.hpp) */
typedef enum {
    RFG_DISTANCE = 0,
    RFG_SIMILARITY = 1,
    RFG_NORMALIZED_DISTANCE = 2,
    RFG_NORMALIZED_SIMILARITY = 3
} rfg_op;

/* which reference API the formula chain follows: the free functions, the Cached*
 * scorers, or experimental::Multi* (whose chains differ in a few corner cases) */
typedef enum { RFG_FORM_FREE = 0, RFG_FORM_CACHED = 1, RFG_FORM_MULTI = 2 } rfg_form;

/* output element types */
typedef enum { RFG_I32 = 0, RFG_I64 = 1, RFG_F64 = 2 } rfg_dtype;

typedef struct {
    int64_t insert_cost;  /* LevenshteinWeightTable (rapidfuzz/details/types.hpp:19-23) */
    int64_t delete_cost;
    int64_t replace_cost;
    double prefix_weight; /* Jaro-Winkler, default 0.1 */
} rfg_params;

/* score_cutoff / score_hint of one call: the integer overloads (size_t) read *_i,
 * the double overloads (normalized, Jaro, Jaro-Winkler, ratio) read *_f */
typedef struct {
    uint64_t cutoff_i;
    double cutoff_f;
    uint64_t hint_i;
    double hint_f;
} rfg_cutoff;

typedef struct {
    const void* data;       /* packed code units */
    const int64_t* offsets; /* count+1 entries, code units */
    int64_t count;
    int32_t char_width;     /* 1, 2, 4 or 8 */
} rfg_strings;

/* flags of batch calls */
#define RFG_DEVICE_INPUTS 1u  /* data/offsets of the batches are device pointers */
#define RFG_DEVICE_OUTPUT 2u  /* out is a device pointer (no copy back) */

typedef struct rfg_cached_s* rfg_cached;
typedef struct rfg_multi_s* rfg_multi;
typedef struct rfg_corpus_s* rfg_corpus;
typedef struct rfg_server_s* rfg_server;

/* ------------------------------------------------------------------ library */

int rfg_abi_version(void);
const char* rfg_last_error(void);
/* device the library runs on (default 0); must precede the first other call */
rfg_status rfg_set_device(int device);
/* synchronise the library's streams (the calls below already do for host results) */
rfg_status rfg_synchronize(void);

/* ------------------------------------------------------- free functions (per call)
 * levenshtein_distance / _similarity / _normalized_* (Levenshtein.hpp:140-265),
 * indel_* (Indel.hpp:12-63), lcs_seq_* (LCSseq.hpp:12-63), osa_* (OSA.hpp:12-111),
 * jaro_* (Jaro.hpp:12-61), jaro_winkler_* (JaroWinkler.hpp:11-73),
 * fuzz::ratio (fuzz.hpp:44-48, fuzz_impl.hpp:28-32). */
rfg_status rfg_score_i64(rfg_metric metric, rfg_op op, const void* s1, int64_t len1, int32_t width1,
                         const void* s2, int64_t len2, int32_t width2, const rfg_params* params,
                         uint64_t score_cutoff, uint64_t score_hint, int64_t* result);
rfg_status rfg_score_f64(rfg_metric metric, rfg_op op, const void* s1, int64_t len1, int32_t width1,
                         const void* s2, int64_t len2, int32_t width2, const rfg_params* params,
                         double score_cutoff, double score_hint, double* result);

/* ------------------------------------------------------------- cached scorers
 * CachedLevenshtein (Levenshtein.hpp:421-482), CachedIndel (Indel.hpp:148-183),
 * CachedLCSseq (LCSseq.hpp:197-226), CachedOSA (OSA.hpp:232-271), CachedJaro
 * (Jaro.hpp:195-223), CachedJaroWinkler (JaroWinkler.hpp:168-199), fuzz::CachedRatio
 * (fuzz.hpp:99-126).  create copies s1 to the device; calls are const and reentrant. */
rfg_status rfg_cached_create(rfg_metric metric, const void* s1, int64_t len1, int32_t width1,
                             const rfg_params* params, rfg_cached* out);
rfg_status rfg_cached_destroy(rfg_cached scorer);
/* one choice: Cached*::distance / similarity / normalized_* (distance.hpp:269-388) */
rfg_status rfg_cached_score_i64(rfg_cached scorer, rfg_op op, const void* s2, int64_t len2, int32_t width2,
                                uint64_t score_cutoff, uint64_t score_hint, int64_t* result);
rfg_status rfg_cached_score_f64(rfg_cached scorer, rfg_op op, const void* s2, int64_t len2, int32_t width2,
                                double score_cutoff, double score_hint, double* result);
/* many choices in one launch (the README's scorer-over-choices loop, README.md:153-240):
 * out[i] for choice i, out_dtype element type */
rfg_status rfg_cached_score_many(rfg_cached scorer, rfg_op op, const rfg_strings* choices, rfg_cutoff cutoff,
                                 rfg_dtype out_dtype, void* out, uint32_t flags);

/* ---------------------------------------------------------------- all pairs
 * cdist: out[q * ld + c] = scorer(queries[q]).op(choices[c]) for every pair, following
 * the Cached* chain (form RFG_FORM_CACHED) or the free-function chain.  ld >= count of
 * choices (0 means dense).  This is the batched persistent-kernel path. */
rfg_status rfg_cdist(rfg_metric metric, rfg_op op, rfg_form form, const rfg_strings* queries,
                     const rfg_strings* choices, const rfg_params* params, rfg_cutoff cutoff,
                     rfg_dtype out_dtype, void* out, int64_t ld, uint32_t flags);

/* ------------------------------------------------------------ prepared batches
 * The batched path of cdist with the host work done once: create() classifies the
 * queries, orders the tiles and places every buffer on the device; launch() only
 * enqueues the kernels on the given stream (no allocation, no host synchronisation),
 * so it can be timed with events, relaunched, or captured in a CUDA graph
 * (RFG_LAUNCH_GRAPH captures on the first call and replays afterwards).  out must be
 * device memory.  check() waits for the stream and reports the kernels' own checks.
 * tune() times block size x tile count on this batch and keeps the fastest.
 * (No reference counterpart: this is the persistent-kernel form of the reference's
 * "scorer over all choices" loop, README.md:153-240.) */
typedef struct rfg_batch_s* rfg_batch;
#define RFG_LAUNCH_GRAPH 1u

rfg_status rfg_batch_create(rfg_metric metric, rfg_op op, rfg_form form, const rfg_strings* queries,
                            const rfg_strings* choices, const rfg_params* params, rfg_cutoff cutoff,
                            rfg_dtype out_dtype, void* out, int64_t ld, uint32_t flags, rfg_batch* batch);
rfg_status rfg_batch_launch(rfg_batch batch, void* cuda_stream, uint32_t launch_flags);
rfg_status rfg_batch_check(rfg_batch batch, void* cuda_stream);
rfg_status rfg_batch_tune(rfg_batch batch, void* cuda_stream, int32_t* best_block, int64_t* best_tiles);
rfg_status rfg_batch_destroy(rfg_batch batch);
/* the kernels one launch of the batch runs (as the toolchain names them), separated by
 * ';' into names[0..cap), NUL-terminated; for profiling and logs */
rfg_status rfg_batch_kernels(rfg_batch batch, char* names, size_t cap);
/* the library's own stream (the synchronous entry points run on it) */
rfg_status rfg_get_stream(void** cuda_stream);

/* ------------------------------------------------------------------ extract
 * A corpus keeps a choice list on the device (with its length order precomputed) for
 * repeated extract calls.  rfg_extract returns, per query, the best `limit` (1..32)
 * choices whose score passes score_cutoff -- score >= cutoff for similarity ops,
 * <= cutoff for distance ops -- best first: the README's extract/extractOne loops over
 * a Cached* scorer (README.md:153-214).  Ties go to the lower choice index, or with
 * tie_last_wins to the later one, as the README's extractOne (`score >= best_score`)
 * does.  out_index/out_score hold count*limit entries (-1 / unspecified past
 * out_count[q]); scores are doubles (integer results convert exactly).  Tiles publish
 * their limit-th best so later tiles score under a tightened cutoff, the device form of
 * extractOne passing its running best as score_cutoff. */
rfg_status rfg_corpus_create(const rfg_strings* choices, uint32_t flags, rfg_corpus* corpus);
rfg_status rfg_corpus_destroy(rfg_corpus corpus);
rfg_status rfg_extract(rfg_corpus corpus, rfg_metric metric, rfg_op op, const rfg_strings* queries,
                       const rfg_params* params, rfg_cutoff cutoff, int32_t limit, int32_t tie_last_wins,
                       int64_t* out_index, double* out_score, int32_t* out_count, uint32_t flags);

/* ------------------------------------------------------------------ serving
 * A continuous-batching extract service over device-resident corpora (no reference
 * counterpart; the serving form of the README's extract loops, README.md:153-214).
 * submit() queues a request and returns at once; a loop thread groups queued requests
 * with the same spec (corpus, metric, op, params, cutoff, limit, tie rule, width) into
 * batches of up to max_batch and admits a batch whenever one of max_inflight stream
 * slots is free and its device-memory estimate fits max_device_bytes (0: 80 % of the
 * free device memory at create); batches run concurrently.  A request that alone needs
 * more than max_device_bytes is refused at submit with RFG_ERR_BUSY.  wait() blocks until
 * the request's result is in its out_* buffers (limit entries; out_count set) and reports
 * the submit-to-completion latency, or returns RFG_ERR_BUSY once timeout_s (> 0) has
 * passed without a result (the request stays queued; wait again).  Results equal
 * rfg_extract of the request alone. */
typedef struct {
    int32_t max_inflight;
    int32_t max_batch;
    int64_t max_device_bytes;
} rfg_server_config;

typedef struct {
    int32_t corpus; /* index into the server's corpora */
    rfg_metric metric;
    rfg_op op;
    rfg_params params;
    rfg_cutoff cutoff;
    int32_t limit;          /* 1..32: 1 with tie_last_wins = extractOne */
    int32_t tie_last_wins;
    const void* query;      /* copied at submit */
    int64_t query_len;
    int32_t query_width;
    int64_t* out_index;     /* caller buffers, filled on completion */
    double* out_score;
    int32_t* out_count;
} rfg_request;

rfg_status rfg_server_create(const rfg_corpus* corpora, int32_t ncorpora, const rfg_server_config* config,
                             rfg_server* server);
rfg_status rfg_server_submit(rfg_server server, const rfg_request* request, uint64_t* ticket);
rfg_status rfg_server_wait(rfg_server server, uint64_t ticket, double timeout_s, double* latency_ms);
rfg_status rfg_server_stats(rfg_server server, int64_t* completed, int64_t* batches, int64_t* batched_requests);
rfg_status rfg_server_destroy(rfg_server server);

/* ------------------------------------------------------------------ testing
 * Fault injection on the host for the library's own failure tests (no reference
 * counterpart): after `after` more successful device allocations of the batch engine,
 * every further one fails as if the device were out of memory, so that callers see
 * RFG_ERR_OUT_OF_MEMORY; a negative value switches the injection off. */
rfg_status rfg_testing_fail_device_allocs(int64_t after);

/* Launch-shape override for measurements: the band kernels' work units of 32 x rounds
 * pairs of one query (1..64; 0 restores the default, sized by the class).  Batches
 * prepared afterwards use it, until rfg_batch_tune chooses its own. */
rfg_status rfg_testing_band_rounds(int32_t rounds);

/* Kernel-choice override for measurements: 0 keeps every query off the band kernels
 * (the unbanded multi-word cores score them), 1 restores the default.  Batches prepared
 * afterwards use it, until rfg_batch_tune chooses its own. */
rfg_status rfg_testing_band_mode(int32_t on);

/* ------------------------------------------------------ no-allocation cdist
 * rfg_cdist_noalloc has no counterpart in the reference.  It is for callers that may
 * not allocate device memory (inside another framework's memory manager, in a process
 * whose device memory is reserved up front, or in a service that must not grow after
 * start-up) and already hold their strings and result buffer on the device: queries,
 * choices and out are device pointers, and the call allocates nothing.  Its scratch is a
 * fixed 32 MiB array in the library's device image, shared by every call on a device
 * and held by every GPU that loads the library until exit.  The first call on a device
 * looks up that array's address (make it before any stream capture); calls that
 * overlap on the GPU race on the array and must be serialised.  max_query_len bounds
 * the query lengths (at most 4096 code units); larger values, or a query longer than
 * the bound, return RFG_ERR_INVALID_ARGUMENT (in the second case after the kernel ran:
 * the rows of the other queries are written, that query's row is left as it was).
 * Runs on cuda_stream and waits for it. */
rfg_status rfg_cdist_noalloc(rfg_metric metric, rfg_op op, rfg_form form, const rfg_strings* queries,
                             const rfg_strings* choices, int64_t max_query_len, const rfg_params* params,
                             rfg_cutoff cutoff, rfg_dtype out_dtype, void* out, int64_t ld, void* cuda_stream);

/* ------------------------------------------------------- experimental::Multi*
 * MultiLevenshtein (Levenshtein.hpp:297-419), MultiIndel (Indel.hpp:77-146),
 * MultiLCSseq (LCSseq.hpp:77-195), MultiOSA (OSA.hpp:113-230), MultiJaro (Jaro.hpp:64-193),
 * MultiJaroWinkler (JaroWinkler.hpp:75-166), fuzz::experimental::MultiRatio (fuzz.hpp:50-95).
 * max_len is the MaxLen template argument (8, 16, 32 or 64). */
rfg_status rfg_multi_create(rfg_metric metric, int32_t max_len, size_t count, const rfg_params* params,
                            rfg_multi* out);
rfg_status rfg_multi_destroy(rfg_multi scorer);
rfg_status rfg_multi_insert(rfg_multi scorer, const void* s, int64_t len, int32_t width);
rfg_status rfg_multi_result_count(rfg_multi scorer, size_t* out);
rfg_status rfg_multi_score_i64(rfg_multi scorer, rfg_op op, int64_t* scores, size_t score_count, const void* s2,
                               int64_t len2, int32_t width2, uint64_t score_cutoff);
rfg_status rfg_multi_score_f64(rfg_multi scorer, rfg_op op, double* scores, size_t score_count, const void* s2,
                               int64_t len2, int32_t width2, double score_cutoff);

/* ------------------------------------------------------------------ editops
 * levenshtein_editops (Levenshtein.hpp:282-295), indel_editops (Indel.hpp:65-75) and
 * lcs_seq_editops (LCSseq.hpp:65-75) of many pairs (s1[i], s2[i]): the operations that
 * turn s1[i] into s2[i], in the reference's order (EditOp, rapidfuzz/details/types.hpp:
 * 28-56).  ops[offsets[i], offsets[i + 1]) are pair i's operations; the source / target
 * lengths of pair i are the lengths of s1[i] / s2[i].  capacity >= sum over the pairs of
 * max(len1, len2) (Levenshtein) or len1 + len2 (Indel, LCSseq) always suffices; with less,
 * the call fills offsets and returns RFG_ERR_OUT_OF_RANGE.  score_hint has the reference's
 * meaning (a small hint makes the exact distance the first band); long Levenshtein pairs
 * follow the reference's Hirschberg recursion (Levenshtein_impl.hpp:1184-1257). */
typedef enum { RFG_EDIT_NONE = 0, RFG_EDIT_REPLACE = 1, RFG_EDIT_INSERT = 2, RFG_EDIT_DELETE = 3 } rfg_edit_type;

typedef struct {
    int32_t type; /* rfg_edit_type */
    int32_t reserved;
    int64_t src_pos;
    int64_t dest_pos;
} rfg_editop;

rfg_status rfg_editops(rfg_metric metric, const rfg_strings* s1, const rfg_strings* s2, uint64_t score_hint,
                       rfg_editop* ops, int64_t capacity, int64_t* offsets, uint32_t flags);

#ifdef __cplusplus
}
#endif

#endif /* RAPIDFUZZ_GB300_H */
