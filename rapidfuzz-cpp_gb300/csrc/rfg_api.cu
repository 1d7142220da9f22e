/*
 * rfg_api.cu -- host runtime and C ABI of librapidfuzz_gb300.
 *
 * Every entry point ends in one engine: run_batch() scores a set of queries (the s1
 * side, whose pattern tables are built on the device) against a set of choices (the
 * s2 side).  Queries are classified by pattern words (1, 2, 4, 8 words in registers,
 * or the any-length scratch kernel), each class is ordered longest first and cut
 * into (query, choice-chunk) tiles that persistent CTAs pull from an atomic counter.
 * The free functions and Cached* scorers are batches of one query; Multi* scorers are
 * batches of many short queries against one choice; cdist is the general case.
 *
 * Device memory is taken from the stream-ordered pool (cudaMallocAsync) with a release
 * threshold that keeps it cached between calls.  One library stream; calls from
 * several host threads are serialised by a mutex.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rapidfuzz_gb300.h"
#include "rfg_device.cuh"
#include "rfg_fast.cuh"
#include "rfg_band.cuh"
#include "rfg_kernels.h"
#include "rfg_token.h"

using namespace rfg;

namespace {

thread_local std::string g_err;

rfg_status fail(rfg_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return s;
}

#define RFG_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            return fail(e_ == cudaErrorMemoryAllocation ? RFG_ERR_OUT_OF_MEMORY : RFG_ERR_CUDA,     \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                            \
        }                                                                                           \
    } while (0)

#define RFG_TRY(expr)                        \
    do {                                     \
        rfg_status s_ = (expr);              \
        if (s_ != RFG_OK) return s_;         \
    } while (0)

#define RFG_COUNTERS 256
#define RFG_MAX_ROW_BLOCKS 12

struct Ctx {
    std::atomic<bool> init{false};
    int device = 0;
    int sms = 0;
    int prio_high = 0; /* the device's highest stream priority (urgent launches) */
    cudaStream_t stream = nullptr;
    cudaStream_t copy = nullptr; /* device-to-host result copies overlapping the next row block */
    cudaEvent_t blk_ev[RFG_MAX_ROW_BLOCKS] = {};
    cudaEvent_t prep_ev = nullptr; /* end of a preparation on `stream`, for launches on other streams */
    /* pinned staging of host results bound for pageable memory: two slots, one copied out
     * by the host threads while the other fills */
    unsigned char* stage_h = nullptr;
    size_t stage_slot = 0;
    cudaEvent_t stage_ev[2] = {};
    /* pinned staging of a preparation's small host tables (one copy per preparation);
     * up_ev marks the end of the last copy out of it */
    unsigned char* up_h = nullptr;
    size_t up_cap = 0;
    cudaEvent_t up_ev = nullptr;
    /* the class launches of one batch are independent: launches 1.. run on side streams
     * forked from and joined back into the caller's stream (graph capture records the
     * same fork/join as parallel branches); each origin stream keeps its own set */
    struct SideSet {
        std::vector<cudaStream_t> side;
        std::vector<cudaEvent_t> ev; /* [0] fork, [1..] joins */
    };
    std::unordered_map<cudaStream_t, SideSet> sides;
    /* host results in pinned, mapped memory are stored by the kernels themselves over the
     * host link (RFG_HOST_STORES=0 in the environment copies them from a device buffer) */
    bool host_stores = true;
    std::recursive_mutex mu;
    std::unordered_map<const void*, int> occ; /* (kernel) -> CTAs per SM at the default smem */
};
Ctx g;

thread_local int t_device = -1; /* the device this host thread has made current */

rfg_status ensure_ctx_locked();

/* The library's context, created once (thread-safe); every host thread that calls in has
 * the library's device made current for it. */
rfg_status ensure_ctx()
{
    if (!g.init.load(std::memory_order_acquire)) {
        std::lock_guard<std::recursive_mutex> lk(g.mu);
        RFG_TRY(ensure_ctx_locked());
    }
    if (t_device != g.device) {
        RFG_CUDA(cudaSetDevice(g.device));
        t_device = g.device;
    }
    return RFG_OK;
}

rfg_status ensure_ctx_locked()
{
    if (g.init.load(std::memory_order_relaxed)) return RFG_OK;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(RFG_ERR_NO_DEVICE, "no CUDA device available (%s); this library has no CPU path",
                    cudaGetErrorString(e));
    RFG_CUDA(cudaSetDevice(g.device));
    RFG_CUDA(cudaDeviceGetAttribute(&g.sms, cudaDevAttrMultiProcessorCount, g.device));
    {
        int least = 0, greatest = 0;
        RFG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        g.prio_high = greatest;
    }
    RFG_CUDA(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
    RFG_CUDA(cudaStreamCreateWithFlags(&g.copy, cudaStreamNonBlocking));
    for (auto& e : g.blk_ev) RFG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    RFG_CUDA(cudaEventCreateWithFlags(&g.prep_ev, cudaEventDisableTiming));
    for (auto& e : g.stage_ev) RFG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    RFG_CUDA(cudaEventCreateWithFlags(&g.up_ev, cudaEventDisableTiming));
    if (const char* hs = getenv("RFG_HOST_STORES")) g.host_stores = atoi(hs) != 0;
    cudaMemPool_t pool;
    RFG_CUDA(cudaDeviceGetDefaultMemPool(&pool, g.device));
    uint64_t thr = UINT64_MAX;
    RFG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    g.init.store(true, std::memory_order_release);
    return RFG_OK;
}

/* the pinned staging of small uploads, at least `bytes` long, free of in-flight copies */
rfg_status upload_stage(size_t bytes, unsigned char** h)
{
    RFG_CUDA(cudaEventSynchronize(g.up_ev));
    if (bytes > g.up_cap) {
        if (g.up_h) cudaFreeHost(g.up_h);
        g.up_h = nullptr;
        g.up_cap = 0;
        const size_t cap = std::max<size_t>(bytes, 1u << 20);
        RFG_CUDA(cudaHostAlloc((void**)&g.up_h, cap, cudaHostAllocDefault));
        g.up_cap = cap;
    }
    *h = g.up_h;
    return RFG_OK;
}

/* allocations left before the injected failures of rfg_testing_fail_device_allocs
 * (negative: no injection) */
std::atomic<int64_t> g_fail_allocs_after{-1};

/* stream-ordered device allocation freed at scope exit */
struct DBuf {
    void* p = nullptr;
    cudaStream_t free_on = nullptr; /* stream of the last use (nullptr: the library stream) */
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf()
    {
        if (p) cudaFreeAsync(p, free_on ? free_on : g.stream);
    }
    rfg_status alloc(size_t bytes)
    {
        if (bytes == 0) bytes = 16;
        if (g_fail_allocs_after.load(std::memory_order_relaxed) >= 0 && g_fail_allocs_after.fetch_sub(1) <= 0) {
            g_fail_allocs_after.store(0);
            p = nullptr;
            return fail(RFG_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes failed (injected)", bytes);
        }
        cudaError_t e = cudaMallocAsync(&p, bytes, g.stream);
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(RFG_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes failed: %s", bytes,
                        cudaGetErrorString(e));
        }
        return RFG_OK;
    }
    template <typename T>
    T* as() const
    {
        return static_cast<T*>(p);
    }
};

inline bool valid_width(int w) { return w == 1 || w == 2 || w == 4 || w == 8; }

inline u64 unit_at(const void* data, int width, int64_t i)
{
    switch (width) {
    case 1: return ((const uint8_t*)data)[i];
    case 2: return ((const uint16_t*)data)[i];
    case 4: return ((const uint32_t*)data)[i];
    default: return ((const uint64_t*)data)[i];
    }
}

inline bool is_int_result(int metric, int op)
{
    if (metric == RFG_JARO || metric == RFG_JARO_WINKLER || metric >= RFG_RATIO) return false;
    return op == RFG_DISTANCE || op == RFG_SIMILARITY;
}

/* per-thread scratch of the partial_ratio pairs: W + 1 LCS state words, then 5L + 2
 * 32-bit slots for the window search over a haystack of up to L units */
inline int64_t partial_scratch_words(int W, int64_t L) { return (int64_t)W + 1 + (5 * L + 2 + 1) / 2; }

inline int next_pow2(int x)
{
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

/* queries as the engine needs them: device strings plus host lengths and the number of
 * code units >= 256 of each query (sizes the shared-memory hash table) */
struct QuerySet {
    KStrings dev{};
    std::vector<int64_t> len;
    std::vector<int32_t> wide;
    /* distinct code units below 256 per query (the rows of the band kernel's compact
     * table), or -1 where the query's units were not seen on the host */
    std::vector<int32_t> distinct;
};

/* the metrics whose long queries may take the band kernels (their tables need the
 * distinct code units of the query) */
bool band_candidate(int metric)
{
    return metric == RFG_LEVENSHTEIN || metric == RFG_INDEL || metric == RFG_LCSSEQ || metric == RFG_RATIO;
}

/* lengths and wide-unit counts of a host batch; with want_distinct, the distinct units
 * below 256 of every query longer than 64 units (the band-class candidates) */
rfg_status query_info_from_host(const void* data, const int64_t* off, int64_t n, int width, QuerySet* qs,
                                bool want_distinct = false)
{
    qs->len.resize(n);
    qs->wide.assign(n, 0);
    qs->distinct.assign(n, -1);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t a = off[i], b = off[i + 1];
        if (a < 0 || b < a) return fail(RFG_ERR_INVALID_ARGUMENT, "offsets must be non-decreasing and >= 0");
        if (b - a > INT32_MAX) return fail(RFG_ERR_INVALID_ARGUMENT, "strings longer than 2^31-1 code units");
        qs->len[i] = b - a;
        if (!data && b > a) continue;
        const bool dist = want_distinct && b - a > 64;
        if (width == 1 && !dist) continue;
        u64 seen[4] = {0, 0, 0, 0};
        int32_t w = 0;
        for (int64_t k = a; k < b; ++k) {
            const u64 c = unit_at(data, width, k);
            if (c >= 256) ++w;
            else seen[c >> 6] |= 1ull << (c & 63);
        }
        qs->wide[i] = width > 1 ? w : 0;
        if (dist) qs->distinct[i] = popc64(seen[0]) + popc64(seen[1]) + popc64(seen[2]) + popc64(seen[3]);
    }
    return RFG_OK;
}

/* some query is longer than 64 units (a band-class candidate) */
inline bool has_long_query(const int64_t* off, int64_t n)
{
    for (int64_t i = 0; i < n; ++i)
        if (off[i + 1] - off[i] > 64) return true;
    return false;
}

/* copy a host batch to the device (data padded to 16 bytes) */
rfg_status upload_strings(const rfg_strings* s, DBuf* data, DBuf* off, KStrings* out)
{
    const int64_t n = s->count;
    const int64_t units = n > 0 ? s->offsets[n] : 0;
    const size_t bytes = (size_t)units * s->char_width;
    RFG_TRY(data->alloc(bytes + 16));
    RFG_TRY(off->alloc((size_t)(n + 1) * 8));
    if (bytes) RFG_CUDA(cudaMemcpyAsync(data->p, s->data, bytes, cudaMemcpyHostToDevice, g.stream));
    RFG_CUDA(cudaMemcpyAsync(off->p, s->offsets, (size_t)(n + 1) * 8, cudaMemcpyHostToDevice, g.stream));
    out->data = data->as<unsigned char>();
    out->off = off->as<int64_t>();
    out->n = n;
    out->width = s->char_width;
    return RFG_OK;
}

rfg_status check_strings(const rfg_strings* s, const char* what)
{
    if (!s) return fail(RFG_ERR_INVALID_ARGUMENT, "%s is NULL", what);
    if (s->count < 0) return fail(RFG_ERR_INVALID_ARGUMENT, "%s: negative count", what);
    if (!valid_width(s->char_width)) return fail(RFG_ERR_INVALID_ARGUMENT, "%s: char_width must be 1, 2, 4 or 8", what);
    if (!s->offsets) return fail(RFG_ERR_INVALID_ARGUMENT, "%s: offsets is NULL", what);
    return RFG_OK;
}

/* offsets of a host batch: non-decreasing from 0 up, strings shorter than 2^31 units */
rfg_status check_offsets(const int64_t* off, int64_t n, const char* what)
{
    for (int64_t i = 0; i < n; ++i)
        if (off[i] < 0 || off[i + 1] < off[i] || off[i + 1] - off[i] > INT32_MAX)
            return fail(RFG_ERR_INVALID_ARGUMENT, "%s: offsets must be non-decreasing and >= 0", what);
    return RFG_OK;
}

/* token_sort_ratio, partial_token_sort_ratio and QRatio: a host front end over the
 * ratio / partial_ratio engine */
inline bool is_token_metric(int metric)
{
    return (metric >= RFG_TOKEN_SORT_RATIO && metric <= RFG_QRATIO) ||
           (metric >= RFG_TOKEN_SET_RATIO && metric <= RFG_WRATIO);
}
/* the family scored on the device from string parts (FAM_TOKEN) */
inline bool is_token_set_metric(int metric) { return metric >= RFG_TOKEN_SET_RATIO && metric <= RFG_WRATIO; }
inline int token_base(int metric) { return metric == RFG_PARTIAL_TOKEN_SORT_RATIO ? RFG_PARTIAL_RATIO : RFG_RATIO; }

/* the metrics the engine scores directly (every entry point) */
rfg_status check_metric_op(int metric, int op, int form)
{
    if (is_token_metric(metric))
        return fail(RFG_ERR_INVALID_ARGUMENT, "the token scorers take rfg_score_f64, rfg_cached_*, rfg_multi_* and "
                                              "rfg_cdist only");
    if (metric < RFG_LEVENSHTEIN || metric > RFG_PARTIAL_RATIO)
        return fail(RFG_ERR_INVALID_ARGUMENT, "unknown metric %d", metric);
    if (op < RFG_DISTANCE || op > RFG_NORMALIZED_SIMILARITY) return fail(RFG_ERR_INVALID_ARGUMENT, "unknown op %d", op);
    if (form < RFG_FORM_FREE || form > RFG_FORM_MULTI) return fail(RFG_ERR_INVALID_ARGUMENT, "unknown form %d", form);
    if (metric == RFG_RATIO && op != RFG_SIMILARITY)
        return fail(RFG_ERR_INVALID_ARGUMENT, "fuzz::ratio only has a similarity");
    if (metric == RFG_PARTIAL_RATIO && op != RFG_SIMILARITY)
        return fail(RFG_ERR_INVALID_ARGUMENT, "fuzz::partial_ratio only has a similarity");
    if (metric == RFG_PARTIAL_RATIO && form == RFG_FORM_MULTI)
        return fail(RFG_ERR_INVALID_ARGUMENT, "fuzz::partial_ratio has no experimental::Multi form");
    return RFG_OK;
}


/* check_metric_op for the entry points that take the token scorers too */
rfg_status check_any_metric_op(int metric, int op, int form)
{
    if (!is_token_metric(metric)) return check_metric_op(metric, op, form);
    if (op < RFG_DISTANCE || op > RFG_NORMALIZED_SIMILARITY) return fail(RFG_ERR_INVALID_ARGUMENT, "unknown op %d", op);
    if (form < RFG_FORM_FREE || form > RFG_FORM_MULTI) return fail(RFG_ERR_INVALID_ARGUMENT, "unknown form %d", form);
    if (op != RFG_SIMILARITY)
        return fail(RFG_ERR_INVALID_ARGUMENT, "token_sort_ratio, partial_token_sort_ratio and QRatio only have a similarity");
    if ((metric == RFG_PARTIAL_TOKEN_SORT_RATIO || is_token_set_metric(metric)) && form == RFG_FORM_MULTI)
        return fail(RFG_ERR_INVALID_ARGUMENT, "this fuzz scorer has no experimental::Multi form");
    return RFG_OK;
}

ScoreParams to_sp(const rfg_params* p)
{
    ScoreParams sp;
    sp.ins = p ? p->insert_cost : 1;
    sp.del = p ? p->delete_cost : 1;
    sp.rep = p ? p->replace_cost : 1;
    sp.prefix_weight = p ? p->prefix_weight : 0.1;
    return sp;
}

rfg_status check_params(int metric, const ScoreParams& sp)
{
    if (metric == RFG_LEVENSHTEIN && (sp.ins < 0 || sp.del < 0 || sp.rep < 0))
        return fail(RFG_ERR_INVALID_ARGUMENT, "Levenshtein weights must be >= 0");
    return RFG_OK;
}

/* launches whose static plus dynamic shared memory passes 48 KB need the opt-in */
rfg_status allow_dynamic_smem(const void* fn, size_t smem)
{
    static std::map<const void*, size_t> granted;
    auto it = granted.find(fn);
    if (it != granted.end() && it->second >= smem) return RFG_OK;
    cudaFuncAttributes fa;
    RFG_CUDA(cudaFuncGetAttributes(&fa, fn));
    if (fa.sharedSizeBytes + smem > 48 * 1024)
        RFG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    granted[fn] = smem;
    return RFG_OK;
}

int occupancy(const void* fn, int block, size_t smem)
{
    static std::map<std::tuple<const void*, int, size_t>, int> cache;
    const auto key = std::make_tuple(fn, block, smem);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, block, smem) != cudaSuccess || nb < 1) nb = 1;
    cache[key] = nb;
    return nb;
}

/* size class of a query of m code units: pattern words held in registers, 0 = any-length kernel */
inline int word_class(int64_t m)
{
    const int64_t w = (m + 63) / 64;
    if (w <= 1) return 1;
    if (w <= 2) return 2;
    if (w <= 4) return 4;
    if (w <= 8) return 8;
    return 0;
}

struct BatchSpec {
    int metric, op, form;
    ScoreParams sp;
    u64 ci;
    double cf;
    int out_dtype;
    void* out; /* device */
    int64_t ld;
    /* extract epilogue (topk > 0): candidates per (query, chunk) instead of out */
    int topk = 0;
    int tie_last = 0;
    u64* thr = nullptr;
    u64* cand_key = nullptr;
    int64_t* cand_idx = nullptr;
    /* a corpus brings its own chunking and length order */
    const int32_t* fixed_perm = nullptr;
    int64_t fixed_chunk = 0;
    const int32_t* chunk_lmin = nullptr;
    const int32_t* chunk_lmax = nullptr;
    int64_t fixed_maxlen = 0; /* the corpus's longest string */
    /* split the queries into this many contiguous row blocks (host-output pipelining) */
    int row_blocks = 1;
    /* token_set_ratio family: device part-length arrays of the queries and the choices */
    const int32_t* qparts = nullptr;
    const int32_t* cparts = nullptr;
};

inline bool better_high_of(int op) { return op == RFG_SIMILARITY || op == RFG_NORMALIZED_SIMILARITY; }

int64_t g_tiles_target = 0; /* override of the tile-count target (autotuning) */
int g_stage_mode = 1;       /* dense tiles stage their results in shared memory (autotuning) */
int g_mq_mode = 1;          /* one-word unit-weight distances take several queries per thread (autotuning) */
int g_half_mode = 1;        /* queries of <= 32 units run on 32-bit recurrence words (autotuning) */
int g_block_override = 0;   /* override of the tile kernels' block size (autotuning) */
int g_fast_mode = 1;        /* unit-weight one-word distances run on the warp tiles (k_fast) */
/* band launches: the largest pattern table of a band query (bytes), and the shared
 * memory a band CTA takes at most (warps x slice) */
#define RFG_BAND_MAX_TABLE (48 * 1024)
#define RFG_BAND_MAX_SMEM (96 * 1024)
int g_count_filter = 1; /* the warp tiles' count filter (hist_lower_bound) */
int g_band_rounds = 0; /* band units of 32 x this many pairs (0: sized by the class; autotuning) */
int g_band_mode = 1;        /* unit-weight Levenshtein and the LCS families with a band narrower than the pattern run on k_band */
int64_t g_fast_window = 512; /* choice positions per warp window of k_fast (autotuning) */

/* query classes per row block: 0..3 = 1, 2, 4, 8 register words, 4 = any length, 5.. =
 * the band classes (band_class_words(k - 5) 32-bit words of band, rfg_core.cuh) */
constexpr int NCLS = 5 + BAND_CLASSES;

/* the band class of a query of m units (band_class_words index), or -1 (band_class in
 * rfg_core.cuh, shared with the host work counter) */
int band_class_of(const BatchSpec& spec, int64_t m, int64_t maxlen)
{
    return band_class(spec.metric, spec.op, spec.form, spec.sp, spec.ci, spec.cf, m, maxlen);
}

/* A prepared batch: everything a launch needs is on the device, so enqueue() only
 * resets the tile counters and launches the kernels (no host work, no allocation,
 * no synchronisation) -- relaunchable and capturable in a CUDA graph. */
struct LaunchRec {
    const void* fn;
    unsigned grid;
    int block;
    size_t smem;
    KParams a;
    int rblock; /* row block (a contiguous range of queries) the launch belongs to */
    int urgent = 0; /* 1: launched at the device's highest priority (the block's critical path) */
};

struct Prepared {
    std::vector<LaunchRec> launches;
    DBuf packed, small, scratch[1], jtab, chist;
    /* in `packed` (one upload): the query lists of the classes, the choice visiting order
     * and the choices' offsets and lengths in that order (these two: dense results only) */
    const int32_t* qlist = nullptr;
    const int32_t* perm = nullptr;
    const int64_t* poff = nullptr;
    const int32_t* plen = nullptr;
    const int4* prec = nullptr; /* k_fast visiting records */
    const int4* brec = nullptr; /* band launches: the choices' records in length order */
    const BandQuery* bq = nullptr; /* band launches: per-query records, each class's in a run */
    /* which kinds of launches the preparation holds (what the tuner has to sweep) */
    bool has_fast = false, has_band = false, has_tiles = false;
    bool has_pre = false; /* pre.a / grid: the per-query table pass before the row blocks */
    bool has_hist = false; /* hist: the choices' count histograms before the warp tiles */
    KParams hist{};
    KParams pre;
    int* counters = nullptr;
    int* err = nullptr;
    int64_t scratch_words = 0;
    int64_t chunk = 0, nchunks = 0;
    /* query rows of each row block; a host-output cdist copies block b while block b+1
     * computes */
    std::vector<std::pair<int64_t, int64_t>> rows;
    Prepared() = default;
    Prepared(const Prepared&) = delete;
    Prepared& operator=(const Prepared&) = delete;
    void free_on(cudaStream_t st)
    {
        packed.free_on = small.free_on = scratch[0].free_on = jtab.free_on = chist.free_on = st;
    }
};

/* Host-side choice offsets (for the length order of each chunk): read from the device
 * when the batch lives there. */
rfg_status choice_lengths(const KStrings& c, const int64_t* host_off, std::vector<int32_t>* len,
                          std::vector<int64_t>* tmp)
{
    const int64_t nc = c.n;
    if (!host_off) {
        tmp->resize(nc + 1);
        RFG_CUDA(cudaMemcpyAsync(tmp->data(), c.off, (nc + 1) * 8, cudaMemcpyDeviceToHost, g.stream));
        RFG_CUDA(cudaStreamSynchronize(g.stream));
        host_off = tmp->data();
    }
    /* device-resident offsets are seen here first: a batch with broken offsets is
     * refused before any kernel reads strings through them */
    RFG_TRY(check_offsets(host_off, nc, "choices"));
    len->resize(nc);
    for (int64_t i = 0; i < nc; ++i) (*len)[i] = (int32_t)(host_off[i + 1] - host_off[i]);
    return RFG_OK;
}

/* stable counting sort of each chunk's positions by choice length */
void chunk_length_order(const std::vector<int32_t>& len, int64_t chunk, std::vector<int32_t>* perm)
{
    const int64_t nc = (int64_t)len.size();
    perm->resize(nc);
    std::vector<int64_t> count;
    for (int64_t c0 = 0; c0 < nc; c0 += chunk) {
        const int64_t c1 = std::min(nc, c0 + chunk);
        int32_t lo = INT32_MAX, hi = 0;
        for (int64_t i = c0; i < c1; ++i) {
            lo = std::min(lo, len[i]);
            hi = std::max(hi, len[i]);
        }
        const int64_t range = (int64_t)hi - lo + 1;
        if (range > 4 * (c1 - c0) + 1024) { /* wide length range: comparison sort */
            std::vector<int32_t> idx(c1 - c0);
            for (int64_t i = c0; i < c1; ++i) idx[i - c0] = (int32_t)i;
            std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return len[a] < len[b]; });
            std::copy(idx.begin(), idx.end(), perm->begin() + c0);
            continue;
        }
        count.assign(range + 1, 0);
        for (int64_t i = c0; i < c1; ++i) ++count[len[i] - lo + 1];
        for (int64_t k = 1; k <= range; ++k) count[k] += count[k - 1];
        for (int64_t i = c0; i < c1; ++i) (*perm)[c0 + count[len[i] - lo]++] = (int32_t)i;
    }
}

/* query indices (ascending) -> longest first, ties in index order; counting sort when the
 * length range is small */
void sort_by_length_desc(std::vector<int32_t>* v, const std::vector<int64_t>& len)
{
    const size_t n = v->size();
    if (n < 2) return;
    int64_t lo = INT64_MAX, hi = 0;
    for (int32_t i : *v) {
        lo = std::min(lo, len[i]);
        hi = std::max(hi, len[i]);
    }
    if (hi - lo > (int64_t)(4 * n + 1024)) {
        std::stable_sort(v->begin(), v->end(), [&](int32_t a, int32_t b) { return len[a] > len[b]; });
        return;
    }
    std::vector<int32_t> count(hi - lo + 2, 0), out(n);
    for (int32_t i : *v) ++count[hi - len[i] + 1];
    for (size_t k = 1; k < count.size(); ++k) count[k] += count[k - 1];
    for (int32_t i : *v) out[count[hi - len[i]]++] = i;
    v->swap(out);
}

rfg_status prepare_batch(const QuerySet& q, const KStrings& c, const BatchSpec& spec, Prepared* pb,
                         const int64_t* host_choice_off = nullptr)
{
    const int64_t nq = q.dev.n, nc = c.n;
    RFG_TRY(pb->small.alloc(RFG_COUNTERS * sizeof(int)));
    pb->counters = pb->small.as<int>();
    pb->err = pb->counters + RFG_COUNTERS - 1;
    if (nq == 0 || nc == 0) return RFG_OK;
    const int fam = metric_family(spec.metric, spec.form, spec.sp);

    /* row blocks: contiguous query ranges, each with its own launches */
    const int64_t R = std::max<int64_t>(1, std::min<int64_t>({(int64_t)spec.row_blocks, RFG_MAX_ROW_BLOCKS, nq}));
    const int64_t rb = (nq + R - 1) / R;
    for (int64_t b = 0; b < R; ++b) pb->rows.emplace_back(b * rb, std::min(nq, (b + 1) * rb));
    const int64_t nblk = (int64_t)pb->rows.size();

    /* the choices' lengths (for the band classes and the length order below) */
    std::vector<int32_t> clen;
    std::vector<int64_t> off_tmp;
    int64_t host_max_choice_len = 0;
    if (!spec.fixed_perm) {
        RFG_TRY(choice_lengths(c, host_choice_off, &clen, &off_tmp));
        for (int32_t l : clen) host_max_choice_len = std::max<int64_t>(host_max_choice_len, l);
    }
    /* classes: 1, 2, 4, 8 register words; index 4 = any length; 5.. = the band classes of
     * unit-weight Levenshtein and of the LCS families (band_class_words(k - 5) 32-bit
     * words); one set per row block */
    const bool band_fam = (fam == FAM_LEV && spec.metric == RFG_LEVENSHTEIN) ||
                          (fam == FAM_LCS && (spec.metric == RFG_INDEL || spec.metric == RFG_LCSSEQ || spec.metric == RFG_RATIO));
    const bool band_ok = g_band_mode != 0 && band_fam && band_metric(spec.metric, spec.sp) && spec.form != RFG_FORM_MULTI &&
                         spec.topk == 0 && !spec.fixed_perm && c.width == 1 && nc < INT32_MAX;
    std::vector<std::vector<int32_t>> cls(nblk * NCLS);
    std::vector<int64_t> cls_maxlen(nblk * NCLS, 0);
    std::vector<int32_t> cls_wide(nblk * NCLS, 0);
    std::vector<int64_t> cls_bwords(nblk * NCLS, 0); /* band classes: row words of the largest table */
    for (int64_t b = 0; b < nblk; ++b)
        for (int64_t i = pb->rows[b].first; i < pb->rows[b].second; ++i) {
            int k;
            if (fam == FAM_WF || fam == FAM_NONE || fam == FAM_PARTIAL || fam == FAM_TOKEN) k = 4;
            else {
                const int wc = word_class(q.len[i]);
                k = wc == 1 ? 0 : wc == 2 ? 1 : wc == 4 ? 2 : wc == 8 ? 3 : 4;
            }
            int64_t bwords = 0;
            if (band_ok && k > 0 && q.distinct[i] >= 0) {
                const int bc = band_class_of(spec, q.len[i], host_max_choice_len);
                /* the query's table (distinct units + the zero row) must fit a warp's slice */
                if (bc >= 0) bwords = (int64_t)(q.distinct[i] + 1) * band_row_stride((int)q.len[i], band_class_words(bc));
                if (bc >= 0 && bwords * 4 <= RFG_BAND_MAX_TABLE) k = 5 + bc;
            }
            const int64_t bk = b * NCLS + k;
            cls[bk].push_back((int32_t)i);
            cls_maxlen[bk] = std::max(cls_maxlen[bk], q.len[i]);
            cls_wide[bk] = std::max(cls_wide[bk], q.wide[i]);
            if (k >= 5) cls_bwords[bk] = std::max(cls_bwords[bk], bwords);
        }
    size_t total = 0;
    for (auto& v : cls) {
        sort_by_length_desc(&v, q.len);
        total += v.size();
    }
    std::vector<int32_t> qall;
    qall.reserve(total);
    std::vector<size_t> cls_off(nblk * NCLS);
    for (int64_t bk = 0; bk < nblk * NCLS; ++bk) {
        cls_off[bk] = qall.size();
        qall.insert(qall.end(), cls[bk].begin(), cls[bk].end());
    }

    /* one chunking of the choices for every class, each chunk visited in length order */
    int64_t chunk;
    int64_t stage = 0; /* staged window of the dense tiles (elements), 0 = direct stores */
    /* unit-weight distance: the chain is d <= K ? d : K + 1 (fast path of the tile kernels) */
    const bool fast_ok = spec.form != RFG_FORM_MULTI && spec.op == RFG_DISTANCE &&
                         ((spec.metric == RFG_LEVENSHTEIN && fam == FAM_LEV && spec.sp.ins == 1 &&
                           spec.sp.del == 1 && spec.sp.rep == 1) ||
                          spec.metric == RFG_INDEL || spec.metric == RFG_OSA);
    /* the normalized chains of the same unit-weight metrics (integer cutoff tabulated) */
    const bool norm_ok = spec.form != RFG_FORM_MULTI &&
                         (spec.op == RFG_NORMALIZED_DISTANCE || spec.op == RFG_NORMALIZED_SIMILARITY ||
                          spec.metric == RFG_RATIO) &&
                         ((spec.metric == RFG_LEVENSHTEIN && fam == FAM_LEV && spec.sp.ins == 1 &&
                           spec.sp.del == 1 && spec.sp.rep == 1) ||
                          spec.metric == RFG_INDEL || spec.metric == RFG_RATIO || spec.metric == RFG_OSA);
    const bool jaro_ok = fam == FAM_JARO && spec.form != RFG_FORM_MULTI;
    const bool mq_ok = (fast_ok || norm_ok || jaro_ok) && spec.topk == 0 && !spec.fixed_perm && g_stage_mode != 0 &&
                       g_mq_mode != 0;
    const int32_t* dperm = nullptr;
    std::vector<int32_t> perm, pl;
    std::vector<int64_t> po;
    /* the warp tiles (k_fast) take the one-word class of a unit-weight distance whose
     * pattern tables need no hash rows; they visit the choices in windows of their own,
     * each sorted by length, through 16-byte records */
    bool fast_any = false;
    for (int64_t b = 0; b < nblk; ++b)
        if (!cls[b * NCLS].empty() && (c.width == 1 || cls_wide[b * NCLS] == 0)) fast_any = true;
    fast_any = fast_any && fast_ok && spec.topk == 0 && !spec.fixed_perm && g_fast_mode != 0;
    const int64_t fwin = std::max<int64_t>(32, std::min<int64_t>(2048, g_fast_window / 8 * 8));
    std::vector<int32_t> frec;
    if (spec.fixed_perm) {
        chunk = spec.fixed_chunk;
        dperm = spec.fixed_perm;
    }
    else {
        const int64_t target_all = g_tiles_target > 0 ? g_tiles_target : (int64_t)g.sms * 32;
        const int blk = g_block_override > 0 ? g_block_override : 256;
        chunk = (nc * rb + target_all - 1) / target_all;
        chunk = std::max<int64_t>(chunk, blk);
        chunk = std::min<int64_t>(chunk, std::max<int64_t>(nc, 1));
        chunk = (chunk + blk - 1) / blk * blk;
        if (spec.topk == 0 && g_stage_mode != 0) {
            /* windows of up to 32 KB of results, each its own length-sorted run (a
             * quarter of that per query row in the several-queries kernel) */
            const int64_t cap = (spec.out_dtype == RFG_I32 ? 8192 : 4096) / (mq_ok ? mq_queries(fam) : 1);
            if (chunk > cap) chunk = (chunk + cap - 1) / cap * cap;
            stage = std::min(chunk, cap);
        }
        const int64_t* hoff = host_choice_off ? host_choice_off : off_tmp.data();
        chunk_length_order(clen, stage ? stage : chunk, &perm);
        if (spec.topk == 0) {
            /* offsets and lengths in visiting order */
            po.resize(nc);
            pl.resize(nc);
            for (int64_t i = 0; i < nc; ++i) {
                po[i] = hoff[perm[i]];
                pl[i] = clen[perm[i]];
            }
        }
        if (fast_any) {
            std::vector<int32_t> fperm;
            chunk_length_order(clen, fwin, &fperm);
            frec.resize((size_t)nc * 4);
            for (int64_t i = 0; i < nc; ++i) {
                const int32_t ci = fperm[i];
                const uint64_t o = (uint64_t)hoff[ci];
                frec[4 * i] = (int32_t)(uint32_t)o;
                frec[4 * i + 1] = (int32_t)(uint32_t)(o >> 32);
                frec[4 * i + 2] = clen[ci];
                frec[4 * i + 3] = (int32_t)(ci - i / fwin * fwin);
            }
        }
    }
    /* band classes: the choices in one length order ({offset low, high, length, index}),
     * and per query its passing run of that order (band_range) cut into units */
    std::vector<int32_t> brec;
    std::vector<BandQuery> bqv;
    std::vector<size_t> cls_bq(nblk * NCLS, 0);
    std::vector<int64_t> cls_units(nblk * NCLS, 0), cls_rounds(nblk * NCLS, 1);
    bool any_band = false;
    for (int64_t bk = 0; bk < nblk * NCLS; ++bk)
        if (bk % NCLS >= 5 && !cls[bk].empty()) any_band = true;
    if (any_band) {
        const int64_t* hoff = host_choice_off ? host_choice_off : off_tmp.data();
        std::vector<int32_t> gperm;
        chunk_length_order(clen, std::max<int64_t>(nc, 1), &gperm);
        std::vector<int32_t> slen(nc);
        brec.resize((size_t)nc * 4);
        for (int64_t i = 0; i < nc; ++i) {
            const int32_t ci = gperm[i];
            const uint64_t o = (uint64_t)hoff[ci];
            brec[4 * i] = (int32_t)(uint32_t)o;
            brec[4 * i + 1] = (int32_t)(uint32_t)(o >> 32);
            brec[4 * i + 2] = slen[i] = clen[ci];
            brec[4 * i + 3] = ci;
        }
        for (int64_t bk = 0; bk < nblk * NCLS; ++bk) {
            if (bk % NCLS < 5 || cls[bk].empty()) continue;
            const size_t first = bqv.size();
            int64_t npass = 0;
            for (int32_t qi : cls[bk]) {
                i64 nlo = 1, nhi = 0, Kmax = 0;
                BandQuery r{};
                r.qi = qi;
                if (band_range(spec.metric, spec.op, spec.form, spec.sp, spec.ci, spec.cf, q.len[qi], host_max_choice_len,
                               &nlo, &nhi, &Kmax)) {
                    r.nlo = (int32_t)nlo;
                    r.nhi = (int32_t)nhi;
                    r.plo = (int32_t)(std::lower_bound(slen.begin(), slen.end(), r.nlo) - slen.begin());
                    r.phi = (int32_t)(std::upper_bound(slen.begin(), slen.end(), r.nhi) - slen.begin());
                }
                else { /* nothing passes: every pair is filled */
                    r.nlo = 1;
                    r.nhi = 0;
                }
                npass += r.phi - r.plo;
                bqv.push_back(r);
            }
            /* units of `rounds` groups of 32 pairs (one table build each): as many
             * groups as keep about two units per resident warp */
            const int64_t rounds = g_band_rounds > 0 ? g_band_rounds
                                                     : std::min<int64_t>(8, std::max<int64_t>(1, npass / ((int64_t)g.sms * 2048)));
            int64_t ustart = 0;
            for (size_t i = first; i < bqv.size(); ++i) {
                bqv[i].ustart = (int32_t)std::min<int64_t>(ustart, INT32_MAX);
                ustart += (bqv[i].phi - bqv[i].plo + 32 * rounds - 1) / (32 * rounds);
            }
            BandQuery end{};
            end.ustart = (int32_t)std::min<int64_t>(ustart, INT32_MAX);
            bqv.push_back(end);
            cls_bq[bk] = first;
            cls_units[bk] = ustart;
            cls_rounds[bk] = rounds;
        }
    }
    {
        /* the host tables leave in one copy from pinned staging */
        size_t tot = 0;
        auto reserve = [&](size_t bytes) {
            const size_t o = tot;
            tot += (bytes + 15) / 16 * 16;
            return o;
        };
        const size_t oq = reserve(qall.size() * 4), operm = reserve(perm.size() * 4), opo = reserve(po.size() * 8),
                     opl = reserve(pl.size() * 4), ofr = reserve(frec.size() * 4), obr = reserve(brec.size() * 4),
                     obq = reserve(bqv.size() * sizeof(BandQuery));
        unsigned char* h;
        RFG_TRY(upload_stage(tot, &h));
        memcpy(h + oq, qall.data(), qall.size() * 4);
        if (!perm.empty()) memcpy(h + operm, perm.data(), perm.size() * 4);
        if (!po.empty()) memcpy(h + opo, po.data(), po.size() * 8);
        if (!pl.empty()) memcpy(h + opl, pl.data(), pl.size() * 4);
        if (!frec.empty()) memcpy(h + ofr, frec.data(), frec.size() * 4);
        if (!brec.empty()) memcpy(h + obr, brec.data(), brec.size() * 4);
        if (!bqv.empty()) memcpy(h + obq, bqv.data(), bqv.size() * sizeof(BandQuery));
        RFG_TRY(pb->packed.alloc(tot));
        RFG_CUDA(cudaMemcpyAsync(pb->packed.p, h, tot, cudaMemcpyHostToDevice, g.stream));
        RFG_CUDA(cudaEventRecord(g.up_ev, g.stream));
        unsigned char* d = pb->packed.as<unsigned char>();
        pb->qlist = (const int32_t*)(d + oq);
        if (!perm.empty()) dperm = pb->perm = (const int32_t*)(d + operm);
        if (!po.empty()) {
            pb->poff = (const int64_t*)(d + opo);
            pb->plen = (const int32_t*)(d + opl);
        }
        if (!frec.empty()) pb->prec = (const int4*)(d + ofr);
        if (!brec.empty()) pb->brec = (const int4*)(d + obr);
        if (!bqv.empty()) pb->bq = (const BandQuery*)(d + obq);
    }
    pb->chunk = chunk;
    pb->nchunks = (nc + chunk - 1) / chunk;
    const bool topk = spec.topk > 0;
    const int64_t max_choice_len = spec.fixed_perm ? RFG_JT_MAXT : host_max_choice_len;

    std::vector<size_t> generic_recs;
    size_t scratch_bytes = 0;
    /* within a row block the band classes go first, widest first: their few long pairs
     * set the block's critical path, and the block scheduler serves launches in order */
    for (int64_t kb = 0; kb < nblk * NCLS; ++kb) {
        const int kk = (int)(kb % NCLS);
        const int k = kk < BAND_CLASSES ? NCLS - 1 - kk : kk - BAND_CLASSES;
        const int64_t bk = kb - kk + k;
        if (cls[bk].empty()) continue;
        KParams a;
        memset(&a, 0, sizeof a);
        a.q = q.dev;
        a.c = c;
        a.qlist = pb->qlist + cls_off[bk];
        a.nq = (int32_t)cls[bk].size();
        a.counter = pb->counters + bk;
        a.err = pb->err;
        a.metric = spec.metric;
        a.op = spec.op;
        a.form = spec.form;
        a.sp = spec.sp;
        a.ci = spec.ci;
        a.cf = spec.cf;
        a.out = spec.out;
        a.out_dtype = spec.out_dtype;
        a.ld = spec.ld;
        a.qparts = spec.qparts;
        a.cparts = spec.cparts;
        const bool needs_table = fam != FAM_WF && fam != FAM_NONE;
        a.hcap = (needs_table && c.width > 1 && cls_wide[bk] > 0) ? next_pow2(2 * cls_wide[bk]) : 0;

        const void* fn;
        int block;
        size_t smem = 0;
        int per_sm;
        /* a class with too few (query, chunk) tiles to fill the GPU takes smaller tiles
         * with direct stores (a staged window must cover whole sorted runs) */
        const int64_t nchunks_full = (nc + chunk - 1) / chunk;
        const bool small_class =
            k < 4 && !topk && (int64_t)cls[bk].size() * nchunks_full < (int64_t)g.sms * 8 && chunk > 256;
        if (k >= 5) {
            /* banded Levenshtein / LCS: warp tasks of passing pairs and of row fills, each
             * warp with its own table in shared memory */
            const int B = band_class_words(k - 5);
            const bool lcs = fam == FAM_LCS;
            const void* fb = band_kernel(c.width, B, lcs);
            if (!fb) return fail(RFG_ERR_INVALID_ARGUMENT, "no band kernel for this code-unit width");
            a.scratch_per_thread = cls_bwords[bk];
            /* normalized chains: the cutoff table (the LCS families' spans n - m in [-32B, 32B]) */
            const bool norm = spec.op == RFG_NORMALIZED_DISTANCE || spec.op == RFG_NORMALIZED_SIMILARITY ||
                              spec.metric == RFG_RATIO;
            a.tab_t = norm ? (lcs ? 64 * B : 32 * B) : -1;
            if (fast_ok) {
                a.fast = 1;
                a.fast_k = clamp_bound(spec.ci);
            }
            a.prec = pb->brec;
            a.band_q = pb->bq + cls_bq[bk];
            a.chunk = cls_rounds[bk];
            a.nchunks = cls_units[bk];
            const int64_t fills = (int64_t)a.nq * ((nc + RFG_BAND_FILL - 1) / RFG_BAND_FILL);
            if (cls_units[bk] + fills > INT32_MAX) return fail(RFG_ERR_INVALID_ARGUMENT, "batch too large for one launch");
            const size_t per = band_warp_bytes(a.tab_t, a.scratch_per_thread);
            const int warps = (int)std::max<size_t>(1, std::min<size_t>(8, (size_t)RFG_BAND_MAX_SMEM / per));
            const int bblock = 32 * warps;
            const size_t bsm = per * warps;
            RFG_TRY(allow_dynamic_smem(fb, bsm));
            const int64_t bslots = (int64_t)g.sms * std::max(1, occupancy(fb, bblock, bsm));
            const int64_t tasks = cls_units[bk] + fills;
            /* the widest bands hold the longest pairs and few of them: their CTAs are
             * served first, ahead of the classes that fill the GPU */
            pb->launches.push_back(LaunchRec{fb, (unsigned)std::min<int64_t>((tasks + warps - 1) / warps, bslots), bblock,
                                             bsm, a, (int)(bk / NCLS), B >= 4 ? 1 : 0});
            pb->has_band = true;
            continue;
        }
        const bool use_fast = k == 0 && fast_any && a.hcap == 0 && pb->prec;
        const bool use_mq = !use_fast && k == 0 && mq_ok && a.hcap == 0 && stage > 0 && !small_class;
        if (!use_fast) pb->has_tiles = true;
        if (use_fast) {
            /* warp tiles: one task = (Q queries, one window); queries of at most 32 units
             * (the tail of the longest-first class) in their own launch on 32-bit words */
            const int Qf = fast_queries(fam);
            const int fblock = RFG_FAST_WARPS * 32;
            a.prec = pb->prec;
            a.stage = fwin;
            a.nchunks = (nc + fwin - 1) / fwin;
            a.chunk = 1;
            a.fast = 1;
            a.fast_k = clamp_bound(spec.ci);
            const size_t esz = spec.out_dtype == RFG_I32 ? 4 : 8;
            a.vec = ((uintptr_t)spec.out % 16 == 0) && ((spec.ld * (int64_t)esz) % 16 == 0) && (fwin * (int64_t)esz) % 16 == 0;
            /* the count filter, below cutoffs at which a 64-unit pattern's bound can
             * still exceed K (its histograms, one pass over the choices, run first) */
            if (g_count_filter && a.fast_k < 2 * RFG_HIST_MAXLEN) {
                if (!pb->chist.p) {
                    RFG_TRY(pb->chist.alloc((size_t)std::max<int64_t>(nc, 1) * 32));
                    pb->hist = a;
                    pb->has_hist = true;
                }
                a.chist = pb->chist.as<uint4>();
                a.cfilter = 1;
            }
            const std::vector<int32_t>& v = cls[bk];
            int64_t nlong = 0;
            while (nlong < (int64_t)v.size() && q.len[v[nlong]] > 32) ++nlong;
            for (int half = 0; half < 2; ++half) {
                const int64_t n0 = half ? nlong : 0, n1 = half ? (int64_t)v.size() : nlong;
                if (n1 <= n0) continue;
                const void* ff = fam == FAM_LEV ? fast_kernel_lev(c.width, half) : fam == FAM_LCS ? fast_kernel_lcs(c.width, half)
                                                                                              : fast_kernel_osa(c.width, half);
                const size_t fsm = fast_smem_bytes(Qf, half, fwin, a.fast_k < 0xffff);
                RFG_TRY(allow_dynamic_smem(ff, fsm));
                const int64_t fslots = (int64_t)g.sms * occupancy(ff, fblock, fsm);
                KParams h = a;
                h.qlist = a.qlist + n0;
                h.nq = (int32_t)(n1 - n0);
                h.counter = pb->counters + (half ? nblk * NCLS + bk / NCLS : bk);
                const int64_t tasks = (h.nq + Qf - 1) / Qf * h.nchunks;
                if (tasks > INT32_MAX) return fail(RFG_ERR_INVALID_ARGUMENT, "batch too large for one launch");
                const int64_t warps = std::max<int64_t>(1, std::min<int64_t>(tasks, fslots * RFG_FAST_WARPS));
                pb->launches.push_back(
                    LaunchRec{ff, (unsigned)((warps + RFG_FAST_WARPS - 1) / RFG_FAST_WARPS), fblock, fsm, h, (int)(bk / NCLS)});
            }
            pb->has_fast = true;
            continue;
        }
        if (use_mq && fam == FAM_JARO) {
            fn = tiles_mq_kernel_jaro(c.width);
            block = g_block_override > 0 ? g_block_override : 256;
            a.stage = stage;
            smem = tiles_mq_jaro_smem_bytes(stage, mq_queries(fam));
            RFG_TRY(allow_dynamic_smem(fn, smem));
            per_sm = occupancy(fn, block, smem);
        }
        else if (use_mq) {
            switch (fam) {
            case FAM_LEV: fn = tiles_mq_kernel_lev(c.width, !fast_ok, false); break;
            case FAM_LCS: fn = tiles_mq_kernel_lcs(c.width, !fast_ok, false); break;
            default: fn = tiles_mq_kernel_osa(c.width, !fast_ok, false);
            }
            block = g_block_override > 0 ? g_block_override : 256;
            a.stage = stage;
            smem = tiles_mq_smem_bytes(stage, spec.out_dtype,
                                       fast_ok ? 0 : (int)std::min<int64_t>(RFG_JT_MAXT, max_choice_len) + 1,
                                       mq_queries(fam));
            RFG_TRY(allow_dynamic_smem(fn, smem));
            per_sm = occupancy(fn, block, smem);
        }
        else if (k < 4) {
            const int W = 1 << k;
            switch (fam) {
            case FAM_LEV: fn = tiles_kernel_lev(c.width, W, topk); break;
            case FAM_LCS: fn = tiles_kernel_lcs(c.width, W, topk); break;
            case FAM_OSA: fn = tiles_kernel_osa(c.width, W, topk); break;
            default: fn = tiles_kernel_jaro(c.width, W, topk);
            }
            block = g_block_override > 0 ? g_block_override : 256;
            smem = tiles_smem_bytes(W, a.hcap);
            if (stage && !small_class) {
                a.stage = stage;
                smem += (size_t)stage * (spec.out_dtype == RFG_I32 ? 4 : 8);
            }
            RFG_TRY(allow_dynamic_smem(fn, smem));
            per_sm = occupancy(fn, block, smem);
        }
        else {
            fn = generic_kernel(fam == FAM_NONE ? FAM_WF : fam, c.width, topk);
            block = 128;
            const int wmax = (fam == FAM_WF || fam == FAM_NONE) ? 0 : (int)((cls_maxlen[bk] + 63) / 64);
            const size_t table = wmax ? ((size_t)(256 + a.hcap + 1) * wmax + a.hcap) * 8 : 0;
            if (table > 0 && table <= 100 * 1024) {
                /* pattern table in shared memory; per-thread state stays in scratch */
                a.pm_smem = 1;
                smem = table;
                RFG_TRY(allow_dynamic_smem(fn, smem));
            }
            per_sm = std::min(occupancy(fn, block, smem), 8);
        }
        /* tiles: (query, chunk), longest queries first; persistent CTAs fill every SM */
        const int64_t slots = (int64_t)g.sms * per_sm;
        int64_t cchunk = chunk;
        if (small_class) {
            const int64_t want = slots * 4;
            int64_t cc = ((int64_t)cls[bk].size() * nc + want - 1) / want;
            cc = std::max<int64_t>(cc, block);
            cchunk = std::min(chunk, (cc + block - 1) / block * block);
        }
        if (k == 4 && !topk) {
            /* the any-length class has few, heavy queries: smaller tiles so that every
             * resident CTA gets work (no locality is needed here: results go straight out) */
            const int64_t want = slots * 4;
            int64_t cc = ((int64_t)cls[bk].size() * nc + want - 1) / want;
            cc = std::max<int64_t>(cc, block);
            cc = (cc + block - 1) / block * block;
            cchunk = std::min(chunk, cc);
        }
        a.chunk = cchunk;
        a.perm = dperm;
        a.topk = spec.topk;
        a.tie_last = spec.tie_last;
        a.better_high = better_high_of(spec.op);
        a.thr = spec.thr;
        a.cand_key = spec.cand_key;
        a.cand_idx = spec.cand_idx;
        a.chunk_lmin = spec.chunk_lmin;
        a.chunk_lmax = spec.chunk_lmax;
        a.tab_t = (int)std::min<int64_t>(RFG_JT_MAXT, max_choice_len);
        if (fam == FAM_JARO && !topk && spec.form != RFG_FORM_MULTI && k < 4) {
            if (!pb->jtab.p) {
                RFG_TRY(pb->jtab.alloc((size_t)nq * sizeof(JaroTab)));
                pb->pre = a;
                pb->has_pre = true;
            }
            a.jtab = pb->jtab.as<JaroTab>();
        }
        if (pb->poff) {
            a.poff = pb->poff;
            a.plen = pb->plen;
        }
        if (fast_ok) {
            a.fast = 1;
            a.fast_k = clamp_bound(spec.ci);
        }
        a.nchunks = (nc + cchunk - 1) / cchunk;
        const int64_t mqq = mq_queries(fam);
        const int64_t ntiles = (use_mq ? ((int64_t)a.nq + mqq - 1) / mqq : (int64_t)a.nq) * a.nchunks;
        if (ntiles > INT32_MAX) return fail(RFG_ERR_INVALID_ARGUMENT, "batch too large for one launch");
        const int64_t grid = std::min<int64_t>(ntiles, slots);
        if (k == 4) {
            /* any-length kernel: pattern table + per-thread state in global scratch */
            const int wmax = (fam == FAM_WF || fam == FAM_NONE) ? 0 : (int)((cls_maxlen[bk] + 63) / 64);
            int64_t per_thread;
            switch (fam) {
            case FAM_LEV: per_thread = 2 * (int64_t)wmax; break;
            case FAM_LCS: per_thread = wmax; break;
            case FAM_OSA: per_thread = 4 * (int64_t)wmax; break;
            case FAM_JARO: per_thread = 2 * (int64_t)wmax; break;
            case FAM_PARTIAL:
                per_thread = partial_scratch_words(
                    wmax, std::max<int64_t>(cls_maxlen[bk], spec.fixed_perm ? spec.fixed_maxlen : max_choice_len));
                break;
            case FAM_TOKEN:
                per_thread = tok_scratch_words(
                    wmax, std::max<int64_t>(cls_maxlen[bk], spec.fixed_perm ? spec.fixed_maxlen : max_choice_len));
                break;
            default: per_thread = cls_maxlen[bk] + 1;
            }
            a.wmax = wmax;
            a.scratch_per_thread = per_thread;
            a.scratch_per_cta = (wmax && !a.pm_smem ? (int64_t)(256 + a.hcap + 1) * wmax + a.hcap : 0) +
                                (int64_t)block * per_thread;
            /* row blocks run one after another: their any-length launches share one region */
            scratch_bytes = std::max(scratch_bytes, (size_t)grid * a.scratch_per_cta * 8);
            generic_recs.push_back(pb->launches.size());
        }
        if (use_mq && fam != FAM_JARO && g_half_mode) {
            /* the class is sorted longest first: its queries of at most 32 units are the
             * tail, and run in their own launch on 32-bit recurrence words */
            const std::vector<int32_t>& v = cls[bk];
            int64_t nlong = 0;
            while (nlong < (int64_t)v.size() && q.len[v[nlong]] > 32) ++nlong;
            const int64_t nshort = (int64_t)v.size() - nlong;
            if (nshort > 0) {
                const void* fh = fam == FAM_LEV ? tiles_mq_kernel_lev(c.width, !fast_ok, true)
                                 : fam == FAM_LCS ? tiles_mq_kernel_lcs(c.width, !fast_ok, true)
                                                  : tiles_mq_kernel_osa(c.width, !fast_ok, true);
                const int qh = mq_queries_half(fam);
                const size_t smem_h =
                    tiles_mq_smem_bytes(stage, spec.out_dtype,
                                        fast_ok ? 0 : (int)std::min<int64_t>(RFG_JT_MAXT, max_choice_len) + 1, qh);
                RFG_TRY(allow_dynamic_smem(fh, smem_h));
                const int64_t slots_h = (int64_t)g.sms * occupancy(fh, block, smem_h);
                KParams h = a;
                h.qlist = a.qlist + nlong;
                h.nq = (int32_t)nshort;
                h.counter = pb->counters + nblk * NCLS + bk / NCLS;
                const int64_t tiles_h = (nshort + qh - 1) / qh * a.nchunks;
                pb->launches.push_back(
                    LaunchRec{fh, (unsigned)std::min<int64_t>(tiles_h, slots_h), block, smem_h, h, (int)(bk / NCLS)});
                if (nlong == 0) continue;
                a.nq = (int32_t)nlong;
                const int64_t tiles_l = (nlong + mqq - 1) / mqq * a.nchunks;
                pb->launches.push_back(
                    LaunchRec{fn, (unsigned)std::min<int64_t>(tiles_l, slots), block, smem, a, (int)(bk / NCLS)});
                continue;
            }
        }
        pb->launches.push_back(LaunchRec{fn, (unsigned)grid, block, smem, a, (int)(bk / NCLS)});
    }
    if (!generic_recs.empty()) {
        RFG_TRY(pb->scratch[0].alloc(scratch_bytes));
        pb->scratch_words = (int64_t)(scratch_bytes / 8);
        for (size_t i : generic_recs) pb->launches[i].a.scratch = pb->scratch[0].as<u64>();
    }
    return RFG_OK;
}

/* the launches of row block b, forked over side streams and joined back into st */
rfg_status enqueue_block(Prepared& pb, int b, cudaStream_t st)
{
    std::vector<const LaunchRec*> ls;
    for (const LaunchRec& L : pb.launches)
        if (L.rblock == b) ls.push_back(&L);
    const size_t nl = ls.size();
    Ctx::SideSet& ss = g.sides[st];
    while (nl > 1 && ss.side.size() < nl - 1) {
        cudaStream_t x;
        RFG_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        ss.side.push_back(x);
    }
    while (nl > 1 && ss.ev.size() < nl) {
        cudaEvent_t e;
        RFG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ss.ev.push_back(e);
    }
    if (nl > 1) RFG_CUDA(cudaEventRecord(ss.ev[0], st));
    for (size_t i = 0; i < nl; ++i) {
        const LaunchRec& L = *ls[i];
        cudaStream_t s = st;
        if (i > 0) {
            s = ss.side[i - 1];
            RFG_CUDA(cudaStreamWaitEvent(s, ss.ev[0], 0));
        }
        KParams a = L.a;
        void* args[] = {&a};
        if (L.urgent) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(L.grid);
            cfg.blockDim = dim3(L.block);
            cfg.dynamicSmemBytes = L.smem;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributePriority;
            attr[0].val.priority = g.prio_high;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            RFG_CUDA(cudaLaunchKernelExC(&cfg, L.fn, args));
        }
        else
            RFG_CUDA(cudaLaunchKernel(L.fn, dim3(L.grid), dim3(L.block), args, L.smem, s));
        if (i > 0) RFG_CUDA(cudaEventRecord(ss.ev[i], s));
    }
    for (size_t i = 1; i < nl; ++i) RFG_CUDA(cudaStreamWaitEvent(st, ss.ev[i], 0));
    return RFG_OK;
}

/* the per-query table pass that the row blocks read */
rfg_status enqueue_pre(Prepared& pb, cudaStream_t st)
{
    if (pb.has_hist && pb.hist.c.n > 0) {
        KParams h = pb.hist;
        uint4* out = pb.chist.as<uint4>();
        void* hargs[] = {&h, &out};
        const unsigned hgrid = (unsigned)std::min<int64_t>((h.c.n + RFG_HIST_WARPS - 1) / RFG_HIST_WARPS, (int64_t)g.sms * 8);
        RFG_CUDA(cudaLaunchKernel(fast_hist_kernel(), dim3(hgrid), dim3(RFG_HIST_WARPS * 32), hargs, 0, st));
    }
    if (!pb.has_pre || pb.pre.q.n == 0) return RFG_OK;
    KParams a = pb.pre;
    JaroTab* out = pb.jtab.as<JaroTab>();
    void* args[] = {&a, &out};
    RFG_CUDA(cudaLaunchKernel(jaro_tables_kernel(), dim3((unsigned)a.q.n), dim3(256), args, 0, st));
    return RFG_OK;
}

rfg_status enqueue_batch(Prepared& pb, cudaStream_t st)
{
    RFG_CUDA(cudaMemsetAsync(pb.counters, 0, RFG_COUNTERS * sizeof(int), st));
    RFG_TRY(enqueue_pre(pb, st));
    for (size_t b = 0; b < std::max<size_t>(pb.rows.size(), 1); ++b) RFG_TRY(enqueue_block(pb, (int)b, st));
    return RFG_OK;
}

rfg_status check_batch(const Prepared& pb, cudaStream_t st)
{
    int h_err = 0;
    RFG_CUDA(cudaMemcpyAsync(&h_err, pb.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    RFG_CUDA(cudaStreamSynchronize(st));
    if (h_err) return fail(RFG_ERR_DEVICE_CHECK, "device-side check failed (code %d)", h_err);
    return RFG_OK;
}

/* Score every (query, choice) pair on the device, results to spec.out (device). */
rfg_status run_batch(const QuerySet& q, const KStrings& c, const BatchSpec& spec,
                     const int64_t* host_choice_off = nullptr)
{
    Prepared pb;
    RFG_TRY(prepare_batch(q, c, spec, &pb, host_choice_off));
    RFG_TRY(enqueue_batch(pb, g.stream));
    return check_batch(pb, g.stream);
}

size_t dtype_size(int dt) { return dt == RFG_I32 ? 4 : 8; }

rfg_status check_dtype(int metric, int op, int dt)
{
    if (dt < RFG_I32 || dt > RFG_F64) return fail(RFG_ERR_INVALID_ARGUMENT, "unknown output dtype");
    if (!is_int_result(metric, op) && dt != RFG_F64)
        return fail(RFG_ERR_INVALID_ARGUMENT, "this metric/op returns doubles: use RFG_F64");
    return RFG_OK;
}

rfg_status token_cdist(int metric, int op, int form, const rfg_strings* Q, bool q_dev, const rfg_strings* C,
                       bool c_dev, const rfg_params* p, rfg_cutoff cut, int dt, void* out, int64_t ld, bool dev_out);

/* host memory the driver has not pinned or registered */
bool is_pageable(const void* p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return at.type == cudaMemoryTypeUnregistered;
}

constexpr size_t kStageSlot = 32u << 20;

rfg_status stage_reserve(size_t slot)
{
    if (g.stage_slot >= slot) return RFG_OK;
    if (g.stage_h) cudaFreeHost(g.stage_h);
    g.stage_h = nullptr;
    g.stage_slot = 0;
    RFG_CUDA(cudaHostAlloc((void**)&g.stage_h, 2 * slot, cudaHostAllocDefault));
    g.stage_slot = slot;
    return RFG_OK;
}

/* rows of row_bytes from a packed source to dst rows dpitch apart, over the host threads
 * (the first touch of fresh pageable pages is the cost, and it spreads over cores) */
void copy_rows_parallel(unsigned char* dst, size_t dpitch, const unsigned char* src, size_t row_bytes, int64_t rows)
{
    const size_t total = row_bytes * (size_t)rows;
    const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
    const int64_t nt = std::min<int64_t>({hw, 16, std::max<int64_t>(1, (int64_t)(total >> 22))});
    auto part = [&](int64_t t) {
        if (dpitch == row_bytes) { /* one contiguous range */
            const size_t a = total * t / nt, b = total * (t + 1) / nt;
            memcpy(dst + a, src + a, b - a);
            return;
        }
        for (int64_t r = rows * t / nt; r < rows * (t + 1) / nt; ++r)
            memcpy(dst + (size_t)r * dpitch, src + (size_t)r * row_bytes, row_bytes);
    };
    if (nt == 1) {
        part(0);
        return;
    }
    std::vector<std::thread> th;
    for (int64_t t = 1; t < nt; ++t) th.emplace_back(part, t);
    part(0);
    for (auto& x : th) x.join();
}

/* cdist over host or device batches.  qparts / cparts: the device part-length arrays of
 * the token_set_ratio family (Q and C are then the part concatenations) */
rfg_status cdist_impl(int metric, int op, int form, const rfg_strings* Q, const rfg_strings* C, const rfg_params* p,
                      rfg_cutoff cut, int dt, void* out, int64_t ld, uint32_t flags, const int32_t* qparts = nullptr,
                      const int32_t* cparts = nullptr)
{
    if (is_token_metric(metric) && !qparts)
        return token_cdist(metric, op, form, Q, flags & RFG_DEVICE_INPUTS, C, flags & RFG_DEVICE_INPUTS, p, cut, dt, out,
                           ld, flags & RFG_DEVICE_OUTPUT);
    RFG_TRY(qparts ? check_any_metric_op(metric, op, form) : check_metric_op(metric, op, form));
    RFG_TRY(check_strings(Q, "queries"));
    RFG_TRY(check_strings(C, "choices"));
    RFG_TRY(check_dtype(metric, op, dt));
    const ScoreParams sp = to_sp(p);
    RFG_TRY(check_params(metric, sp));
    const int64_t nq = Q->count, nc = C->count;
    if (ld == 0) ld = nc;
    if (ld < nc) return fail(RFG_ERR_INVALID_ARGUMENT, "ld must be >= the number of choices");
    if (!out && nq * nc) return fail(RFG_ERR_INVALID_ARGUMENT, "out is NULL");
    const bool dev_in = flags & RFG_DEVICE_INPUTS;
    if (!dev_in) { /* host offsets are checked before the device is touched */
        RFG_TRY(check_offsets(Q->offsets, nq, "queries"));
        RFG_TRY(check_offsets(C->offsets, nc, "choices"));
    }
    RFG_TRY(ensure_ctx());

    QuerySet qs;
    DBuf qd, qo, cd, co, od;
    KStrings ck;
    if (dev_in) {
        /* pattern tables need the query lengths and wide-unit counts on the host */
        std::vector<int64_t> off(nq + 1);
        RFG_CUDA(cudaMemcpyAsync(off.data(), Q->offsets, (nq + 1) * 8, cudaMemcpyDeviceToHost, g.stream));
        RFG_CUDA(cudaStreamSynchronize(g.stream));
        RFG_TRY(check_offsets(off.data(), nq, "queries")); /* before anything is read through them */
        const bool want = band_candidate(metric) && has_long_query(off.data(), nq);
        std::vector<unsigned char> qh;
        if ((Q->char_width > 1 || want) && nq && off[nq] > off[0]) {
            qh.resize((size_t)off[nq] * Q->char_width);
            RFG_CUDA(cudaMemcpyAsync(qh.data(), Q->data, qh.size(), cudaMemcpyDeviceToHost, g.stream));
            RFG_CUDA(cudaStreamSynchronize(g.stream));
        }
        RFG_TRY(query_info_from_host(qh.data(), off.data(), nq, Q->char_width, &qs, want));
        qs.dev = KStrings{(const unsigned char*)Q->data, Q->offsets, nq, Q->char_width};
        ck = KStrings{(const unsigned char*)C->data, C->offsets, nc, C->char_width};
    }
    else {
        if ((!Q->data && nq && Q->offsets[nq]) || (!C->data && nc && C->offsets[nc]))
            return fail(RFG_ERR_INVALID_ARGUMENT, "string data is NULL");
        RFG_TRY(query_info_from_host(Q->data, Q->offsets, nq, Q->char_width, &qs, band_candidate(metric)));
        for (int64_t i = 0; i < nc; ++i)
            if (C->offsets[i] < 0 || C->offsets[i + 1] < C->offsets[i] || C->offsets[i + 1] - C->offsets[i] > INT32_MAX)
                return fail(RFG_ERR_INVALID_ARGUMENT, "choice offsets must be non-decreasing and >= 0");
        RFG_TRY(upload_strings(Q, &qd, &qo, &qs.dev));
        RFG_TRY(upload_strings(C, &cd, &co, &ck));
    }
    BatchSpec spec;
    spec.metric = metric;
    spec.op = op;
    spec.form = form;
    spec.sp = sp;
    spec.ci = cut.cutoff_i;
    spec.cf = cut.cutoff_f;
    spec.out_dtype = dt;
    spec.ld = ld;
    spec.qparts = qparts;
    spec.cparts = cparts;
    const size_t esz = dtype_size(dt);
    if (flags & RFG_DEVICE_OUTPUT) {
        spec.out = out;
        return run_batch(qs, ck, spec, dev_in ? nullptr : C->offsets);
    }
    if (g.host_stores && nq * nc) {
        /* pinned host memory mapped into the device's address space: the tiles' coalesced
         * row segments cross the host link as they are written, no device buffer and no
         * copy afterwards */
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, out) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) {
            spec.out = at.devicePointer;
            return run_batch(qs, ck, spec, dev_in ? nullptr : C->offsets);
        }
        cudaGetLastError();
    }
    RFG_TRY(od.alloc((size_t)nq * ld * esz));
    spec.out = od.p;
    /* host results: row blocks of about 16 MB, block b copied out while b+1 computes */
    const size_t bytes = (size_t)nq * ld * esz;
    spec.row_blocks = (int)std::min<size_t>(8, std::max<size_t>(1, bytes / (16u << 20)));
    Prepared pb;
    struct CopyJoin { /* the copies end before od and pb are released, on every path */
        ~CopyJoin() { cudaStreamSynchronize(g.copy); }
    } join;
    RFG_TRY(prepare_batch(qs, ck, spec, &pb, dev_in ? nullptr : C->offsets));
    RFG_CUDA(cudaMemsetAsync(pb.counters, 0, RFG_COUNTERS * sizeof(int), g.stream));
    RFG_TRY(enqueue_pre(pb, g.stream));
    const size_t row_bytes = (size_t)nc * esz;
    if (nc && bytes >= (8u << 20) && is_pageable(out)) {
        /* pageable destination: row pieces of <= 32 MB go to pinned staging on the copy
         * stream and on to `out` on the host threads, the next piece in flight meanwhile */
        const int64_t prow = std::max<int64_t>(1, (int64_t)(kStageSlot / row_bytes));
        RFG_TRY(stage_reserve((size_t)prow * row_bytes));
        struct Piece {
            int b;
            int64_t r0, r1;
        };
        std::vector<Piece> pieces;
        for (size_t b = 0; b < pb.rows.size(); ++b) {
            RFG_TRY(enqueue_block(pb, (int)b, g.stream));
            RFG_CUDA(cudaEventRecord(g.blk_ev[b], g.stream));
            for (int64_t r = pb.rows[b].first; r < pb.rows[b].second; r += prow)
                pieces.push_back(Piece{(int)b, r, std::min<int64_t>(pb.rows[b].second, r + prow)});
        }
        auto issue = [&](size_t i) -> rfg_status {
            const Piece& P = pieces[i];
            RFG_CUDA(cudaStreamWaitEvent(g.copy, g.blk_ev[P.b], 0));
            RFG_CUDA(cudaMemcpy2DAsync(g.stage_h + (i & 1) * g.stage_slot, row_bytes,
                                       (const char*)od.p + (size_t)P.r0 * ld * esz, ld * esz, row_bytes, P.r1 - P.r0,
                                       cudaMemcpyDeviceToHost, g.copy));
            RFG_CUDA(cudaEventRecord(g.stage_ev[i & 1], g.copy));
            return RFG_OK;
        };
        if (!pieces.empty()) RFG_TRY(issue(0));
        for (size_t i = 0; i < pieces.size(); ++i) {
            if (i + 1 < pieces.size()) RFG_TRY(issue(i + 1));
            RFG_CUDA(cudaEventSynchronize(g.stage_ev[i & 1]));
            copy_rows_parallel((unsigned char*)out + (size_t)pieces[i].r0 * ld * esz, ld * esz,
                               g.stage_h + (i & 1) * g.stage_slot, row_bytes, pieces[i].r1 - pieces[i].r0);
        }
        RFG_CUDA(cudaStreamSynchronize(g.copy));
        return check_batch(pb, g.stream);
    }
    for (size_t b = 0; b < pb.rows.size(); ++b) {
        RFG_TRY(enqueue_block(pb, (int)b, g.stream));
        const int64_t r0 = pb.rows[b].first, r1 = pb.rows[b].second;
        if (r1 <= r0 || nc == 0) continue;
        RFG_CUDA(cudaEventRecord(g.blk_ev[b], g.stream));
        RFG_CUDA(cudaStreamWaitEvent(g.copy, g.blk_ev[b], 0));
        RFG_CUDA(cudaMemcpy2DAsync((char*)out + (size_t)r0 * ld * esz, ld * esz,
                                   (const char*)od.p + (size_t)r0 * ld * esz, ld * esz, nc * esz, r1 - r0,
                                   cudaMemcpyDeviceToHost, g.copy));
    }
    RFG_CUDA(cudaStreamSynchronize(g.copy));
    return check_batch(pb, g.stream);
}

/* a host copy of a batch (the token front end downloads device batches) */
struct HostStrings {
    std::vector<unsigned char> data;
    std::vector<int64_t> off;
};


rfg_status download_strings(const rfg_strings* s, HostStrings* h, const char* what)
{
    const int64_t n = s->count;
    h->off.assign((size_t)n + 1, 0);
    RFG_CUDA(cudaMemcpyAsync(h->off.data(), s->offsets, (size_t)(n + 1) * 8, cudaMemcpyDeviceToHost, g.stream));
    RFG_CUDA(cudaStreamSynchronize(g.stream));
    RFG_TRY(check_offsets(h->off.data(), n, what));
    const size_t bytes = n ? (size_t)h->off[n] * s->char_width : 0;
    h->data.assign(bytes + 16, 0);
    if (bytes) {
        RFG_CUDA(cudaMemcpyAsync(h->data.data(), s->data, bytes, cudaMemcpyDeviceToHost, g.stream));
        RFG_CUDA(cudaStreamSynchronize(g.stream));
    }
    return RFG_OK;
}

/* token_sort_ratio / partial_token_sort_ratio (fuzz_impl.hpp:294-360): the engine's ratio /
 * partial_ratio over sorted_split(s).join() of every string, made on the host threads
 * (rfg_token.cpp); the reference's `score_cutoff > 100` early exit is the engine's own
 * result there.  QRatio (fuzz_impl.hpp:887-931): ratio, then 0 wherever the query or the
 * choice is empty (ratio only gives a non-zero there when both are). */
rfg_status token_cdist(int metric, int op, int form, const rfg_strings* Q, bool q_dev, const rfg_strings* C,
                       bool c_dev, const rfg_params* p, rfg_cutoff cut, int dt, void* out, int64_t ld, bool dev_out)
{
    RFG_TRY(check_any_metric_op(metric, op, form));
    RFG_TRY(check_strings(Q, "queries"));
    RFG_TRY(check_strings(C, "choices"));
    RFG_TRY(check_dtype(metric, op, dt));
    const int64_t nq = Q->count, nc = C->count;
    if (ld == 0) ld = nc;
    if (ld < nc) return fail(RFG_ERR_INVALID_ARGUMENT, "ld must be >= the number of choices");
    if (!out && nq * nc) return fail(RFG_ERR_INVALID_ARGUMENT, "out is NULL");
    RFG_TRY(ensure_ctx());
    HostStrings hq, hc, jq, jc;
    rfg_strings q = *Q, c = *C;
    if (q_dev) {
        RFG_TRY(download_strings(Q, &hq, "queries"));
        q.data = hq.data.data();
        q.offsets = hq.off.data();
    }
    if (c_dev) {
        RFG_TRY(download_strings(C, &hc, "choices"));
        c.data = hc.data.data();
        c.offsets = hc.off.data();
    }
    RFG_TRY(check_offsets(q.offsets, nq, "queries"));
    RFG_TRY(check_offsets(c.offsets, nc, "choices"));
    if ((!q.data && nq && q.offsets[nq] > q.offsets[0]) || (!c.data && nc && c.offsets[nc] > c.offsets[0]))
        return fail(RFG_ERR_INVALID_ARGUMENT, "string data is NULL");
    if (is_token_set_metric(metric)) {
        /* the parts each metric reads: the string (WRatio), S (all but
         * partial_token_set_ratio), J (the partial forms and WRatio) */
        const bool orig = metric == RFG_WRATIO, srt = metric != RFG_PARTIAL_TOKEN_SET_RATIO;
        const bool ddp = metric == RFG_PARTIAL_TOKEN_SET_RATIO || metric == RFG_PARTIAL_TOKEN_RATIO || metric == RFG_WRATIO;
        std::vector<int32_t> qp, cp;
        token_parts_set(q.data, q.offsets, nq, q.char_width, orig, srt, ddp, &jq.data, &jq.off, &qp);
        token_parts_set(c.data, c.offsets, nc, c.char_width, orig, srt, ddp, &jc.data, &jc.off, &cp);
        q.data = jq.data.data();
        q.offsets = jq.off.data();
        c.data = jc.data.data();
        c.offsets = jc.off.data();
        DBuf dqp, dcp;
        RFG_TRY(dqp.alloc(qp.size() * 4));
        RFG_TRY(dcp.alloc(cp.size() * 4));
        if (!qp.empty()) RFG_CUDA(cudaMemcpyAsync(dqp.p, qp.data(), qp.size() * 4, cudaMemcpyHostToDevice, g.stream));
        if (!cp.empty()) RFG_CUDA(cudaMemcpyAsync(dcp.p, cp.data(), cp.size() * 4, cudaMemcpyHostToDevice, g.stream));
        return cdist_impl(metric, op, form, &q, &c, p, cut, dt, out, ld, dev_out ? RFG_DEVICE_OUTPUT : 0,
                          dqp.as<int32_t>(), dcp.as<int32_t>());
    }
    if (metric != RFG_QRATIO) {
        token_sort_join_set(q.data, q.offsets, nq, q.char_width, &jq.data, &jq.off);
        token_sort_join_set(c.data, c.offsets, nc, c.char_width, &jc.data, &jc.off);
        q.data = jq.data.data();
        q.offsets = jq.off.data();
        c.data = jc.data.data();
        c.offsets = jc.off.data();
    }
    RFG_TRY(cdist_impl(token_base(metric), op, form, &q, &c, p, cut, dt, out, ld, dev_out ? RFG_DEVICE_OUTPUT : 0));
    if (metric != RFG_QRATIO) return RFG_OK;
    std::vector<int64_t> lists; /* empty query rows, then empty choice columns */
    for (int64_t i = 0; i < nq; ++i)
        if (q.offsets[i + 1] == q.offsets[i]) lists.push_back(i);
    const int64_t nr = (int64_t)lists.size();
    for (int64_t j = 0; j < nc; ++j)
        if (c.offsets[j + 1] == c.offsets[j]) lists.push_back(j);
    const int64_t ncol = (int64_t)lists.size() - nr;
    if (!nr || !ncol) return RFG_OK;
    if (!dev_out) {
        for (int64_t a = 0; a < nr; ++a)
            for (int64_t b = 0; b < ncol; ++b) ((double*)out)[lists[a] * ld + lists[nr + b]] = 0.0;
        return RFG_OK;
    }
    DBuf d;
    RFG_TRY(d.alloc(lists.size() * 8));
    RFG_CUDA(cudaMemcpyAsync(d.p, lists.data(), lists.size() * 8, cudaMemcpyHostToDevice, g.stream));
    double* o = (double*)out;
    const int64_t* rows = d.as<int64_t>();
    const int64_t* cols = rows + nr;
    void* args[] = {&o, &ld, &rows, (void*)&nr, &cols, (void*)&ncol};
    const int64_t blocks = std::min<int64_t>((nr * ncol + 255) / 256, 152 * 16);
    RFG_CUDA(cudaLaunchKernel(zero_pairs_kernel(), dim3((unsigned)blocks), dim3(256), args, 0, g.stream));
    return RFG_OK;
}

/* One pair in one round trip (the per-call path of the free functions and the cached
 * scorers): both strings, their offsets, the tile list and the zeroed counter and check
 * flag leave in one copy from pinned staging memory, one CTA of the any-length kernel
 * scores the pair, and the check flag and the result return in one copy.
 *
 * The reference's Cached* scorers are const and are called from many host threads at
 * once (its README's OpenMP loop over choices), so this path takes no library-wide
 * lock: every host thread gets a slot of its own -- pinned staging, device staging and
 * scratch, and a stream -- on its first call, and its calls run on that stream while
 * other threads' calls run on theirs.  Past kPairMaxSlots threads, slots are shared
 * (each slot's mutex serialises its users). */
struct PairSlot {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    unsigned char* h = nullptr; /* pinned */
    unsigned char* d = nullptr;
    u64* scratch = nullptr;
};
constexpr size_t kPairStage = 64 * 1024, kPairHead = 128, kPairScratchWords = 128 * 1024;
constexpr int64_t kPairMaxLen1 = 1024;
constexpr size_t kPairMaxSlots = 64;
std::mutex g_slot_mu;
std::vector<PairSlot*> g_slots; /* never freed: streams and staging live as long as the process */
size_t g_slot_next = 0;
thread_local PairSlot* t_slot = nullptr;

rfg_status pair_slot(PairSlot** out)
{
    if (t_slot) {
        *out = t_slot;
        return RFG_OK;
    }
    std::lock_guard<std::mutex> lk(g_slot_mu);
    if (g_slots.size() >= kPairMaxSlots) {
        t_slot = g_slots[g_slot_next++ % g_slots.size()];
        *out = t_slot;
        return RFG_OK;
    }
    PairSlot* s = new PairSlot();
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&s->h, kPairStage, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->d, kPairStage);
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->scratch, kPairScratchWords * 8);
    if (e != cudaSuccess) {
        if (s->scratch) cudaFree(s->scratch);
        if (s->d) cudaFree(s->d);
        if (s->h) cudaFreeHost(s->h);
        if (s->stream) cudaStreamDestroy(s->stream);
        delete s;
        return fail(RFG_ERR_OUT_OF_MEMORY, "per-thread staging of the per-call path: %s", cudaGetErrorString(e));
    }
    g_slots.push_back(s);
    t_slot = s;
    *out = s;
    return RFG_OK;
}

/* RFG_OK with *done = false: the pair does not fit the one-trip layout (the caller takes
 * the batch path) */
rfg_status score_pair_trip(int metric, int op, int form, const void* s1, int64_t l1, int w1, const void* s2,
                           int64_t l2, int w2, const ScoreParams& sp, rfg_cutoff cut, int dt, void* result,
                           bool* done, const int32_t* qparts = nullptr, const int32_t* cparts = nullptr)
{
    *done = false;
    const size_t b1 = (size_t)l1 * w1, b2 = (size_t)l2 * w2;
    const size_t o1 = kPairHead, o2 = (o1 + b1 + 15) / 16 * 16;
    if (l1 > kPairMaxLen1 || o2 + b2 + 16 > kPairStage) return RFG_OK;
    const int fam = metric_family(metric, form, sp);
    QuerySet qs;
    const int64_t qo[2] = {0, l1};
    RFG_TRY(query_info_from_host(s1, qo, 1, w1, &qs));
    const int hcap = (fam != FAM_WF && fam != FAM_NONE && w2 > 1 && qs.wide[0] > 0) ? next_pow2(2 * qs.wide[0]) : 0;
    const int wmax = (fam == FAM_WF || fam == FAM_NONE) ? 0 : (int)std::max<int64_t>(1, (l1 + 63) / 64);
    int64_t per_thread;
    switch (fam) {
    case FAM_LEV: per_thread = 2 * (int64_t)wmax; break;
    case FAM_LCS: per_thread = wmax; break;
    case FAM_OSA: per_thread = 4 * (int64_t)wmax; break;
    case FAM_JARO: per_thread = 2 * (int64_t)wmax; break;
    case FAM_PARTIAL: per_thread = partial_scratch_words(wmax, std::max(l1, l2)); break;
    case FAM_TOKEN: per_thread = tok_scratch_words(wmax, std::max(l1, l2)); break;
    default: per_thread = l1 + 1;
    }
    if (fam == FAM_TOKEN && (!qparts || !cparts)) return RFG_OK;
    const int block = 128;
    const int64_t table = wmax ? (int64_t)(256 + hcap + 1) * wmax + hcap : 0;
    if (table + block * per_thread > (int64_t)kPairScratchWords) return RFG_OK;
    PairSlot* slot;
    RFG_TRY(pair_slot(&slot));
    std::lock_guard<std::mutex> slot_lk(slot->mu);
    const cudaStream_t st = slot->stream;

    unsigned char* h = slot->h;
    unsigned char* d = slot->d;
    int64_t* hoff = (int64_t*)h;
    hoff[0] = 0;
    hoff[1] = l1;
    hoff[2] = 0;
    hoff[3] = l2;
    ((int32_t*)(h + 32))[0] = 0; /* qlist */
    ((int32_t*)(h + 36))[0] = 0; /* tile counter */
    ((int32_t*)(h + 40))[0] = 0; /* check flag */
    if (qparts) { /* the part lengths of the token_set_ratio family */
        memcpy(h + 64, qparts, 12);
        memcpy(h + 80, cparts, 12);
    }
    if (b1) memcpy(h + o1, s1, b1);
    if (b2) memcpy(h + o2, s2, b2);
    RFG_CUDA(cudaMemcpyAsync(d, h, o2 + b2, cudaMemcpyHostToDevice, st));

    KParams a;
    memset(&a, 0, sizeof a);
    a.q = KStrings{d + o1, (const int64_t*)d, 1, w1};
    a.c = KStrings{d + o2, (const int64_t*)(d + 16), 1, w2};
    a.qlist = (const int32_t*)(d + 32);
    a.nq = 1;
    a.chunk = 1;
    a.nchunks = 1;
    a.counter = (int*)(d + 36);
    a.err = (int*)(d + 40);
    a.metric = metric;
    a.op = op;
    a.form = form;
    a.sp = sp;
    a.ci = cut.cutoff_i;
    a.cf = cut.cutoff_f;
    /* the one-pair calls carry the reference's score_hint (the batch calls have none) */
    a.hint_i = cut.hint_i;
    a.hint_f = cut.hint_f;
    a.has_hint = 1;
    a.out = d + 48;
    a.out_dtype = dt;
    a.ld = 1;
    a.hcap = hcap;
    a.tab_t = -1;
    a.better_high = better_high_of(op);
    a.wmax = wmax;
    a.scratch = slot->scratch;
    if (qparts) {
        a.qparts = (const int32_t*)(d + 64);
        a.cparts = (const int32_t*)(d + 80);
    }
    a.scratch_per_thread = per_thread;
    a.scratch_per_cta = table + block * per_thread;
    const void* fn = generic_kernel(fam == FAM_NONE ? FAM_WF : fam, w2, false);
    void* args[] = {&a};
    RFG_CUDA(cudaLaunchKernel(fn, dim3(1), dim3(block), args, 0, st));
    RFG_CUDA(cudaMemcpyAsync(h + 40, d + 40, 16, cudaMemcpyDeviceToHost, st));
    RFG_CUDA(cudaStreamSynchronize(st));
    const int err = ((int32_t*)(h + 40))[0];
    if (err) return fail(RFG_ERR_DEVICE_CHECK, "device-side check failed (code %d)", err);
    memcpy(result, h + 48, 8);
    *done = true;
    return RFG_OK;
}

/* one pair of the token_set_ratio family: host parts, then the one-trip path (or the batch
 * path for pairs too long for its staging) */
rfg_status token_set_one(int metric, int op, int form, const void* s1, int64_t l1, int w1, const void* s2, int64_t l2,
                         int w2, const rfg_params* p, rfg_cutoff cut, int dt, void* result)
{
    const bool orig = metric == RFG_WRATIO, srt = metric != RFG_PARTIAL_TOKEN_SET_RATIO;
    const bool ddp = metric == RFG_PARTIAL_TOKEN_SET_RATIO || metric == RFG_PARTIAL_TOKEN_RATIO || metric == RFG_WRATIO;
    const int64_t o1[2] = {0, l1}, o2[2] = {0, l2};
    std::vector<unsigned char> d1, d2;
    std::vector<int64_t> f1, f2;
    std::vector<int32_t> p1, p2;
    token_parts_set(s1, o1, 1, w1, orig, srt, ddp, &d1, &f1, &p1);
    token_parts_set(s2, o2, 1, w2, orig, srt, ddp, &d2, &f2, &p2);
    bool done = false;
    RFG_TRY(score_pair_trip(metric, op, form, d1.data(), f1[1], w1, d2.data(), f2[1], w2, to_sp(p), cut, dt, result,
                            &done, p1.data(), p2.data()));
    if (done) return RFG_OK;
    int64_t q1[2] = {0, l1}, q2[2] = {0, l2};
    rfg_strings q{s1, q1, 1, w1}, c{s2, q2, 1, w2};
    std::lock_guard<std::recursive_mutex> lk(g.mu); /* the batch path shares the library's stream */
    return token_cdist(metric, op, form, &q, false, &c, false, p, cut, dt, result, 1, false);
}

/* one pair through the engine */
rfg_status score_one(int metric, int op, int form, const void* s1, int64_t l1, int w1, const void* s2, int64_t l2,
                     int w2, const rfg_params* p, rfg_cutoff cut, int dt, void* result)
{
    if (!valid_width(w1) || !valid_width(w2)) return fail(RFG_ERR_INVALID_ARGUMENT, "char width must be 1, 2, 4 or 8");
    if (l1 < 0 || l2 < 0) return fail(RFG_ERR_INVALID_ARGUMENT, "negative length");
    if ((!s1 && l1) || (!s2 && l2)) return fail(RFG_ERR_INVALID_ARGUMENT, "string data is NULL");
    if (!result) return fail(RFG_ERR_INVALID_ARGUMENT, "result is NULL");
    RFG_TRY(check_any_metric_op(metric, op, form));
    RFG_TRY(check_dtype(metric, op, dt));
    const ScoreParams sp = to_sp(p);
    RFG_TRY(check_params(metric, sp));
    RFG_TRY(ensure_ctx());
    if (is_token_set_metric(metric)) return token_set_one(metric, op, form, s1, l1, w1, s2, l2, w2, p, cut, dt, result);
    std::vector<unsigned char> j1, j2;
    if (is_token_metric(metric)) { /* the front end of token_cdist, for one pair */
        if (metric == RFG_QRATIO && (!l1 || !l2)) {
            *(double*)result = 0.0;
            return RFG_OK;
        }
        if (metric != RFG_QRATIO) {
            l1 = token_sort_join(s1, l1, w1, &j1);
            l2 = token_sort_join(s2, l2, w2, &j2);
            s1 = j1.data();
            s2 = j2.data();
        }
        metric = token_base(metric);
    }
    bool done = false;
    RFG_TRY(score_pair_trip(metric, op, form, s1, l1, w1, s2, l2, w2, sp, cut, dt, result, &done));
    if (done) return RFG_OK;
    int64_t o1[2] = {0, l1}, o2[2] = {0, l2};
    rfg_strings q{s1, o1, 1, w1}, c{s2, o2, 1, w2};
    std::lock_guard<std::recursive_mutex> lk(g.mu); /* the batch path shares the library's stream */
    return cdist_impl(metric, op, form, &q, &c, p, cut, dt, result, 1, 0);
}

} // namespace

namespace rfg {
/* error message of the calling thread, set from other translation units */
rfg_status set_last_error(rfg_status s, const char* msg)
{
    g_err = msg;
    return s;
}
} // namespace rfg

/* ======================================================================== C ABI */

struct rfg_cached_s {
    int metric;
    rfg_params params;
    int width;
    int64_t len;
    std::vector<unsigned char> host; /* s1 (the reference's CachedX keeps a copy too) */
    DBuf data, off;
    QuerySet qs;
};

struct rfg_batch_s {
    QuerySet qs;
    KStrings ck{};
    DBuf qd, qo, cd, co;
    BatchSpec spec{};
    Prepared* pb = nullptr;
    cudaGraphExec_t graph = nullptr;
    int block = 0;
    int64_t tiles = 0;
    ~rfg_batch_s()
    {
        if (graph) cudaGraphExecDestroy(graph);
        delete pb;
    }
};

struct rfg_corpus_s {
    DBuf data, off, perm, lmin, lmax;
    KStrings dev{};
    int64_t chunk = 0;
    int64_t count = 0;
    int64_t maxlen = 0; /* longest string */
    /* the token scorers' twin, built on first use: every string as [string][S][J] (its
     * sorted-split join and the join of its distinct tokens) with the part lengths */
    bool tok = false;
    DBuf tdata, toff, tparts;
    KStrings tdev{};
    int64_t tmaxlen = 0;
};

struct rfg_multi_s {
    int metric;
    int max_len;
    size_t count;
    rfg_params params;
    std::vector<std::vector<u64>> strs; /* inserted strings, code units */
    int width = 1;                      /* widest code unit seen */
};

extern "C" {

int rfg_abi_version(void) { return RFG_ABI_VERSION; }

const char* rfg_last_error(void) { return g_err.c_str(); }

rfg_status rfg_set_device(int device)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (g.init && device != g.device) return fail(RFG_ERR_INVALID_ARGUMENT, "device already selected");
    g.device = device;
    return ensure_ctx();
}

rfg_status rfg_testing_fail_device_allocs(int64_t after)
{
    g_fail_allocs_after.store(after < 0 ? -1 : after);
    return RFG_OK;
}

rfg_status rfg_testing_band_rounds(int32_t rounds)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    g_band_rounds = rounds > 0 ? std::min(rounds, 64) : 0;
    return RFG_OK;
}

rfg_status rfg_testing_band_mode(int32_t on)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    g_band_mode = on ? 1 : 0;
    return RFG_OK;
}

rfg_status rfg_synchronize(void)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    RFG_TRY(ensure_ctx());
    RFG_CUDA(cudaStreamSynchronize(g.stream));
    return RFG_OK;
}

rfg_status rfg_score_i64(rfg_metric metric, rfg_op op, const void* s1, int64_t len1, int32_t width1, const void* s2,
                         int64_t len2, int32_t width2, const rfg_params* params, uint64_t score_cutoff,
                         uint64_t score_hint, int64_t* result)
{
    /* no library-wide lock: the per-pair path runs on this thread's own slot */
    if (!is_int_result(metric, op)) return fail(RFG_ERR_INVALID_ARGUMENT, "this metric/op returns a double");
    rfg_cutoff cut{score_cutoff, 0.0, score_hint, 0.0};
    return score_one(metric, op, RFG_FORM_FREE, s1, len1, width1, s2, len2, width2, params, cut, RFG_I64, result);
}

rfg_status rfg_score_f64(rfg_metric metric, rfg_op op, const void* s1, int64_t len1, int32_t width1, const void* s2,
                         int64_t len2, int32_t width2, const rfg_params* params, double score_cutoff, double score_hint,
                         double* result)
{
    if (is_int_result(metric, op)) return fail(RFG_ERR_INVALID_ARGUMENT, "this metric/op returns an integer");
    rfg_cutoff cut{0, score_cutoff, 0, score_hint};
    return score_one(metric, op, RFG_FORM_FREE, s1, len1, width1, s2, len2, width2, params, cut, RFG_F64, result);
}

rfg_status rfg_cached_create(rfg_metric metric, const void* s1, int64_t len1, int32_t width1, const rfg_params* params,
                             rfg_cached* out)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!out) return fail(RFG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    const bool sim_only = metric == RFG_RATIO || metric == RFG_PARTIAL_RATIO || is_token_metric(metric);
    RFG_TRY(check_any_metric_op(metric, sim_only ? RFG_SIMILARITY : RFG_DISTANCE, RFG_FORM_CACHED));
    if (!valid_width(width1)) return fail(RFG_ERR_INVALID_ARGUMENT, "char width must be 1, 2, 4 or 8");
    if (len1 < 0 || (!s1 && len1)) return fail(RFG_ERR_INVALID_ARGUMENT, "invalid s1");
    RFG_TRY(check_params(metric, to_sp(params)));
    RFG_TRY(ensure_ctx());
    rfg_cached_s* h = new rfg_cached_s();
    h->metric = metric;
    const ScoreParams sp = to_sp(params);
    h->params = rfg_params{sp.ins, sp.del, sp.rep, sp.prefix_weight};
    h->width = width1;
    h->len = len1;
    h->host.assign((const unsigned char*)s1, (const unsigned char*)s1 + len1 * width1);
    if (metric == RFG_TOKEN_SORT_RATIO || metric == RFG_PARTIAL_TOKEN_SORT_RATIO) { /* the sorted-split join, as
                                                                                      CachedTokenSortRatio keeps */
        std::vector<unsigned char> j;
        len1 = h->len = token_sort_join(s1, len1, width1, &j);
        h->host.assign(j.begin(), j.begin() + len1 * width1);
    }
    int64_t off[2] = {0, len1};
    rfg_strings q{h->host.data(), off, 1, width1};
    rfg_status st = query_info_from_host(h->host.data(), off, 1, width1, &h->qs, band_candidate(metric));
    if (st == RFG_OK) st = upload_strings(&q, &h->data, &h->off, &h->qs.dev);
    if (st == RFG_OK && cudaStreamSynchronize(g.stream) != cudaSuccess) st = fail(RFG_ERR_CUDA, "upload failed");
    if (st != RFG_OK) {
        delete h;
        return st;
    }
    *out = h;
    return RFG_OK;
}

rfg_status rfg_cached_destroy(rfg_cached h)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    delete h;
    return RFG_OK;
}

static rfg_status cached_many(rfg_cached h, int op, const rfg_strings* C, rfg_cutoff cut, int dt, void* out,
                              uint32_t flags)
{
    if (!h) return fail(RFG_ERR_INVALID_ARGUMENT, "scorer is NULL");
    if (is_token_metric(h->metric)) {
        int64_t qo[2] = {0, h->len};
        rfg_strings q{h->host.data(), qo, 1, h->width};
        return token_cdist(h->metric, op, RFG_FORM_CACHED, &q, false, C, flags & RFG_DEVICE_INPUTS, &h->params, cut, dt,
                           out, C ? C->count : 0, flags & RFG_DEVICE_OUTPUT);
    }
    RFG_TRY(check_metric_op(h->metric, op, RFG_FORM_CACHED));
    RFG_TRY(check_strings(C, "choices"));
    RFG_TRY(check_dtype(h->metric, op, dt));
    RFG_TRY(ensure_ctx());
    const int64_t nc = C->count;
    DBuf cd, co, od;
    KStrings ck;
    if (flags & RFG_DEVICE_INPUTS) ck = KStrings{(const unsigned char*)C->data, C->offsets, nc, C->char_width};
    else {
        for (int64_t i = 0; i < nc; ++i)
            if (C->offsets[i] < 0 || C->offsets[i + 1] < C->offsets[i])
                return fail(RFG_ERR_INVALID_ARGUMENT, "choice offsets must be non-decreasing and >= 0");
        RFG_TRY(upload_strings(C, &cd, &co, &ck));
    }
    BatchSpec spec;
    spec.metric = h->metric;
    spec.op = op;
    spec.form = RFG_FORM_CACHED;
    spec.sp = to_sp(&h->params);
    spec.ci = cut.cutoff_i;
    spec.cf = cut.cutoff_f;
    spec.out_dtype = dt;
    spec.ld = nc;
    if (flags & RFG_DEVICE_OUTPUT) spec.out = out;
    else {
        RFG_TRY(od.alloc((size_t)nc * dtype_size(dt)));
        spec.out = od.p;
    }
    RFG_TRY(run_batch(h->qs, ck, spec, (flags & RFG_DEVICE_INPUTS) ? nullptr : C->offsets));
    if (!(flags & RFG_DEVICE_OUTPUT) && nc) {
        RFG_CUDA(cudaMemcpyAsync(out, od.p, (size_t)nc * dtype_size(dt), cudaMemcpyDeviceToHost, g.stream));
        RFG_CUDA(cudaStreamSynchronize(g.stream));
    }
    return RFG_OK;
}

rfg_status rfg_cached_score_i64(rfg_cached h, rfg_op op, const void* s2, int64_t len2, int32_t width2,
                                uint64_t score_cutoff, uint64_t score_hint, int64_t* result)
{
    /* const and reentrant like CachedX::distance: no library-wide lock on the per-pair path */
    if (!h) return fail(RFG_ERR_INVALID_ARGUMENT, "scorer is NULL");
    if (!is_int_result(h->metric, op)) return fail(RFG_ERR_INVALID_ARGUMENT, "this metric/op returns a double");
    if (!valid_width(width2) || len2 < 0 || (!s2 && len2) || !result) return fail(RFG_ERR_INVALID_ARGUMENT, "invalid s2");
    RFG_TRY(check_metric_op(h->metric, op, RFG_FORM_CACHED));
    RFG_TRY(ensure_ctx());
    bool done = false;
    RFG_TRY(score_pair_trip(h->metric, op, RFG_FORM_CACHED, h->host.data(), h->len, h->width, s2, len2, width2,
                            to_sp(&h->params), rfg_cutoff{score_cutoff, 0.0, score_hint, 0.0}, RFG_I64, result, &done));
    if (done) return RFG_OK;
    int64_t off[2] = {0, len2};
    rfg_strings c{s2, off, 1, width2};
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    return cached_many(h, op, &c, rfg_cutoff{score_cutoff, 0.0, score_hint, 0.0}, RFG_I64, result, 0);
}

rfg_status rfg_cached_score_f64(rfg_cached h, rfg_op op, const void* s2, int64_t len2, int32_t width2,
                                double score_cutoff, double score_hint, double* result)
{
    if (!h) return fail(RFG_ERR_INVALID_ARGUMENT, "scorer is NULL");
    if (is_int_result(h->metric, op)) return fail(RFG_ERR_INVALID_ARGUMENT, "this metric/op returns an integer");
    if (!valid_width(width2) || len2 < 0 || (!s2 && len2) || !result) return fail(RFG_ERR_INVALID_ARGUMENT, "invalid s2");
    RFG_TRY(check_any_metric_op(h->metric, op, RFG_FORM_CACHED));
    RFG_TRY(ensure_ctx());
    int metric = h->metric;
    const void* t2 = s2;
    int64_t n2 = len2;
    std::vector<unsigned char> j2;
    if (is_token_set_metric(metric))
        return token_set_one(metric, op, RFG_FORM_CACHED, h->host.data(), h->len, h->width, s2, len2, width2,
                             &h->params, rfg_cutoff{0, score_cutoff, 0, score_hint}, RFG_F64, result);
    if (is_token_metric(metric)) { /* CachedTokenSortRatio / CachedPartialTokenSortRatio / CachedQRatio */
        if (metric == RFG_QRATIO && (!h->len || !len2)) {
            *result = 0.0;
            return RFG_OK;
        }
        if (metric != RFG_QRATIO) {
            n2 = token_sort_join(s2, len2, width2, &j2);
            t2 = j2.data();
        }
        metric = token_base(metric);
    }
    bool done = false;
    RFG_TRY(score_pair_trip(metric, op, RFG_FORM_CACHED, h->host.data(), h->len, h->width, t2, n2, width2,
                            to_sp(&h->params), rfg_cutoff{0, score_cutoff, 0, score_hint}, RFG_F64, result, &done));
    if (done) return RFG_OK;
    int64_t off[2] = {0, len2};
    rfg_strings c{s2, off, 1, width2};
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    return cached_many(h, op, &c, rfg_cutoff{0, score_cutoff, 0, score_hint}, RFG_F64, result, 0);
}

rfg_status rfg_cached_score_many(rfg_cached h, rfg_op op, const rfg_strings* choices, rfg_cutoff cutoff,
                                 rfg_dtype out_dtype, void* out, uint32_t flags)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    return cached_many(h, op, choices, cutoff, out_dtype, out, flags);
}

rfg_status rfg_cdist(rfg_metric metric, rfg_op op, rfg_form form, const rfg_strings* queries,
                     const rfg_strings* choices, const rfg_params* params, rfg_cutoff cutoff, rfg_dtype out_dtype,
                     void* out, int64_t ld, uint32_t flags)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    return cdist_impl(metric, op, form, queries, choices, params, cutoff, out_dtype, out, ld, flags);
}

/* ---------------------------------------------------------------- Multi* */

static size_t multi_vec_size(int max_len)
{
    /* AVX2 lanes of the reference build: 256 bits / lane width (Levenshtein.hpp:307-324) */
    return max_len <= 8 ? 32 : max_len <= 16 ? 16 : max_len <= 32 ? 8 : 4;
}

static size_t multi_result_count(const rfg_multi_s* h)
{
    const size_t v = multi_vec_size(h->max_len);
    return (h->count + v - 1) / v * v;
}

rfg_status rfg_multi_create(rfg_metric metric, int32_t max_len, size_t count, const rfg_params* params, rfg_multi* out)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!out) return fail(RFG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    const bool sim_only = metric == RFG_RATIO || is_token_metric(metric);
    RFG_TRY(check_any_metric_op(metric, sim_only ? RFG_SIMILARITY : RFG_DISTANCE, RFG_FORM_MULTI));
    if (max_len != 8 && max_len != 16 && max_len != 32 && max_len != 64)
        return fail(RFG_ERR_INVALID_ARGUMENT, "MaxLen must be 8, 16, 32 or 64");
    const ScoreParams sp = to_sp(params);
    /* MultiLevenshtein only supports insert = delete = 1, replace <= 2 (Levenshtein.hpp:338-339) */
    if (metric == RFG_LEVENSHTEIN && (sp.del != 1 || sp.ins != 1 || sp.rep > 2 || sp.rep < 0))
        return fail(RFG_ERR_INVALID_ARGUMENT, "unsupported weights");
    rfg_multi_s* h = new rfg_multi_s();
    h->metric = metric;
    h->max_len = max_len;
    h->count = count;
    h->params = rfg_params{sp.ins, sp.del, sp.rep, sp.prefix_weight};
    *out = h;
    return RFG_OK;
}

rfg_status rfg_multi_destroy(rfg_multi h)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    delete h;
    return RFG_OK;
}

rfg_status rfg_multi_insert(rfg_multi h, const void* s, int64_t len, int32_t width)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!h) return fail(RFG_ERR_INVALID_ARGUMENT, "scorer is NULL");
    if (!valid_width(width) || len < 0 || (!s && len)) return fail(RFG_ERR_INVALID_ARGUMENT, "invalid string");
    if (h->strs.size() >= h->count) return fail(RFG_ERR_INVALID_ARGUMENT, "out of bounds insert");
    std::vector<unsigned char> j;
    if (h->metric == RFG_TOKEN_SORT_RATIO) { /* MultiTokenSortRatio inserts the sorted-split join */
        len = token_sort_join(s, len, width, &j);
        s = j.data();
    }
    if (len > h->max_len) return fail(RFG_ERR_INVALID_ARGUMENT, "string longer than MaxLen");
    std::vector<u64> v(len);
    for (int64_t i = 0; i < len; ++i) v[i] = unit_at(s, width, i);
    h->strs.push_back(std::move(v));
    h->width = std::max(h->width, (int)width);
    return RFG_OK;
}

rfg_status rfg_multi_result_count(rfg_multi h, size_t* out)
{
    if (!h || !out) return fail(RFG_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = multi_result_count(h);
    return RFG_OK;
}

static rfg_status multi_score(rfg_multi h, int op, void* scores, size_t score_count, const void* s2, int64_t len2,
                              int32_t width2, rfg_cutoff cut, int dt)
{
    if (!h) return fail(RFG_ERR_INVALID_ARGUMENT, "scorer is NULL");
    RFG_TRY(check_any_metric_op(h->metric, op, RFG_FORM_MULTI));
    if (!valid_width(width2) || len2 < 0 || (!s2 && len2)) return fail(RFG_ERR_INVALID_ARGUMENT, "invalid s2");
    const size_t rc = multi_result_count(h);
    if (score_count < rc) return fail(RFG_ERR_INVALID_ARGUMENT, "scores has to have >= result_count() elements");
    if (!scores && rc) return fail(RFG_ERR_INVALID_ARGUMENT, "scores is NULL");
    if (h->metric == RFG_QRATIO && !len2) { /* MultiQRatio: the inserted strings score 0 (fuzz.hpp:752-767) */
        for (size_t i = 0; i < h->strs.size(); ++i) ((double*)scores)[i] = 0.0;
        return RFG_OK;
    }
    /* declared slots not inserted yet, and the padding up to result_count(), score as
     * empty strings */
    const int w = h->width;
    std::vector<int64_t> off(rc + 1, 0);
    for (size_t i = 0; i < rc; ++i) off[i + 1] = off[i] + (i < h->strs.size() ? (int64_t)h->strs[i].size() : 0);
    std::vector<unsigned char> data((size_t)off[rc] * w + 8);
    for (size_t i = 0; i < h->strs.size(); ++i)
        for (size_t k = 0; k < h->strs[i].size(); ++k) {
            const u64 v = h->strs[i][k];
            unsigned char* dst = data.data() + (size_t)(off[i] + k) * w;
            memcpy(dst, &v, w); /* little-endian: the low w bytes */
        }
    rfg_strings q{data.data(), off.data(), (int64_t)rc, w};
    int64_t o2[2] = {0, len2};
    rfg_strings c{s2, o2, 1, width2};
    return cdist_impl(h->metric, op, RFG_FORM_MULTI, &q, &c, &h->params, cut, dt, scores, 1, 0);
}

rfg_status rfg_multi_score_i64(rfg_multi h, rfg_op op, int64_t* scores, size_t score_count, const void* s2,
                               int64_t len2, int32_t width2, uint64_t score_cutoff)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (h && !is_int_result(h->metric, op)) return fail(RFG_ERR_INVALID_ARGUMENT, "this metric/op returns doubles");
    return multi_score(h, op, scores, score_count, s2, len2, width2, rfg_cutoff{score_cutoff, 0.0, 0, 0.0}, RFG_I64);
}

rfg_status rfg_multi_score_f64(rfg_multi h, rfg_op op, double* scores, size_t score_count, const void* s2,
                               int64_t len2, int32_t width2, double score_cutoff)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (h && is_int_result(h->metric, op)) return fail(RFG_ERR_INVALID_ARGUMENT, "this metric/op returns integers");
    return multi_score(h, op, scores, score_count, s2, len2, width2, rfg_cutoff{0, score_cutoff, 0, 0.0}, RFG_F64);
}

/* ----------------------------------------------------------------- extract */

} /* extern "C" */

namespace rfg {
/* Device buffers of one in-flight extract (freed on its stream once it is done). */
struct ExtractJob {
    Prepared pb;
    DBuf thr, ckey, cidx, oidx, oscore, ocount;
    int64_t nq = 0;
    int k = 0;
    void free_on(cudaStream_t st)
    {
        pb.free_on(st);
        thr.free_on = ckey.free_on = cidx.free_on = oidx.free_on = oscore.free_on = ocount.free_on = st;
    }
};

/* Enqueue extract/extractOne of the queries against a corpus on stream st: the tile
 * kernels keep each tile's best `k`, a merge kernel keeps each query's best `k`. */
rfg_status extract_enqueue(rfg_corpus c, const QuerySet& q, int metric, int op, const ScoreParams& sp,
                           rfg_cutoff cut, int k, int tie_last, cudaStream_t st, ExtractJob* job,
                           const int32_t* qparts = nullptr)
{
    const int64_t nq = q.dev.n;
    job->nq = nq;
    job->k = k;
    if (nq == 0) return RFG_OK;
    const int64_t nchunks = c->count ? (c->count + c->chunk - 1) / c->chunk : 0;
    RFG_TRY(job->oidx.alloc((size_t)nq * k * 8));
    RFG_TRY(job->oscore.alloc((size_t)nq * k * 8));
    RFG_TRY(job->ocount.alloc((size_t)nq * 4));
    RFG_CUDA(cudaMemsetAsync(job->oidx.p, 0xff, (size_t)nq * k * 8, g.stream));
    RFG_CUDA(cudaMemsetAsync(job->ocount.p, 0, (size_t)nq * 4, g.stream));
    if (nchunks == 0) return RFG_OK;
    RFG_TRY(job->thr.alloc((size_t)nq * 8));
    RFG_TRY(job->ckey.alloc((size_t)nq * nchunks * k * 8));
    RFG_TRY(job->cidx.alloc((size_t)nq * nchunks * k * 8));
    RFG_CUDA(cudaMemsetAsync(job->thr.p, 0, (size_t)nq * 8, g.stream));
    BatchSpec spec;
    spec.metric = metric;
    spec.op = op;
    spec.form = RFG_FORM_CACHED;
    spec.sp = sp;
    spec.ci = cut.cutoff_i;
    spec.cf = cut.cutoff_f;
    spec.out_dtype = RFG_F64;
    spec.out = nullptr;
    spec.ld = 0;
    spec.topk = k;
    spec.tie_last = tie_last;
    spec.thr = job->thr.as<u64>();
    spec.cand_key = job->ckey.as<u64>();
    spec.cand_idx = job->cidx.as<int64_t>();
    spec.fixed_perm = c->perm.as<int32_t>();
    spec.fixed_chunk = c->chunk;
    spec.chunk_lmin = c->lmin.as<int32_t>();
    spec.chunk_lmax = c->lmax.as<int32_t>();
    spec.fixed_maxlen = c->maxlen;
    if (qparts) { /* token scorers: the parts of the queries and of the corpus twin */
        spec.fixed_maxlen = c->tmaxlen;
        spec.qparts = qparts;
        spec.cparts = c->tparts.as<int32_t>();
    }
    RFG_TRY(prepare_batch(q, qparts ? c->tdev : c->dev, spec, &job->pb));
    if (st != g.stream) {
        /* uploads, resets and the tile lists were enqueued on the library stream */
        RFG_CUDA(cudaEventRecord(g.prep_ev, g.stream));
        RFG_CUDA(cudaStreamWaitEvent(st, g.prep_ev, 0));
    }
    RFG_TRY(enqueue_batch(job->pb, st));
    const int is_int = is_int_result(metric, op);
    const int bh = better_high_of(op);
    void* args[] = {&job->ckey.p, &job->cidx.p, (void*)&nchunks, &k, &tie_last, (void*)&bh, (void*)&is_int,
                    &job->oidx.p, &job->oscore.p, &job->ocount.p};
    RFG_CUDA(cudaLaunchKernel(topk_merge_kernel(), dim3((unsigned)nq), dim3(256), args, 0, st));
    job->free_on(st);
    return RFG_OK;
}
} // namespace rfg

namespace rfg {
/* the serving loop's view of extract (rfg_server.cu) */
struct ServerJob {
    ExtractJob ej;
    DBuf qd, qo;
    QuerySet qs;
};

int64_t corpus_chunks(rfg_corpus c) { return c->count ? (c->count + c->chunk - 1) / c->chunk : 0; }

rfg_status server_extract_enqueue(rfg_corpus c, const unsigned char* qdata, const int64_t* qoff, int64_t nq,
                                  int width, int metric, int op, const rfg_params* p, rfg_cutoff cut, int k,
                                  int tie_last, cudaStream_t st, void** job, int64_t* est_bytes)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    RFG_TRY(ensure_ctx());
    ServerJob* j = new ServerJob();
    *job = j;
    *est_bytes = 0;
    rfg_strings q{qdata, qoff, nq, width};
    RFG_TRY(query_info_from_host(qdata, qoff, nq, width, &j->qs));
    RFG_TRY(upload_strings(&q, &j->qd, &j->qo, &j->qs.dev));
    const ScoreParams sp = to_sp(p);
    RFG_TRY(check_params(metric, sp));
    RFG_TRY(extract_enqueue(c, j->qs, metric, op, sp, cut, k, tie_last, st, &j->ej));
    j->qd.free_on = j->qo.free_on = st;
    return RFG_OK;
}

rfg_status server_extract_results(void* job, int64_t* idx, double* score, int32_t* count, cudaStream_t st)
{
    ServerJob* j = (ServerJob*)job;
    const int64_t nq = j->ej.nq, k = j->ej.k;
    if (!nq) return RFG_OK;
    RFG_CUDA(cudaMemcpyAsync(idx, j->ej.oidx.p, (size_t)nq * k * 8, cudaMemcpyDeviceToHost, st));
    RFG_CUDA(cudaMemcpyAsync(score, j->ej.oscore.p, (size_t)nq * k * 8, cudaMemcpyDeviceToHost, st));
    RFG_CUDA(cudaMemcpyAsync(count, j->ej.ocount.p, (size_t)nq * 4, cudaMemcpyDeviceToHost, st));
    return RFG_OK;
}

void server_extract_free(void* job)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    delete (ServerJob*)job;
}

/* the two code-unit types of a pair set: f(TA(), TB()) */
template <typename F>
void with_unit_types(int wa, int wb, F f)
{
    auto second = [&](auto ta) {
        switch (wb) {
        case 1: f(ta, uint8_t()); break;
        case 2: f(ta, uint16_t()); break;
        case 4: f(ta, uint32_t()); break;
        default: f(ta, uint64_t()); break;
        }
    };
    switch (wa) {
    case 1: second(uint8_t()); break;
    case 2: second(uint16_t()); break;
    case 4: second(uint32_t()); break;
    default: second(uint64_t()); break;
    }
}

/* pairs [i0, i1): common prefix and suffix lengths, the Hirschberg-regime mark and the
 * sizes of each pair's matrix region (words) and operation slots */
template <typename TA, typename TB>
void editops_sizes(const TA* ad, const int64_t* ao, const TB* bd, const int64_t* bo, bool lev, bool one_byte,
                   int64_t i0, int64_t i1, int64_t* pre, int64_t* suf, int64_t* msize, int64_t* osize,
                   unsigned char* hb)
{
    for (int64_t i = i0; i < i1; ++i) {
        const int64_t la = ao[i + 1] - ao[i], lb = bo[i + 1] - bo[i];
        int64_t p = 0, q = 0;
        if (la && lb) {
            const TA* s1 = ad + ao[i];
            const TB* s2 = bd + bo[i];
            while (p < la && p < lb && (u64)s1[p] == (u64)s2[p]) ++p;
            while (q < la - p && q < lb - p && (u64)s1[la - 1 - q] == (u64)s2[lb - 1 - q]) ++q;
        }
        pre[i] = p;
        suf[i] = q;
        const int64_t m = la - p - q, n = lb - p - q, W = (m + 63) / 64;
        if (lev && m >= 65 && n >= 10 && 2 * (uint64_t)m * (uint64_t)n / 8 >= (1u << 20)) {
            /* the reference may split this pair with Hirschberg's algorithm: k_editops_hb's
             * pattern table, row vectors, band row offsets and band (a bound of every leaf's) */
            const int64_t Wa = std::max<int64_t>(1, (la + 63) / 64);
            hb[i] = 1;
            msize[i] = (one_byte ? 256 * Wa : 0) + 4 * Wa + (lb + 1) + (1 << 17) + 5 * lb + 20 * Wa + 64;
        }
        else msize[i] = m && n ? (lev ? 2 : 1) * W * n : 0;
        osize[i] = lev ? std::max(m, n) : m + n;
    }
}

} // namespace rfg

extern "C" {

rfg_status rfg_corpus_create(const rfg_strings* C, uint32_t flags, rfg_corpus* out)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!out) return fail(RFG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    RFG_TRY(check_strings(C, "choices"));
    if (!(flags & RFG_DEVICE_INPUTS)) RFG_TRY(check_offsets(C->offsets, C->count, "choices"));
    RFG_TRY(ensure_ctx());
    rfg_corpus c = new rfg_corpus_s();
    const int64_t nc = C->count;
    rfg_status st = RFG_OK;
    std::vector<int64_t> hoff;
    const int64_t* off = C->offsets;
    if (flags & RFG_DEVICE_INPUTS) {
        hoff.resize(nc + 1);
        if (cudaMemcpy(hoff.data(), C->offsets, (nc + 1) * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = fail(RFG_ERR_CUDA, "reading choice offsets failed");
        off = hoff.data();
        if (st == RFG_OK) st = check_offsets(off, nc, "choices");
        /* the corpus keeps its own copy: callers may free theirs */
        if (st == RFG_OK) st = c->data.alloc((size_t)off[nc] * C->char_width + 16);
        if (st == RFG_OK) st = c->off.alloc((size_t)(nc + 1) * 8);
        if (st == RFG_OK && off[nc])
            if (cudaMemcpyAsync(c->data.p, C->data, (size_t)off[nc] * C->char_width, cudaMemcpyDeviceToDevice,
                                g.stream) != cudaSuccess)
                st = fail(RFG_ERR_CUDA, "copying the corpus failed");
        if (st == RFG_OK &&
            cudaMemcpyAsync(c->off.p, C->offsets, (nc + 1) * 8, cudaMemcpyDeviceToDevice, g.stream) != cudaSuccess)
            st = fail(RFG_ERR_CUDA, "copying the corpus failed");
        c->dev = KStrings{c->data.as<unsigned char>(), c->off.as<int64_t>(), nc, C->char_width};
    }
    else {
        for (int64_t i = 0; i < nc && st == RFG_OK; ++i)
            if (off[i] < 0 || off[i + 1] < off[i]) st = fail(RFG_ERR_INVALID_ARGUMENT, "offsets must be non-decreasing");
        if (st == RFG_OK) st = upload_strings(C, &c->data, &c->off, &c->dev);
    }
    c->count = nc;
    c->chunk = 4096;
    if (st == RFG_OK && nc) {
        /* one global length order: chunks then hold narrow length ranges that extract
         * tiles can test against the running threshold */
        std::vector<int32_t> len(nc), perm;
        for (int64_t i = 0; i < nc; ++i) {
            len[i] = (int32_t)std::min<int64_t>(off[i + 1] - off[i], INT32_MAX);
            c->maxlen = std::max<int64_t>(c->maxlen, len[i]);
        }
        chunk_length_order(len, nc, &perm);
        const int64_t nch = (nc + c->chunk - 1) / c->chunk;
        std::vector<int32_t> lmin(nch), lmax(nch);
        for (int64_t k = 0; k < nch; ++k) {
            lmin[k] = len[perm[k * c->chunk]];
            lmax[k] = len[perm[std::min(nc, (k + 1) * c->chunk) - 1]];
        }
        st = c->perm.alloc((size_t)nc * 4);
        if (st == RFG_OK) st = c->lmin.alloc((size_t)nch * 4);
        if (st == RFG_OK) st = c->lmax.alloc((size_t)nch * 4);
        if (st == RFG_OK &&
            (cudaMemcpyAsync(c->perm.p, perm.data(), (size_t)nc * 4, cudaMemcpyHostToDevice, g.stream) != cudaSuccess ||
             cudaMemcpyAsync(c->lmin.p, lmin.data(), (size_t)nch * 4, cudaMemcpyHostToDevice, g.stream) != cudaSuccess ||
             cudaMemcpyAsync(c->lmax.p, lmax.data(), (size_t)nch * 4, cudaMemcpyHostToDevice, g.stream) != cudaSuccess))
            st = fail(RFG_ERR_CUDA, "uploading the corpus order failed");
        if (st == RFG_OK && cudaStreamSynchronize(g.stream) != cudaSuccess) st = fail(RFG_ERR_CUDA, "corpus upload failed");
    }
    if (st != RFG_OK) {
        delete c;
        return st;
    }
    *out = c;
    return RFG_OK;
}

rfg_status rfg_corpus_destroy(rfg_corpus c)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (c) cudaDeviceSynchronize();
    delete c;
    return RFG_OK;
}

/* the corpus's token twin (rfg_corpus_s::tok) */
static rfg_status corpus_token_twin(rfg_corpus c)
{
    if (c->tok) return RFG_OK;
    HostStrings h;
    const rfg_strings dv{c->dev.data, c->dev.off, c->count, c->dev.width};
    RFG_TRY(download_strings(&dv, &h, "corpus"));
    std::vector<unsigned char> td;
    std::vector<int64_t> to;
    std::vector<int32_t> tp;
    token_parts_set(h.data.data(), h.off.data(), c->count, c->dev.width, true, true, true, &td, &to, &tp);
    const rfg_strings tv{td.data(), to.data(), c->count, c->dev.width};
    RFG_TRY(upload_strings(&tv, &c->tdata, &c->toff, &c->tdev));
    RFG_TRY(c->tparts.alloc(tp.size() * 4));
    if (!tp.empty()) RFG_CUDA(cudaMemcpyAsync(c->tparts.p, tp.data(), tp.size() * 4, cudaMemcpyHostToDevice, g.stream));
    RFG_CUDA(cudaStreamSynchronize(g.stream));
    c->tmaxlen = 0;
    for (int64_t i = 0; i < c->count; ++i) c->tmaxlen = std::max<int64_t>(c->tmaxlen, to[i + 1] - to[i]);
    c->tok = true;
    return RFG_OK;
}

rfg_status rfg_extract(rfg_corpus c, rfg_metric metric, rfg_op op, const rfg_strings* Q, const rfg_params* p,
                       rfg_cutoff cut, int32_t limit, int32_t tie_last_wins, int64_t* out_index, double* out_score,
                       int32_t* out_count, uint32_t flags)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!c) return fail(RFG_ERR_INVALID_ARGUMENT, "corpus is NULL");
    const bool tok = is_token_metric(metric);
    RFG_TRY(tok ? check_any_metric_op(metric, op, RFG_FORM_CACHED) : check_metric_op(metric, op, RFG_FORM_CACHED));
    RFG_TRY(check_strings(Q, "queries"));
    if (limit < 1 || limit > RFG_MAX_TOPK) return fail(RFG_ERR_INVALID_ARGUMENT, "limit must be in [1, 32]");
    if (!out_index || !out_score || !out_count) return fail(RFG_ERR_INVALID_ARGUMENT, "NULL output");
    const ScoreParams sp = to_sp(p);
    RFG_TRY(check_params(metric, sp));
    RFG_TRY(ensure_ctx());
    QuerySet qs;
    DBuf qd, qo, qp;
    const int64_t nq = Q->count;
    if (tok) { /* the queries' parts on the host, then the corpus twin */
        HostStrings hq, jq;
        rfg_strings q = *Q;
        if (flags & RFG_DEVICE_INPUTS) {
            RFG_TRY(download_strings(Q, &hq, "queries"));
            q.data = hq.data.data();
            q.offsets = hq.off.data();
        }
        RFG_TRY(check_offsets(q.offsets, nq, "queries"));
        if (!q.data && nq && q.offsets[nq] > q.offsets[0]) return fail(RFG_ERR_INVALID_ARGUMENT, "string data is NULL");
        std::vector<int32_t> parts;
        token_parts_set(q.data, q.offsets, nq, q.char_width, true, true, true, &jq.data, &jq.off, &parts);
        const rfg_strings qt{jq.data.data(), jq.off.data(), nq, q.char_width};
        RFG_TRY(query_info_from_host(qt.data, qt.offsets, nq, qt.char_width, &qs));
        RFG_TRY(upload_strings(&qt, &qd, &qo, &qs.dev));
        RFG_TRY(qp.alloc(parts.size() * 4));
        if (!parts.empty())
            RFG_CUDA(cudaMemcpyAsync(qp.p, parts.data(), parts.size() * 4, cudaMemcpyHostToDevice, g.stream));
        RFG_TRY(corpus_token_twin(c));
    }
    else if (flags & RFG_DEVICE_INPUTS) {
        std::vector<int64_t> off(nq + 1);
        RFG_CUDA(cudaMemcpy(off.data(), Q->offsets, (nq + 1) * 8, cudaMemcpyDeviceToHost));
        std::vector<unsigned char> qh;
        if (Q->char_width > 1 && nq) {
            qh.resize((size_t)off[nq] * Q->char_width);
            RFG_CUDA(cudaMemcpy(qh.data(), Q->data, qh.size(), cudaMemcpyDeviceToHost));
        }
        RFG_TRY(query_info_from_host(qh.data(), off.data(), nq, Q->char_width, &qs));
        qs.dev = KStrings{(const unsigned char*)Q->data, Q->offsets, nq, Q->char_width};
    }
    else {
        RFG_TRY(query_info_from_host(Q->data, Q->offsets, nq, Q->char_width, &qs));
        RFG_TRY(upload_strings(Q, &qd, &qo, &qs.dev));
    }
    ExtractJob job;
    RFG_TRY(extract_enqueue(c, qs, metric, op, sp, cut, limit, tie_last_wins ? 1 : 0, g.stream, &job,
                            tok ? qp.as<int32_t>() : nullptr));
    job.free_on(nullptr);
    if (nq) {
        const cudaMemcpyKind kind = (flags & RFG_DEVICE_OUTPUT) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        RFG_CUDA(cudaMemcpyAsync(out_index, job.oidx.p, (size_t)nq * limit * 8, kind, g.stream));
        RFG_CUDA(cudaMemcpyAsync(out_score, job.oscore.p, (size_t)nq * limit * 8, kind, g.stream));
        RFG_CUDA(cudaMemcpyAsync(out_count, job.ocount.p, (size_t)nq * 4, kind, g.stream));
    }
    return check_batch(job.pb, g.stream);
}

/* ----------------------------------------------------------------- editops */

rfg_status rfg_editops(rfg_metric metric, const rfg_strings* S1, const rfg_strings* S2, uint64_t score_hint,
                       rfg_editop* ops, int64_t capacity, int64_t* offsets, uint32_t flags)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (metric != RFG_LEVENSHTEIN && metric != RFG_INDEL && metric != RFG_LCSSEQ)
        return fail(RFG_ERR_INVALID_ARGUMENT, "editops exist for Levenshtein, Indel and LCSseq");
    RFG_TRY(check_strings(S1, "s1"));
    RFG_TRY(check_strings(S2, "s2"));
    if (S1->count != S2->count) return fail(RFG_ERR_INVALID_ARGUMENT, "s1 and s2 must hold the same number of strings");
    if (!offsets) return fail(RFG_ERR_INVALID_ARGUMENT, "offsets is NULL");
    if (capacity < 0 || (!ops && capacity)) return fail(RFG_ERR_INVALID_ARGUMENT, "invalid ops buffer");
    RFG_TRY(ensure_ctx());
    const int64_t np = S1->count;
    HostStrings h1, h2;
    rfg_strings a = *S1, b = *S2;
    if (flags & RFG_DEVICE_INPUTS) {
        RFG_TRY(download_strings(S1, &h1, "s1"));
        RFG_TRY(download_strings(S2, &h2, "s2"));
        a.data = h1.data.data();
        a.offsets = h1.off.data();
        b.data = h2.data.data();
        b.offsets = h2.off.data();
    }
    RFG_TRY(check_offsets(a.offsets, np, "s1"));
    RFG_TRY(check_offsets(b.offsets, np, "s2"));
    if ((!a.data && np && a.offsets[np] > a.offsets[0]) || (!b.data && np && b.offsets[np] > b.offsets[0]))
        return fail(RFG_ERR_INVALID_ARGUMENT, "string data is NULL");
    const bool lev = metric == RFG_LEVENSHTEIN;
    /* common affixes (remove_common_affix, common_impl.hpp:46-81) and region sizes, over
     * the host threads; the sizes become offsets afterwards */
    std::vector<int64_t> pre(np), suf(np), moff(np + 1, 0), ooff(np + 1, 0);
    std::vector<unsigned char> hb(np, 0);
    const bool one_byte = a.char_width == 1 && b.char_width == 1;
    const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
    const int64_t nt = std::min<int64_t>({hw, 16, std::max<int64_t>(1, np / 16384)});
    auto range = [&](int64_t t) {
        with_unit_types(a.char_width, b.char_width, [&](auto ta, auto tb) {
            editops_sizes((const decltype(ta)*)a.data, a.offsets, (const decltype(tb)*)b.data, b.offsets, lev,
                          one_byte, np * t / nt, np * (t + 1) / nt, pre.data(), suf.data(), moff.data() + 1,
                          ooff.data() + 1, hb.data());
        });
    };
    if (nt == 1) range(0);
    else {
        std::vector<std::thread> th;
        for (int64_t t = 1; t < nt; ++t) th.emplace_back(range, t);
        range(0);
        for (auto& x : th) x.join();
    }
    for (int64_t i = 0; i < np; ++i) {
        moff[i + 1] += moff[i];
        ooff[i + 1] += ooff[i];
    }
    const bool any_hb = np && memchr(hb.data(), 1, (size_t)np) != nullptr;
    if (np == 0) {
        offsets[0] = 0;
        return RFG_OK;
    }
    DBuf da, dao, db, dbo, dpre, dsuf, dmo, doo, dcount, dops, derr, dhb;
    KStrings ka, kb;
    RFG_TRY(upload_strings(&a, &da, &dao, &ka));
    RFG_TRY(upload_strings(&b, &db, &dbo, &kb));
    RFG_TRY(dpre.alloc(np * 8));
    RFG_TRY(dsuf.alloc(np * 8));
    RFG_TRY(dmo.alloc((np + 1) * 8));
    RFG_TRY(doo.alloc((np + 1) * 8));
    RFG_TRY(dcount.alloc(np * 8));
    RFG_TRY(dops.alloc((size_t)ooff[np] * sizeof(rfg_editop)));
    RFG_TRY(derr.alloc(sizeof(int)));
    RFG_CUDA(cudaMemsetAsync(derr.p, 0, sizeof(int), g.stream));
    static_assert(sizeof(EditopDev) == sizeof(rfg_editop), "editop layouts");
    RFG_CUDA(cudaMemcpyAsync(dpre.p, pre.data(), np * 8, cudaMemcpyHostToDevice, g.stream));
    RFG_CUDA(cudaMemcpyAsync(dsuf.p, suf.data(), np * 8, cudaMemcpyHostToDevice, g.stream));
    RFG_CUDA(cudaMemcpyAsync(doo.p, ooff.data(), (np + 1) * 8, cudaMemcpyHostToDevice, g.stream));
    if (any_hb) {
        RFG_TRY(dhb.alloc(np));
        RFG_CUDA(cudaMemcpyAsync(dhb.p, hb.data(), np, cudaMemcpyHostToDevice, g.stream));
    }
    /* launches of pairs whose matrices fit 256M words of scratch together */
    const int64_t budget = (int64_t)1 << 28;
    int64_t maxw = 0;
    for (int64_t i = 0; i < np; ++i) maxw = std::max(maxw, moff[i + 1] - moff[i]);
    DBuf dmat;
    RFG_TRY(dmat.alloc((size_t)std::max(maxw, std::min(budget, moff[np])) * 8 + 8));
    std::vector<int64_t> lmo(np + 1);
    for (int64_t p0 = 0; p0 < np;) {
        int64_t p1 = p0 + 1;
        while (p1 < np && moff[p1 + 1] - moff[p0] <= std::max(budget, maxw)) ++p1;
        for (int64_t i = p0; i <= p1; ++i) lmo[i] = moff[i] - moff[p0]; /* offsets within this launch */
        RFG_CUDA(cudaMemcpyAsync(dmo.as<int64_t>() + p0, lmo.data() + p0, (p1 - p0 + 1) * 8, cudaMemcpyHostToDevice,
                                 g.stream));
        EditopsParams prm{ka,           kb,          dpre.as<int64_t>(),     dsuf.as<int64_t>(),  dmo.as<int64_t>(),
                          doo.as<int64_t>(), dmat.as<u64>(), dops.as<EditopDev>(), dcount.as<int64_t>(), derr.as<int>(),
                          p0,           p1 - p0,     lev ? 1 : 0,          any_hb ? dhb.as<unsigned char>() : nullptr,
                          score_hint};
        void* args[] = {&prm};
        RFG_CUDA(cudaLaunchKernel(editops_kernel(), dim3((unsigned)((p1 - p0 + 127) / 128)), dim3(128), args, 0,
                                  g.stream));
        if (any_hb)
            RFG_CUDA(cudaLaunchKernel(editops_hb_kernel(), dim3((unsigned)((p1 - p0 + 63) / 64)), dim3(64), args, 0,
                                      g.stream));
        RFG_CUDA(cudaStreamSynchronize(g.stream)); /* the scratch is reused by the next launch */
        p0 = p1;
    }
    std::vector<int64_t> cnt(np);
    int h_err = 0;
    RFG_CUDA(cudaMemcpyAsync(cnt.data(), dcount.p, np * 8, cudaMemcpyDeviceToHost, g.stream));
    RFG_CUDA(cudaMemcpyAsync(&h_err, derr.p, sizeof(int), cudaMemcpyDeviceToHost, g.stream));
    RFG_CUDA(cudaStreamSynchronize(g.stream));
    if (h_err) return fail(RFG_ERR_DEVICE_CHECK, "device-side check failed (code %d)", h_err);
    offsets[0] = 0;
    for (int64_t i = 0; i < np; ++i) offsets[i + 1] = offsets[i] + cnt[i];
    if (offsets[np] > capacity)
        return fail(RFG_ERR_OUT_OF_RANGE, "the editops need %lld slots, capacity is %lld", (long long)offsets[np],
                    (long long)capacity);
    if (offsets[np] == 0) return RFG_OK;
    /* pack on the device, then one copy of exactly the operations */
    DBuf doff, dpacked;
    RFG_TRY(doff.alloc((np + 1) * 8));
    RFG_TRY(dpacked.alloc((size_t)offsets[np] * sizeof(rfg_editop)));
    RFG_CUDA(cudaMemcpyAsync(doff.p, offsets, (np + 1) * 8, cudaMemcpyHostToDevice, g.stream));
    const EditopDev* src = dops.as<EditopDev>();
    const int64_t* po = doo.as<int64_t>();
    const int64_t* pf = doff.as<int64_t>();
    EditopDev* dst = dpacked.as<EditopDev>();
    void* pargs[] = {(void*)&src, (void*)&po, (void*)&pf, (void*)&dst, (void*)&np};
    RFG_CUDA(cudaLaunchKernel(editops_pack_kernel(), dim3((unsigned)((np + 127) / 128)), dim3(128), pargs, 0,
                              g.stream));
    RFG_CUDA(cudaMemcpyAsync(ops, dpacked.p, (size_t)offsets[np] * sizeof(rfg_editop), cudaMemcpyDeviceToHost,
                             g.stream));
    RFG_CUDA(cudaStreamSynchronize(g.stream));
    return RFG_OK;
}

/* --------------------------------------------------------- prepared batches */

/* the launch-shape knobs of a preparation (what rfg_batch_tune chooses) */
struct TuneChoice {
    int block = 0;        /* tile kernels' block size (0: default) */
    int64_t tiles = 0;    /* tile-count target (0: default) */
    int stage = 1;        /* dense tiles stage results in shared memory */
    int64_t window = 512; /* warp tiles: choice positions per window */
    int band = 1;         /* band classes on (k_band) or off (the general kernels) */
    int rounds = 0;       /* band units: 32 x rounds pairs (0: sized by the class) */
};

static rfg_status batch_reprepare(rfg_batch b, const TuneChoice& c)
{
    const int ob = g_block_override, os = g_stage_mode, obd = g_band_mode, orr = g_band_rounds;
    const int64_t ot = g_tiles_target, ow = g_fast_window;
    g_band_rounds = c.rounds;
    g_block_override = c.block;
    g_tiles_target = c.tiles;
    g_stage_mode = c.stage;
    g_fast_window = c.window;
    g_band_mode = c.band;
    Prepared* np = new Prepared();
    rfg_status st = prepare_batch(b->qs, b->ck, b->spec, np);
    g_block_override = ob;
    g_tiles_target = ot;
    g_stage_mode = os;
    g_fast_window = ow;
    g_band_mode = obd;
    g_band_rounds = orr;
    if (st == RFG_OK && cudaStreamSynchronize(g.stream) != cudaSuccess) st = fail(RFG_ERR_CUDA, "prepare failed");
    if (st != RFG_OK) {
        delete np;
        return st;
    }
    delete b->pb;
    b->pb = np;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->block = c.block;
    b->tiles = c.tiles;
    return RFG_OK;
}

static rfg_status batch_reprepare_shape(rfg_batch b, int block, int64_t tiles, int stage = 1)
{
    TuneChoice c;
    c.block = block;
    c.tiles = tiles;
    c.stage = stage;
    c.window = g_fast_window;
    c.band = g_band_mode;
    c.rounds = g_band_rounds;
    return batch_reprepare(b, c);
}

rfg_status rfg_batch_create(rfg_metric metric, rfg_op op, rfg_form form, const rfg_strings* Q, const rfg_strings* C,
                            const rfg_params* p, rfg_cutoff cut, rfg_dtype dt, void* out, int64_t ld, uint32_t flags,
                            rfg_batch* outb)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!outb) return fail(RFG_ERR_INVALID_ARGUMENT, "batch is NULL");
    *outb = nullptr;
    RFG_TRY(check_metric_op(metric, op, form));
    RFG_TRY(check_strings(Q, "queries"));
    RFG_TRY(check_strings(C, "choices"));
    RFG_TRY(check_dtype(metric, op, dt));
    const ScoreParams sp = to_sp(p);
    RFG_TRY(check_params(metric, sp));
    if (!out) return fail(RFG_ERR_INVALID_ARGUMENT, "out (device memory) is NULL");
    const int64_t nq = Q->count, nc = C->count;
    if (ld == 0) ld = nc;
    if (ld < nc) return fail(RFG_ERR_INVALID_ARGUMENT, "ld must be >= the number of choices");
    if (!(flags & RFG_DEVICE_INPUTS)) { /* host offsets are checked before the device is touched */
        RFG_TRY(check_offsets(Q->offsets, nq, "queries"));
        RFG_TRY(check_offsets(C->offsets, nc, "choices"));
    }
    RFG_TRY(ensure_ctx());
    rfg_batch b = new rfg_batch_s();
    rfg_status st = RFG_OK;
    if (flags & RFG_DEVICE_INPUTS) {
        std::vector<int64_t> off(nq + 1);
        std::vector<unsigned char> qh;
        if (cudaMemcpy(off.data(), Q->offsets, (nq + 1) * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = fail(RFG_ERR_CUDA, "reading query offsets failed");
        if (st == RFG_OK) st = check_offsets(off.data(), nq, "queries"); /* before anything is read through them */
        const bool want = band_candidate(metric) && st == RFG_OK && has_long_query(off.data(), nq);
        if (st == RFG_OK && (Q->char_width > 1 || want) && nq && off[nq] > off[0]) {
            qh.resize((size_t)off[nq] * Q->char_width);
            if (cudaMemcpy(qh.data(), Q->data, qh.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
                st = fail(RFG_ERR_CUDA, "reading queries failed");
        }
        if (st == RFG_OK) st = query_info_from_host(qh.data(), off.data(), nq, Q->char_width, &b->qs, want);
        b->qs.dev = KStrings{(const unsigned char*)Q->data, Q->offsets, nq, Q->char_width};
        b->ck = KStrings{(const unsigned char*)C->data, C->offsets, nc, C->char_width};
    }
    else {
        st = query_info_from_host(Q->data, Q->offsets, nq, Q->char_width, &b->qs, band_candidate(metric));
        if (st == RFG_OK) st = upload_strings(Q, &b->qd, &b->qo, &b->qs.dev);
        if (st == RFG_OK) st = upload_strings(C, &b->cd, &b->co, &b->ck);
    }
    b->spec.metric = metric;
    b->spec.op = op;
    b->spec.form = form;
    b->spec.sp = sp;
    b->spec.ci = cut.cutoff_i;
    b->spec.cf = cut.cutoff_f;
    b->spec.out_dtype = dt;
    b->spec.out = out;
    b->spec.ld = ld;
    if (st == RFG_OK) st = batch_reprepare_shape(b, 0, 0);
    if (st != RFG_OK) {
        delete b;
        return st;
    }
    *outb = b;
    return RFG_OK;
}

rfg_status rfg_batch_launch(rfg_batch b, void* stream, uint32_t launch_flags)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!b) return fail(RFG_ERR_INVALID_ARGUMENT, "batch is NULL");
    cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
    if (!(launch_flags & RFG_LAUNCH_GRAPH)) return enqueue_batch(*b->pb, st);
    if (!b->graph) {
        cudaGraph_t graph;
        RFG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        rfg_status s = enqueue_batch(*b->pb, st);
        cudaError_t e = cudaStreamEndCapture(st, &graph);
        if (s != RFG_OK) return s;
        if (e != cudaSuccess) return fail(RFG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            b->graph = nullptr;
            return fail(RFG_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
        }
    }
    RFG_CUDA(cudaGraphLaunch(b->graph, st));
    return RFG_OK;
}

rfg_status rfg_batch_check(rfg_batch b, void* stream)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!b) return fail(RFG_ERR_INVALID_ARGUMENT, "batch is NULL");
    return check_batch(*b->pb, stream ? (cudaStream_t)stream : g.stream);
}

/* tuned shapes, kept per (metric, op, form, output type, code-unit widths, and power-of-two
 * buckets of the longest query, the query count and the choice count): a later batch of
 * the same kind takes the stored choice without sweeping */
typedef std::tuple<int, int, int, int, int, int, int, int, int> TuneKey;
std::map<TuneKey, TuneChoice> g_tune_cache;

static int log2_bucket(int64_t x)
{
    int b = 0;
    while (x > 1) {
        x >>= 1;
        ++b;
    }
    return b;
}

rfg_status rfg_batch_tune(rfg_batch b, void* stream, int32_t* best_block, int64_t* best_tiles)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!b) return fail(RFG_ERR_INVALID_ARGUMENT, "batch is NULL");
    cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
    int64_t maxq = 0;
    for (int64_t l : b->qs.len) maxq = std::max(maxq, l);
    const TuneKey key{b->spec.metric, b->spec.op, b->spec.form, b->spec.out_dtype, b->qs.dev.width, b->ck.width,
                      log2_bucket(maxq), log2_bucket(b->qs.dev.n), log2_bucket(b->ck.n)};
    auto hit = g_tune_cache.find(key);
    if (hit != g_tune_cache.end()) {
        RFG_TRY(batch_reprepare(b, hit->second));
        RFG_TRY(check_batch(*b->pb, st));
        if (best_block) *best_block = hit->second.block;
        if (best_tiles) *best_tiles = hit->second.tiles;
        return RFG_OK;
    }
    cudaEvent_t e0, e1;
    RFG_CUDA(cudaEventCreate(&e0));
    RFG_CUDA(cudaEventCreate(&e1));
    float best_t = 1e30f;
    TuneChoice best;
    best.window = g_fast_window;
    best.band = g_band_mode;
    auto trial = [&](const TuneChoice& c) -> rfg_status {
        RFG_TRY(batch_reprepare(b, c));
        float times[3];
        for (int r = 0; r < 3; ++r) {
            RFG_CUDA(cudaEventRecord(e0, st));
            RFG_TRY(enqueue_batch(*b->pb, st));
            RFG_CUDA(cudaEventRecord(e1, st));
            RFG_CUDA(cudaEventSynchronize(e1));
            RFG_CUDA(cudaEventElapsedTime(&times[r], e0, e1));
        }
        std::sort(times, times + 3);
        if (times[1] < best_t) {
            best_t = times[1];
            best = c;
        }
        return RFG_OK;
    };
    /* the default shape first; then the knobs of the launch kinds the batch holds, one
     * at a time from the best so far: the band classes on or off (words per thread sized
     * by the band, or by the pattern), the warp tiles' window, and the tile kernels'
     * block size, tile count and staging */
    RFG_TRY(trial(best));
    const bool fast = b->pb->has_fast, band = b->pb->has_band;
    if (band) {
        TuneChoice c = best;
        c.band = 0;
        RFG_TRY(trial(c));
    }
    if (fast)
        for (int64_t w : {256, 1024, 2048}) {
            TuneChoice c = best;
            c.window = w;
            RFG_TRY(trial(c));
        }
    RFG_TRY(batch_reprepare(b, best));
    if (b->pb->has_tiles) {
        const TuneChoice base = best;
        const int blocks[] = {128, 256};
        const int mults[] = {2, 4, 8, 16, 32};
        for (int stage = 1; stage >= 0; --stage)
            for (int blk : blocks)
                for (int mu : mults) {
                    TuneChoice c = base;
                    c.block = blk;
                    c.tiles = (int64_t)g.sms * mu * (256 / blk) * 2;
                    c.stage = stage;
                    RFG_TRY(trial(c));
                }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    RFG_TRY(batch_reprepare(b, best));
    RFG_TRY(check_batch(*b->pb, st));
    g_tune_cache[key] = best;
    if (best_block) *best_block = best.block;
    if (best_tiles) *best_tiles = best.tiles;
    return RFG_OK;
}

rfg_status rfg_batch_destroy(rfg_batch b)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!b) return RFG_OK;
    cudaDeviceSynchronize();
    delete b;
    return RFG_OK;
}

rfg_status rfg_batch_kernels(rfg_batch b, char* names, size_t cap)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!b || !names || cap == 0) return fail(RFG_ERR_INVALID_ARGUMENT, "batch or buffer is NULL");
    std::string all;
    auto add = [&](const void* fn) {
        const char* nm = nullptr;
        if (cudaFuncGetName(&nm, fn) != cudaSuccess || !nm) nm = "?";
        if (!all.empty()) all += ';';
        all += nm;
    };
    if (b->pb->has_pre) add(jaro_tables_kernel());
    if (b->pb->has_hist) add(fast_hist_kernel());
    for (const LaunchRec& L : b->pb->launches) add(L.fn);
    if (all.size() + 1 > cap) return fail(RFG_ERR_INVALID_ARGUMENT, "buffer too small (%zu bytes needed)", all.size() + 1);
    memcpy(names, all.c_str(), all.size() + 1);
    return RFG_OK;
}

rfg_status rfg_get_stream(void** stream)
{
    std::lock_guard<std::recursive_mutex> lk(g.mu);
    if (!stream) return fail(RFG_ERR_INVALID_ARGUMENT, "stream is NULL");
    RFG_TRY(ensure_ctx());
    *stream = (void*)g.stream;
    return RFG_OK;
}

} /* extern "C" */
