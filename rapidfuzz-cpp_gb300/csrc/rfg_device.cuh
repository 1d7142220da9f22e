/*
 * rfg_device.cuh -- the scoring kernels: one persistent CTA per SM slot pulls
 * (query, choice-chunk) tiles from an atomic work counter, builds the query's
 * pattern-match table in shared memory and scores the chunk one pair per thread.
 *
 * Shared-memory pattern table (the device form of BlockPatternMatchVector,
 * rapidfuzz/details/PatternMatchVector.hpp:136-221): `rows` holds W words per row;
 * rows 0..255 are code units below 256, rows 256..256+hcap-1 the slots of an
 * open-addressing table for wider code units (keys in `keys`, 0 = empty, so the
 * reference's CPython-style 128-slot map becomes a linear-probing table sized by the
 * host to twice the query's wide code units), and the last row is all zero (code
 * units the query does not contain).  Text characters are resolved to a row index
 * once; the cores then read `rows[r * W + w]`.
 */
#pragma once
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>

#include "rfg_core.cuh"

namespace rfg {

struct KStrings {
    const unsigned char* data; /* packed code units */
    const int64_t* off;        /* count+1 offsets in code units */
    int64_t n;
    int width;
};

/* one query of a band launch: its first work unit, its passing choices [plo, phi) in
 * the length order of the choices (the lengths [nlo, nhi]), its index; the record after
 * a launch's last query holds the launch's unit count in ustart */
struct BandQuery {
    int32_t ustart, plo, phi, nlo, nhi, qi, pad0, pad1;
};

struct KParams {
    KStrings q, c;
    const int32_t* qlist; /* queries of this launch (size class), longest first */
    int32_t nq;
    int64_t chunk;   /* choices per tile */
    int64_t nchunks;
    int* counter;    /* tile counter, zero before the launch */
    int* err;        /* device-side check flag */
    int metric, op, form;
    ScoreParams sp;
    u64 ci;
    double cf;
    /* the caller's score_hint (has_hint: given; the integer ops read hint_i, the
     * normalized ones hint_f): the first band of the score-hint doubling */
    u64 hint_i;
    double hint_f;
    int has_hint;
    void* out;
    int out_dtype; /* 0 i32, 1 i64, 2 f64 */
    int64_t ld;
    int hcap;      /* hash slots for code units >= 256 (power of two, or 0) */
    int tab_t;     /* per-query length tables cover text lengths 0..tab_t (<= RFG_JT_MAXT) */
    const int32_t* perm; /* choice order within each chunk (length-sorted), or nullptr */
    /* extract epilogue (topk > 0): instead of a dense matrix, every (query, chunk) tile
     * keeps its best topk results in cand_key/cand_idx[(q * nchunks + chunk) * topk + r];
     * keys order results best-first: the score's bits for similarity ops, their
     * complement for distance ops.  thr[q] is the running threshold key of query q
     * (raised by every tile that fills its topk), used to tighten the cutoff. */
    int topk;
    /* corpus with a global length order: per-chunk length range; extract tiles then visit
     * each query's chunks from its own length outwards and skip chunks whose lengths all
     * fail the running threshold */
    const int32_t* chunk_lmin;
    const int32_t* chunk_lmax;
    int tie_last;    /* equal scores: the later choice wins (extractOne) instead of the earlier */
    int better_high; /* 1: larger scores are better (similarity ops) */
    u64* thr;
    u64* cand_key;
    int64_t* cand_idx;
    /* generic (scratch) kernels */
    u64* scratch;
    int64_t scratch_per_cta;    /* u64 words of the per-CTA pattern table region */
    int64_t scratch_per_thread; /* u64 words of each thread's state */
    int wmax;                   /* pattern words of the generic class */
    int pm_smem;                /* 1: the generic pattern table lives in dynamic shared memory */
    /* dense tiles: results of each window of `stage` choice positions (one length-sorted
     * run of the permutation) gather in shared memory and leave as coalesced row
     * segments; 0 = store each result where it belongs */
    int64_t stage;
    /* 1: distance with unit weights (Levenshtein 1/1/1, Indel, OSA; free or cached form):
     * the whole chain is d <= K ? d : K + 1 with K = fast_k (the cutoff clamped to 2^62-1) */
    int fast;
    i64 fast_k;
    /* Jaro / Jaro-Winkler: every query's JaroTab, filled by k_jaro_tables before the
     * tile kernels (null: the tile kernel builds it) */
    const JaroTab* jtab;
    /* per visiting position p: start offset and length of choice perm[p] (coalesced
     * loads that do not wait for perm); null when the batch brings its own order */
    const int64_t* poff;
    const int32_t* plen;
    /* token_set_ratio family: part lengths (original, sorted join, deduplicated join) of
     * every query / choice string, three int32 each */
    const int32_t* qparts;
    const int32_t* cparts;
    /* warp tiles of the distance fast path (k_fast): per visiting position {offset (low,
     * high 32 bits), length, index within its window}, windows of `stage` positions each
     * sorted by length; vec = 1 when every result row segment of a window starts on a
     * 16-byte boundary */
    const int4* prec;
    int vec;
    /* warp tiles: per visiting position the choice's count histogram (two uint4,
     * hist_lower_bound), and whether the count filter runs (cfilter) */
    const uint4* chist;
    int cfilter;
    /* band launches: the queries' records (BandQuery) */
    const BandQuery* band_q;
};

/* editops of many pairs (k_editops): one operation, laid out as rfg_editop */
struct EditopDev {
    int32_t type;
    int32_t reserved;
    int64_t src_pos;
    int64_t dest_pos;
};

struct EditopsParams {
    KStrings a, b;       /* s1 and s2 of every pair */
    const int64_t* pre;  /* common prefix length per pair */
    const int64_t* suf;  /* common suffix length per pair */
    const int64_t* moff; /* first scratch word of each pair's matrix (within the launch) */
    const int64_t* ooff; /* first operation slot of each pair's output region */
    u64* mat;
    EditopDev* ops;
    int64_t* count; /* operations per pair */
    int* err;       /* device-side check flag */
    int64_t p0, np; /* the pairs of this launch */
    int lev;        /* 1: Levenshtein, 0: LCSseq / Indel */
    /* Levenshtein pairs that may need the reference's Hirschberg recursion (hb[i] = 1) run
     * in k_editops_hb with the caller's score hint; the others in k_editops */
    const unsigned char* hb;
    uint64_t hint;
};

/* ----------------------------------------------------------------- helpers */

__device__ __forceinline__ u64 load_unit(const unsigned char* base, int width, int64_t i)
{
    switch (width) {
    case 1: return __ldg(base + i);
    case 2: return __ldg((const unsigned short*)base + i);
    case 4: return __ldg((const unsigned int*)base + i);
    default: return __ldg((const unsigned long long*)base + i);
    }
}

__device__ __forceinline__ u32 hash_slot(u64 c, int hmask) { return (u32)((c * 0x9E3779B97F4A7C15ull) >> 32) & (u32)hmask; }

/* row index of code unit c in a table with hcap hash slots */
__device__ __forceinline__ int resolve_row(const u64* keys, int hcap, u64 c)
{
    if (c < 256) return (int)c;
    if (!hcap) return 256;
    u32 k = hash_slot(c, hcap - 1);
    for (int probe = 0; probe < hcap; ++probe) {
        const u64 key = keys[k];
        if (key == c) return 256 + (int)k;
        if (key == 0) break;
        k = (k + 1) & (u32)(hcap - 1);
    }
    return 256 + hcap;
}

/* Build the pattern table of query string (base, m, width) into rows/keys.  Must be
 * called by all threads of the CTA; ends with a barrier. */
template <int W>
__device__ void build_pm(u64* rows, u64* keys, int hcap, const unsigned char* base, int m, int width, int* err)
{
    const int nrows = 256 + hcap + 1;
    for (int i = threadIdx.x; i < nrows * W; i += blockDim.x) rows[i] = 0;
    for (int i = threadIdx.x; i < hcap; i += blockDim.x) keys[i] = 0;
    __syncthreads();
    if (hcap) {
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const u64 c = load_unit(base, width, i);
            if (c < 256) continue;
            u32 k = hash_slot(c, hcap - 1);
            int probe = 0;
            for (; probe < hcap; ++probe) {
                const u64 old = atomicCAS((unsigned long long*)&keys[k], 0ull, (unsigned long long)c);
                if (old == 0 || old == c) break;
                k = (k + 1) & (u32)(hcap - 1);
            }
            if (probe == hcap) atomicExch(err, 1); /* table sized too small by the host */
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const u64 c = load_unit(base, width, i);
        const int r = resolve_row(keys, hcap, c);
        if (r < 256 + hcap) atomicOr((unsigned long long*)&rows[r * W + (i >> 6)], 1ull << (i & 63));
    }
    __syncthreads();
}

/* pattern accessors over resolved rows */
template <int W>
struct PMRows {
    const u64* rows;
    __device__ __forceinline__ u64 operator()(u64 r) const { return rows[r * W]; }
    __device__ __forceinline__ u64 operator()(u64 r, int w) const { return rows[r * W + w]; }
};

/* text accessor: yields the resolved row of s2[j] */
template <typename CT, bool WIDE>
struct TextRows {
    const CT* p;
    const u64* keys;
    int hcap;
    __device__ __forceinline__ u64 operator[](int j) const
    {
        const u64 c = (u64)__ldg(p + j);
        if (!WIDE) return c;
        return (u64)resolve_row(keys, hcap, c);
    }
};

static __device__ __noinline__ double int_result_as_double(i64 v) { return (double)v; }

__device__ __forceinline__ void store_result(const KParams& a, int64_t q, int64_t c, i64 vi, double vf, bool is_int)
{
    const int64_t idx = q * a.ld + c;
    switch (a.out_dtype) {
    case 0: ((int32_t*)a.out)[idx] = (int32_t)vi; break;
    case 1: ((int64_t*)a.out)[idx] = vi; break;
    default: ((double*)a.out)[idx] = is_int ? int_result_as_double(vi) : vf;
    }
}

__device__ __forceinline__ bool result_is_int(int metric, int op)
{
    if (metric == JARO || metric == JARO_WINKLER || metric >= RATIO) return false;
    return op == DISTANCE || op == SIMILARITY;
}

/* ------------------------------------------------------- extract epilogue */

#define RFG_MAX_TOPK 32

/* per-thread list of the best results so far (extract kernels only) */
template <bool TOPK>
struct TopList {
    int n;
};
template <>
struct TopList<true> {
    u64 key[RFG_MAX_TOPK];
    int64_t idx[RFG_MAX_TOPK];
    int n;
};

__device__ __forceinline__ bool cand_better(u64 ka, int64_t ia, u64 kb, int64_t ib, int tie_last)
{
    if (ia < 0) return false;
    if (ib < 0) return true;
    if (ka != kb) return ka > kb;
    return tie_last ? ia > ib : ia < ib;
}

__device__ __forceinline__ void top_insert(TopList<true>& tl, int k, u64 key, int64_t idx, int tie_last)
{
    if (tl.n == k && !cand_better(key, idx, tl.key[k - 1], tl.idx[k - 1], tie_last)) return;
    int pos = tl.n < k ? tl.n : k - 1;
    while (pos > 0 && cand_better(key, idx, tl.key[pos - 1], tl.idx[pos - 1], tie_last)) {
        tl.key[pos] = tl.key[pos - 1];
        tl.idx[pos] = tl.idx[pos - 1];
        --pos;
    }
    tl.key[pos] = key;
    tl.idx[pos] = idx;
    if (tl.n < k) ++tl.n;
}

__device__ __forceinline__ u64 score_key(bool is_int, i64 vi, double vf, int better_high)
{
    const u64 raw = is_int ? (u64)vi : (u64)__double_as_longlong(vf);
    return better_high ? raw : ~raw;
}

/* the cutoff of one pair, tightened by the query's running threshold */
__device__ __forceinline__ void tightened_cutoff(const KParams& a, int64_t qi, bool is_int, u64* ci, double* cf)
{
    *ci = a.ci;
    *cf = a.cf;
    if (a.topk <= 0 || !a.thr) return;
    const u64 key = *(volatile const u64*)(a.thr + qi);
    if (key == 0) return;
    const u64 raw = a.better_high ? key : ~key;
    if (is_int) *ci = a.better_high ? (raw > a.ci ? raw : a.ci) : (raw < a.ci ? raw : a.ci);
    else {
        const double v = __longlong_as_double((long long)raw);
        *cf = a.better_high ? (v > a.cf ? v : a.cf) : (v < a.cf ? v : a.cf);
    }
}

/* a result passes the (tightened) cutoff: the reference's extract keeps score >= cutoff
 * for similarities and score <= cutoff for distances */
__device__ __forceinline__ bool passes(bool is_int, int better_high, i64 vi, double vf, u64 ci, double cf)
{
    if (is_int) return better_high ? (u64)vi >= ci : (u64)vi <= ci;
    return better_high ? vf >= cf : vf <= cf;
}

/* Block-wide selection of the tile's best results into the candidate arrays; all
 * threads call it; tl is consumed. */
static __device__ void flush_topk(const KParams& a, int64_t qi, int64_t ch, TopList<true>& tl)
{
    __shared__ u64 s_key[32];
    __shared__ int64_t s_idx[32];
    __shared__ int64_t s_win;
    const int k = a.topk;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int head = 0;
    const int64_t base = (qi * a.nchunks + ch) * k;
    u64 last_key = 0;
    int filled = 0;
    for (int r = 0; r < k; ++r) {
        u64 bk = head < tl.n ? tl.key[head] : 0;
        int64_t bi = head < tl.n ? tl.idx[head] : -1;
        for (int o = 16; o > 0; o >>= 1) {
            const u64 ok = __shfl_down_sync(0xffffffffu, bk, o);
            const int64_t oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (cand_better(ok, oi, bk, bi, a.tie_last)) {
                bk = ok;
                bi = oi;
            }
        }
        if (lane == 0) {
            s_key[warp] = bk;
            s_idx[warp] = bi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            u64 wk = s_key[0];
            int64_t wi = s_idx[0];
            for (int w = 1; w < nw; ++w)
                if (cand_better(s_key[w], s_idx[w], wk, wi, a.tie_last)) {
                    wk = s_key[w];
                    wi = s_idx[w];
                }
            a.cand_key[base + r] = wk;
            a.cand_idx[base + r] = wi;
            s_win = wi;
            if (wi >= 0) {
                last_key = wk;
                ++filled;
            }
        }
        __syncthreads();
        const int64_t win = s_win;
        if (win >= 0 && head < tl.n && tl.idx[head] == win) ++head;
        __syncthreads();
    }
    if (threadIdx.x == 0 && filled == k && a.thr) atomicMax((unsigned long long*)(a.thr + qi), last_key);
    tl.n = 0;
}

/* chunk visited at step r of a query whose own length falls in chunk c0: c0, c0+1,
 * c0-1, c0+2, ... (then one-sided once a side is exhausted) */
__device__ __forceinline__ int64_t center_out(int64_t c0, int64_t r, int64_t nchunks)
{
    const int64_t below = c0, above = nchunks - 1 - c0;
    const int64_t m2 = below < above ? below : above;
    if (r == 0) return c0;
    if (r <= 2 * m2) {
        const int64_t k = (r + 1) / 2;
        return (r & 1) ? c0 + k : c0 - k;
    }
    const int64_t t = r - 2 * m2;
    return below > above ? c0 - (m2 + t) : c0 + (m2 + t);
}

/* first chunk whose length range reaches m (chunks are in ascending length order) */
__device__ __forceinline__ int64_t chunk_of_length(const int32_t* lmax, int64_t nchunks, int m)
{
    int64_t lo = 0, hi = nchunks - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (lmax[mid] < m) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* An extract tile can be skipped when no pair of it can pass the running threshold:
 * distance ops of the unit-cost families, where every distance is >= |m - n|. */
__device__ __forceinline__ bool tile_hopeless(const KParams& a, int64_t qi, int m, int64_t ch)
{
    if (!a.chunk_lmin || a.op != DISTANCE) return false;
    const bool unit = a.metric == INDEL || a.metric == LCSSEQ || a.metric == OSA ||
                      (a.metric == LEVENSHTEIN && a.sp.ins == 1 && a.sp.del == 1 && a.sp.rep == 1);
    if (!unit) return false;
    u64 K;
    double unused;
    tightened_cutoff(a, qi, true, &K, &unused);
    const int64_t lo = a.chunk_lmin[ch], hi = a.chunk_lmax[ch];
    if (K >= (u64)0x7fffffff) return false;
    return hi < (int64_t)m - (int64_t)K || lo > (int64_t)m + (int64_t)K;
}

/* dense store, or the extract list */
__device__ __forceinline__ void emit(const KParams& a, int64_t qi, int64_t ci, i64 vi, double vf, bool is_int,
                                     u64 cut_i, double cut_f, TopList<false>* tl, unsigned char* stage = nullptr,
                                     int64_t s0 = 0)
{
    (void)cut_i;
    (void)cut_f;
    (void)tl;
    if (stage) {
        const int64_t i = ci - s0;
        switch (a.out_dtype) {
        case 0: ((int32_t*)stage)[i] = (int32_t)vi; break;
        case 1: ((int64_t*)stage)[i] = vi; break;
        default: ((double*)stage)[i] = is_int ? int_result_as_double(vi) : vf;
        }
        return;
    }
    store_result(a, qi, ci, vi, vf, is_int);
}

/* one window's staged results to out[qi][s0, s1), consecutive threads on consecutive
 * elements */
__device__ __forceinline__ void flush_stage(const KParams& a, const unsigned char* stage, int64_t qi, int64_t s0,
                                            int64_t s1)
{
    const int64_t n = s1 - s0, base = qi * a.ld + s0;
    if (a.out_dtype == 0) {
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) ((int32_t*)a.out)[base + i] = ((const int32_t*)stage)[i];
    }
    else {
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
            ((unsigned long long*)a.out)[base + i] = ((const unsigned long long*)stage)[i];
    }
}

__device__ __forceinline__ void emit(const KParams& a, int64_t qi, int64_t ci, i64 vi, double vf, bool is_int,
                                     u64 cut_i, double cut_f, TopList<true>* tl, unsigned char* = nullptr,
                                     int64_t = 0)
{
    if (passes(is_int, a.better_high, vi, vf, cut_i, cut_f))
        top_insert(*tl, a.topk, score_key(is_int, vi, vf, a.better_high), ci, a.tie_last);
}

/* -------------------------------------------------------- integer families */

template <int FAM, int W, typename PMF, typename TXT>
__device__ __forceinline__ i64 run_int_core(const PMF& pm, int m, const TXT& t, int n, i64 K)
{
    if (FAM == FAM_LCS) {
        if (m == 0 || n == 0) return 0;
        if (K < (i64)(m > n ? m - n : n - m)) return -1; /* Indel distance >= |m-n| */
        if (W == 1) return lcs_word(pm, m, t, n, K);
        return lcs_multi<W>(pm, m, t, n, K);
    }
    if (m == 0) return n;
    const i64 diff = m > n ? m - n : n - m;
    if (K < diff) return K + 1; /* length filter (Levenshtein_impl.hpp:863) */
    if (FAM == FAM_OSA) {
        if (n == 0) return m;
        if (W == 1) return osa_word(pm, m, t, n, K);
        return osa_multi<W>(pm, m, t, n, K);
    }
    /* FAM_LEV */
    if (n == 0) return m;
    if (W == 1) return lev_word(pm, m, t, n, K);
    /* a diagonal band narrower than the full pattern (Levenshtein_impl.hpp:876-897) */
    if (K < m) {
        const i64 band = 2 * K + 1;
        if (W > 1 && band <= 64) return lev_band<1>(pm, W, m, t, n, (int)K);
        if (W > 2 && band <= 128) return lev_band<2>(pm, W, m, t, n, (int)K);
        if (W > 4 && band <= 256) return lev_band<4>(pm, W, m, t, n, (int)K);
    }
    return lev_multi<W>(pm, m, t, n, K);
}

/* unit-weight Levenshtein of a pattern of W > 1 words with bound K (|m - n| <= K, n > 0):
 * the 64-bit diagonal band of 2K + 1 bits when it is narrower than the pattern and at
 * most 512 bits, else every word; the distance, or any value > K */
template <typename PMW, typename TXT>
__device__ __forceinline__ i64 lev_long_core(const PMW& pm, int W, int m, const TXT& txt, int n, i64 K, u64* st)
{
    if (K < m && 2 * K + 1 <= 64) return lev_band<1>(pm, W, m, txt, n, (int)K);
    if (K < m && 2 * K + 1 <= 128) return lev_band<2>(pm, W, m, txt, n, (int)K);
    if (K < m && 2 * K + 1 <= 256) return lev_band<4>(pm, W, m, txt, n, (int)K);
    if (K < m && 2 * K + 1 <= 512) return lev_band<8>(pm, W, m, txt, n, (int)K);
    return lev_multi_rt(pm, W, m, txt, n, K, st, st + W);
}

/* one (query, choice) pair of an integer-valued or Jaro family */
/* per-query length tables (see JaroTab / chain_kd) */
union LenTab {
    JaroTab jt;
    u64 kd[RFG_JT_MAXT + 1];
};

__device__ __forceinline__ bool uses_jaro_tab(const KParams& a) { return a.form != FORM_MULTI && a.tab_t >= 0; }
__device__ __forceinline__ bool uses_kd_tab(const KParams& a)
{
    const int op = a.metric == RATIO ? NORM_SIMILARITY : a.op;
    return a.form != FORM_MULTI && a.tab_t >= 0 && op >= NORM_DISTANCE;
}

/* build the tables of query length m; all threads; ends with a barrier */
template <int FAM>
__device__ __noinline__ void build_len_tab(const KParams& a, int m, LenTab& t)
{
    PairSpec s;
    s.metric = a.metric;
    s.op = a.op;
    s.form = a.form;
    s.l1 = (u64)m;
    s.ci = a.ci;
    s.cf = a.cf;
    s.p = a.sp;
    if (FAM == FAM_JARO) {
        if (!uses_jaro_tab(a)) return;
        if (threadIdx.x == 0) jaro_tab_head(t.jt, s);
        for (int i = threadIdx.x; i < 5 * (a.tab_t + 1); i += blockDim.x) {
            const int p = i / (a.tab_t + 1), tl = i % (a.tab_t + 1);
            t.jt.minc[p][tl] = jaro_tab_minc(s, m, p, tl);
        }
    }
    else {
        if (!uses_kd_tab(a)) return;
        for (int tl = threadIdx.x; tl <= a.tab_t; tl += blockDim.x) {
            s.l2 = (u64)tl;
            t.kd[tl] = chain_kd(s);
        }
    }
    __syncthreads();
}

template <int FAM, int W, typename CT, bool TOPK>
__device__ __forceinline__ void score_pair(const KParams& a, const u64* rows, const u64* keys, int64_t qi, int m,
                                           const u64* qpre, int64_t ci, int64_t o0, int n, TopList<TOPK>* tl,
                                           const LenTab& lt, unsigned char* stage, int64_t s0)
{
    const CT* s2 = (const CT*)a.c.data + o0;
    PairSpec s;
    s.metric = a.metric;
    s.op = a.op;
    s.form = a.form;
    s.l1 = (u64)m;
    s.l2 = (u64)n;
    const bool is_int = result_is_int(a.metric, a.op);
    s.ci = a.ci;
    s.cf = a.cf;
    if (TOPK) tightened_cutoff(a, qi, is_int, &s.ci, &s.cf);
    s.p = a.sp;
    const PMRows<W> pm{rows};
    const TextRows<CT, (sizeof(CT) > 1)> txt{s2, keys, a.hcap};
    i64 vi = 0;
    double vf = 0.0;
    if (FAM == FAM_JARO) {
        i64 prefix = 0;
        const int mx = (m < n ? m : n) < 4 ? (m < n ? m : n) : 4;
        for (; prefix < mx; ++prefix)
            if ((u64)__ldg(s2 + prefix) != qpre[prefix]) break;
        int common = 0, transp = 0;
        if (uses_jaro_tab(a) && n <= a.tab_t && !TOPK) {
            /* the table decides which pairs need counts and whether they can pass; a pair
             * whose common count stays below minc takes the precomputed failing value */
            const unsigned short mc = lt.jt.minc[prefix][n];
            const int cmax = m < n ? m : n;
            const bool one = m == 1 && n == 1;
            bool fail = mc != 0 && !one && (mc == 0xffff || cmax < (int)mc);
            if (mc != 0 && !fail) {
                const int need = one ? 0 : (int)mc;
                if (W == 1) {
                    int bound = (m > n ? m : n) / 2;
                    if (bound > 0) --bound;
                    const int te = n < m + bound ? n : m + bound;
                    if (te <= 64) jaro_word(pm, m, txt, n, &common, &transp, need);
                    else jaro_multi<1>(pm, m, txt, n, &common, &transp);
                }
                else {
                    jaro_multi<W>(pm, m, txt, n, &common, &transp);
                }
                fail = common < need;
            }
            /* counts never read (mc == 0) give the inner Jaro 0.0 unless both strings are
             * empty: the failing value as well */
            if (mc == 0 && !(m == 0 && n == 0)) fail = true;
            vf = fail ? lt.jt.vfail[prefix] : finish_jaro_tab(s, lt.jt, prefix, common, transp);
            emit(a, qi, ci, 0, vf, false, s.ci, s.cf, tl, stage, s0);
            return;
        }
        if (m > 0 && n > 0 && jaro_pair_needs_counts(s, prefix)) {
            if (W == 1) {
                int bound = (m > n ? m : n) / 2;
                if (bound > 0) --bound;
                const int te = n < m + bound ? n : m + bound;
                if (te <= 64) jaro_word(pm, m, txt, n, &common, &transp);
                else jaro_multi<1>(pm, m, txt, n, &common, &transp);
            }
            else {
                jaro_multi<W>(pm, m, txt, n, &common, &transp);
            }
        }
        vf = finish_jaro(s, prefix, common, transp);
        emit(a, qi, ci, 0, vf, false, s.ci, s.cf, tl, stage, s0);
        return;
    }
    if (a.fast) {
        /* extract: the cutoff tightened by the query's running threshold (s.ci) */
        const i64 K = TOPK ? clamp_bound(s.ci) : a.fast_k;
        const i64 raw = run_int_core<FAM, W>(pm, m, txt, n, K);
        i64 d = raw;
        if (FAM == FAM_LCS) d = raw >= 0 ? (i64)m + n - 2 * raw : K + 1;
        emit(a, qi, ci, d <= K ? d : K + 1, 0.0, true, s.ci, s.cf, tl, stage, s0);
        return;
    }
    if (!TOPK && n <= a.tab_t && uses_kd_tab(a)) s.kd_pre = lt.kd[n];
    const Plan pl = plan_int(s);
    i64 raw = 0;
    if (pl.run) raw = run_int_core<FAM, W>(pm, m, txt, n, pl.K);
    finish_int(s, pl, raw, &vi, &vf);
    emit(a, qi, ci, vi, vf, is_int, s.ci, s.cf, tl, stage, s0);
}

/* visiting position p: its choice, the choice's start offset and length */
struct PosMeta {
    int64_t ci, o;
    int n;
};

__device__ __forceinline__ PosMeta load_pos(const KParams& a, int64_t p)
{
    return PosMeta{(int64_t)__ldg(a.perm + p), __ldg(a.poff + p), __ldg(a.plen + p)};
}

/* pull the first 128-byte line of a non-empty choice into L1 (no register waits on it) */
__device__ __forceinline__ void prefetch_text(const KParams& a, const PosMeta& m)
{
    if (m.n > 0) asm volatile("prefetch.global.L1 [%0];" ::"l"(a.c.data + m.o * a.c.width));
}

/* -------------------------------------------------------------- the kernel */

/* resident 256-thread CTAs per SM the register allocation must allow, per word class:
 * the single-word kernels are latency bound and gain from a fifth CTA; the wide classes
 * keep their state in registers */
#ifndef RFG_MINB_W1
#define RFG_MINB_W1 4
#endif
#ifndef RFG_MINB_W2
#define RFG_MINB_W2 4
#endif
#ifndef RFG_MINB_W4
#define RFG_MINB_W4 2
#endif
#ifndef RFG_MINB_W8
#define RFG_MINB_W8 1
#endif
constexpr int tiles_min_blocks(int W)
{
    return W == 1 ? RFG_MINB_W1 : W == 2 ? RFG_MINB_W2 : W == 4 ? RFG_MINB_W4 : RFG_MINB_W8;
}

template <int FAM, typename CT, int W, bool TOPK = false>
__global__ void __launch_bounds__(256, tiles_min_blocks(W)) k_tiles(const KParams a)
{
    extern __shared__ u64 smem[];
    const int nrows = 256 + a.hcap + 1;
    u64* rows = smem;
    u64* keys = smem + (size_t)nrows * W;
    __shared__ int64_t s_tile;
    __shared__ u64 s_qpre[4];
    __shared__ LenTab s_lt;
    int64_t cur_q = -1;
    int m = 0;
    TopList<TOPK> tl;
    tl.n = 0;
    const int64_t ntiles = (int64_t)a.nq * a.nchunks;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(a.counter, 1);
        __syncthreads();
        const int64_t t = s_tile;
        if (t >= ntiles) break;
        /* extract batches sweep the corpus chunk-major (every query of the batch scores a
         * chunk while it is in L2); dense batches go query-major (coalesced rows) */
        const int64_t qi = TOPK ? a.qlist[t % a.nq] : a.qlist[t / a.nchunks];
        int64_t ch = TOPK ? t / a.nq : t % a.nchunks;
        if (TOPK && a.chunk_lmin) {
            const int ql = (int)(a.q.off[qi + 1] - a.q.off[qi]);
            ch = center_out(chunk_of_length(a.chunk_lmax, a.nchunks, ql), ch, a.nchunks);
        }
        if (qi != cur_q) {
            const int64_t q0 = a.q.off[qi];
            m = (int)(a.q.off[qi + 1] - q0);
            const unsigned char* qb = a.q.data + q0 * a.q.width;
            if (m > 64 * W) { /* the host classified this query into a smaller class */
                if (threadIdx.x == 0) atomicExch(a.err, 2);
                m = 64 * W;
            }
            build_pm<W>(rows, keys, a.hcap, qb, m, a.q.width, a.err);
            if (threadIdx.x < 4) s_qpre[threadIdx.x] = (int)threadIdx.x < m ? load_unit(qb, a.q.width, threadIdx.x) : 0;
            if (!TOPK) {
                if (FAM == FAM_JARO && a.jtab && uses_jaro_tab(a)) {
                    /* copy the precomputed table (the doubles and the minc rows) */
                    const u64* src = (const u64*)(a.jtab + qi);
                    u64* dst = (u64*)&s_lt.jt;
                    for (int i = threadIdx.x; i < (int)(sizeof(JaroTab) / 8); i += blockDim.x) dst[i] = __ldg(src + i);
                    __syncthreads();
                }
                else build_len_tab<FAM>(a, m, s_lt);
            }
            __syncthreads();
            cur_q = qi;
        }
        const int64_t c0 = ch * a.chunk;
        const int64_t c1 = c0 + a.chunk < a.c.n ? c0 + a.chunk : a.c.n;
        /* positions of a chunk are visited in length order, so the threads of a warp get
         * pairs of similar work and pairs decided by the length filter cluster into
         * whole warps */
        const bool skip = TOPK && tile_hopeless(a, qi, m, ch);
        unsigned char* stage = (!TOPK && a.stage) ? (unsigned char*)(keys + a.hcap) : nullptr;
        const int64_t win = stage ? a.stage : c1 - c0;
        for (int64_t s0 = c0; s0 < c1 && !skip; s0 += win) {
            const int64_t s1 = s0 + win < c1 ? s0 + win : c1;
            if (!TOPK && a.poff) {
                /* two positions ahead: (choice, offset, length) two iterations early, the
                 * text's first line pulled into L1 one iteration early */
                const int64_t bd = blockDim.x;
                int64_t p = s0 + threadIdx.x;
                PosMeta cur{0, 0, 0}, nxt{0, 0, 0};
                if (p < s1) cur = load_pos(a, p);
                if (p + bd < s1) nxt = load_pos(a, p + bd);
                if (p < s1) prefetch_text(a, cur);
                for (; p < s1; p += bd) {
                    const PosMeta m0 = cur;
                    cur = nxt;
                    if (p + 2 * bd < s1) nxt = load_pos(a, p + 2 * bd);
                    if (p + bd < s1) prefetch_text(a, cur);
                    score_pair<FAM, W, CT, TOPK>(a, rows, keys, qi, m, s_qpre, m0.ci, m0.o, m0.n, &tl, s_lt, stage, s0);
                }
            }
            else {
                for (int64_t p = s0 + threadIdx.x; p < s1; p += blockDim.x) {
                    const int64_t ci = a.perm ? (int64_t)__ldg(a.perm + p) : p;
                    const int64_t o0 = a.c.off[ci];
                    score_pair<FAM, W, CT, TOPK>(a, rows, keys, qi, m, s_qpre, ci, o0, (int)(a.c.off[ci + 1] - o0), &tl,
                                                 s_lt, stage, s0);
                }
            }
            if (stage) {
                __syncthreads();
                flush_stage(a, stage, qi, s0, s1);
                __syncthreads();
            }
        }
        if constexpr (TOPK) flush_topk(a, qi, ch, tl);
        __syncthreads();
    }
}

/* --------------------------------------------- any-length kernel (scratch)
 * Queries longer than 512 code units (and the weighted Wagner-Fischer family) run one
 * pair per thread with their state in global scratch: per CTA a pattern table of
 * (256 + hcap + 1) * wmax words plus hcap keys, then per thread scratch_per_thread
 * words of recurrence state (VP/VN/..., Jaro flags, or the Wagner-Fischer row). */

template <typename CT>
struct RawText {
    const CT* p;
    __device__ __forceinline__ u64 operator[](int j) const { return (u64)__ldg(p + j); }
};

struct RawQuery {
    const unsigned char* p;
    int width;
    __device__ __forceinline__ u64 operator[](int j) const { return load_unit(p, width, j); }
};

struct PMRowsRT {
    const u64* rows;
    int W;
    __device__ __forceinline__ u64 operator()(u64 r, int w) const { return rows[r * W + w]; }
};

/* build_pm for a runtime word count, table in global memory */
__device__ inline void build_pm_rt(u64* rows, u64* keys, int hcap, int W, const unsigned char* base, int m,
                                   int width, int* err)
{
    const int64_t nrows = 256 + hcap + 1;
    for (int64_t i = threadIdx.x; i < nrows * W; i += blockDim.x) rows[i] = 0;
    for (int i = threadIdx.x; i < hcap; i += blockDim.x) keys[i] = 0;
    __syncthreads();
    if (hcap) {
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const u64 c = load_unit(base, width, i);
            if (c < 256) continue;
            u32 k = hash_slot(c, hcap - 1);
            int probe = 0;
            for (; probe < hcap; ++probe) {
                const u64 old = atomicCAS((unsigned long long*)&keys[k], 0ull, (unsigned long long)c);
                if (old == 0 || old == c) break;
                k = (k + 1) & (u32)(hcap - 1);
            }
            if (probe == hcap) atomicExch(err, 1);
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const u64 c = load_unit(base, width, i);
        const int r = resolve_row(keys, hcap, c);
        if (r < 256 + hcap) atomicOr((unsigned long long*)&rows[(int64_t)r * W + (i >> 6)], 1ull << (i & 63));
    }
    __syncthreads();
}

template <int FAM, typename CT, bool TOPK = false>
__device__ __forceinline__ void score_pair_generic(const KParams& a, const u64* rows, const u64* keys, int W,
                                                   int64_t qi, int m, const unsigned char* qb, int64_t ci, u64* st,
                                                   TopList<TOPK>* tl = nullptr)
{
    const int64_t o0 = a.c.off[ci], o1 = a.c.off[ci + 1];
    const int n = (int)(o1 - o0);
    const CT* s2 = (const CT*)a.c.data + o0;
    PairSpec s;
    s.metric = a.metric;
    s.op = a.op;
    s.form = a.form;
    s.l1 = (u64)m;
    s.l2 = (u64)n;
    const bool is_int = result_is_int(a.metric, a.op);
    s.ci = a.ci;
    s.cf = a.cf;
    if (TOPK) tightened_cutoff(a, qi, is_int, &s.ci, &s.cf);
    s.p = a.sp;
    const PMRowsRT pm{rows, W};
    const TextRows<CT, (sizeof(CT) > 1)> txt{s2, keys, a.hcap};
    i64 vi = 0;
    double vf = 0.0;
    if (FAM == FAM_PARTIAL) {
        /* fuzz::partial_ratio: W + 1 state words, then the window bookkeeping */
        vf = partial_ratio_dev(pm, W, m, txt, n, s.cf, st, (u32*)(st + W + 1));
        emit(a, qi, ci, 0, vf, false, s.ci, s.cf, tl);
        return;
    }
    if (FAM == FAM_TOKEN) {
        /* the token_set_ratio family over the parts of both concatenations */
        const int32_t* qp = a.qparts + 3 * qi;
        const int32_t* cp = a.cparts + 3 * ci;
        const RawQuery q{qb, a.q.width};
        const RawText<CT> c{s2};
        typedef TokPair<PMRowsRT, RawQuery, decltype(txt), RawText<CT>> Pair;
        const Pair p{&pm, W, &q, &txt, &c, qp[0], qp[1], qp[2], __ldg(cp), __ldg(cp + 1), __ldg(cp + 2)};
        /* extract: every pair is scored with the caller's cutoff (the running threshold
         * only filters), so the lists equal a dense matrix filtered afterwards */
        vf = token_family_dev(a.metric, p, a.cf, st);
        emit(a, qi, ci, 0, vf, false, s.ci, s.cf, tl);
        return;
    }
    if (FAM == FAM_JARO) {
        const RawQuery q{qb, a.q.width};
        i64 prefix = 0;
        const int mx = (m < n ? m : n) < 4 ? (m < n ? m : n) : 4;
        for (; prefix < mx; ++prefix)
            if ((u64)__ldg(s2 + prefix) != q[prefix]) break;
        int common = 0, transp = 0;
        if (m > 0 && n > 0 && jaro_pair_needs_counts(s, prefix))
            jaro_multi_rt(pm, W, m, txt, n, &common, &transp, st, st + W);
        vf = finish_jaro(s, prefix, common, transp);
        emit(a, qi, ci, 0, vf, false, s.ci, s.cf, tl);
        return;
    }
    const Plan pl = plan_int(s);
    i64 raw = 0;
    if (pl.run) {
        const i64 K = pl.K;
        const i64 diff = m > n ? m - n : n - m;
        if (FAM == FAM_WF) {
            const RawQuery q{qb, a.q.width};
            const RawText<CT> t2{s2};
            raw = (i64)wf_distance(q, m, t2, n, a.sp, (u64)K, st);
        }
        else if (FAM == FAM_LCS) {
            if (m == 0 || n == 0) raw = 0;
            else if (K < diff) raw = -1;
            else raw = lcs_multi_rt(pm, W, m, txt, n, K, st);
        }
        else if (m == 0) raw = n;
        else if (K < diff) raw = K + 1;
        else if (n == 0) raw = m;
        else if (FAM == FAM_OSA) raw = osa_multi_rt(pm, W, m, txt, n, K, st, st + W, st + 2 * W, st + 3 * W);
        else {
            /* the score-hint doubling of uniform_levenshtein_distance
             * (Levenshtein_impl.hpp:876-897): bands of bound h, 2h, 4h ... below K first;
             * the first whose distance fits its bound is exact */
            i64 h = a.has_hint && m > 64 && K >= 4 && lev_mode(s.p) == LEV_UNIFORM && s.p.ins == 1
                        ? lev_hint_bound(s, a.hint_i, a.hint_f)
                        : K;
            h = h > diff ? h : diff;
            bool done = false;
            while (h < K) {
                const i64 d = lev_long_core(pm, W, m, txt, n, h, st);
                if (d <= h) {
                    raw = d;
                    done = true;
                    break;
                }
                h = h > K / 2 ? K : (h > 0 ? 2 * h : 1);
            }
            if (!done) raw = lev_long_core(pm, W, m, txt, n, K, st);
        }
    }
    finish_int(s, pl, raw, &vi, &vf);
    emit(a, qi, ci, vi, vf, is_int, s.ci, s.cf, tl);
}

template <int FAM, typename CT, bool TOPK = false>
__global__ void __launch_bounds__(256) k_generic(const KParams a)
{
    extern __shared__ u64 gsm[];
    const int W = a.wmax;
    const int64_t table = (int64_t)(256 + a.hcap + 1) * W + a.hcap;
    u64* region = a.scratch + (int64_t)blockIdx.x * a.scratch_per_cta;
    u64* rows = a.pm_smem ? gsm : region;
    u64* keys = rows + (int64_t)(256 + a.hcap + 1) * W;
    u64* st = region + (a.pm_smem ? 0 : table) + (int64_t)threadIdx.x * a.scratch_per_thread;
    __shared__ int64_t s_tile;
    __shared__ int s_next;
    int64_t cur_q = -1;
    int m = 0;
    const unsigned char* qb = nullptr;
    TopList<TOPK> tl;
    tl.n = 0;
    const int64_t ntiles = (int64_t)a.nq * a.nchunks;
    /* partial_ratio and the token scorers cost very different amounts per pair: the
     * threads take the tile's choices one at a time instead of a fixed stride */
    constexpr bool kDynamic = FAM == FAM_PARTIAL || FAM == FAM_TOKEN;
    for (;;) {
        if (threadIdx.x == 0) {
            s_tile = atomicAdd(a.counter, 1);
            s_next = 0;
        }
        __syncthreads();
        const int64_t t = s_tile;
        if (t >= ntiles) break;
        const int64_t qi = TOPK ? a.qlist[t % a.nq] : a.qlist[t / a.nchunks];
        int64_t ch = TOPK ? t / a.nq : t % a.nchunks;
        if (TOPK && a.chunk_lmin) {
            const int ql = (int)(a.q.off[qi + 1] - a.q.off[qi]);
            ch = center_out(chunk_of_length(a.chunk_lmax, a.nchunks, ql), ch, a.nchunks);
        }
        if (qi != cur_q) {
            const int64_t q0 = a.q.off[qi];
            m = (int)(a.q.off[qi + 1] - q0);
            qb = a.q.data + q0 * a.q.width;
            if (FAM != FAM_WF) {
                if (m > 64 * W) {
                    if (threadIdx.x == 0) atomicExch(a.err, 2);
                    m = 64 * W;
                }
                build_pm_rt(rows, keys, a.hcap, W, qb, m, a.q.width, a.err);
            }
            cur_q = qi;
        }
        const int64_t c0 = ch * a.chunk;
        const int64_t c1 = c0 + a.chunk < a.c.n ? c0 + a.chunk : a.c.n;
        const bool skip = TOPK && tile_hopeless(a, qi, m, ch);
        if (!skip && kDynamic)
            for (int64_t p = c0 + atomicAdd(&s_next, 1); p < c1; p = c0 + atomicAdd(&s_next, 1))
                score_pair_generic<FAM, CT, TOPK>(a, rows, keys, W, qi, m, qb,
                                                  a.perm ? (int64_t)__ldg(a.perm + p) : p, st, &tl);
        else if (!skip)
            for (int64_t p = c0 + threadIdx.x; p < c1; p += blockDim.x)
                score_pair_generic<FAM, CT, TOPK>(a, rows, keys, W, qi, m, qb,
                                                  a.perm ? (int64_t)__ldg(a.perm + p) : p, st, &tl);
        if constexpr (TOPK) flush_topk(a, qi, ch, tl);
        __syncthreads();
    }
}

/* ------------------------------------------- several queries per thread
 * Unit-weight distances of one-word patterns whose code units are all below 256
 * (distance, or the normalized chains with the integer cutoff from per-query tables):
 * a tile is (Q consecutive queries of the class, chunk); every thread fetches a
 * choice's text once per block of characters and advances the recurrences of all the
 * tile's queries on it (group_word_dist), so text loads, per-choice bookkeeping and
 * the loop overhead are shared by Q pairs and the independent recurrences overlap.
 * Q per family (mq_queries): two for Levenshtein, OSA and Jaro, four for Indel / ratio.
 * Results leave through the staged windows (a.stage positions per query row). */
#ifndef RFG_MINB_MQ
#define RFG_MINB_MQ 4
#endif
#ifndef RFG_MINB_MQ_OSA
#define RFG_MINB_MQ_OSA 3 /* four OSA states (VP, VN, D0, previous X) per query */
#endif

struct MQRows {
    const u64* rows;
    __device__ __forceinline__ u64 operator()(int q, unsigned c) const { return rows[q * 257 + c]; }
};

/* the low 32 bits of the rows (patterns of at most 32 units) */
struct MQRows32 {
    const uint32_t* rows;
    __device__ __forceinline__ uint32_t operator()(int q, unsigned c) const { return rows[2 * (q * 257 + c)]; }
};

template <typename CT>
struct MQText {
    const CT* p;
    __device__ __forceinline__ u64 operator[](int j) const
    {
        const u64 c = (u64)__ldg(p + j);
        return c < 256 ? c : 256; /* units the patterns lack: the zero row */
    }
};

template <int FAM, typename CT, bool NORM, int Q, bool HALF = false>
__global__ void __launch_bounds__(256, FAM == FAM_OSA ? RFG_MINB_MQ_OSA : RFG_MINB_MQ) k_tiles_mq(const KParams a)
{
    extern __shared__ u64 smem[];
    u64* rows = smem;
    /* normalized ops (NORM): chain_kd per (query, text length 0..tab_t) */
    const int tn = NORM ? a.tab_t + 1 : 0;
    u64* kdt = smem + Q * 257;
    unsigned char* stage = (unsigned char*)(kdt + Q * tn);
    __shared__ int64_t s_tile;
    __shared__ int64_t s_q[Q];
    __shared__ int s_m[Q];
    const int64_t ngroups = ((int64_t)a.nq + Q - 1) / Q;
    const int64_t ntiles = ngroups * a.nchunks;
    const i64 K = a.fast_k;
    int64_t cur_g = -1;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(a.counter, 1);
        __syncthreads();
        const int64_t t = s_tile;
        if (t >= ntiles) break;
        const int64_t gi = t / a.nchunks, ch = t % a.nchunks;
        if (gi != cur_g) {
            for (int i = threadIdx.x; i < Q * 257; i += blockDim.x) rows[i] = 0;
            if (threadIdx.x < Q) {
                const int64_t k = gi * Q + threadIdx.x;
                int64_t qi = -1;
                int m = 0;
                if (k < a.nq) {
                    qi = a.qlist[k];
                    m = (int)(a.q.off[qi + 1] - a.q.off[qi]);
                    if (m > (HALF ? 32 : 64)) { /* the host classified this query into a smaller class */
                        atomicExch(a.err, 2);
                        m = HALF ? 32 : 64;
                    }
                }
                s_q[threadIdx.x] = qi;
                s_m[threadIdx.x] = m;
            }
            __syncthreads();
            if (NORM) {
                PairSpec sp;
                sp.metric = a.metric;
                sp.op = a.op;
                sp.form = a.form;
                sp.ci = a.ci;
                sp.cf = a.cf;
                sp.p = a.sp;
                for (int i = threadIdx.x; i < Q * tn; i += blockDim.x) {
                    sp.l1 = (u64)s_m[i / tn];
                    sp.l2 = (u64)(i % tn);
                    kdt[i] = chain_kd(sp);
                }
            }
            for (int q = 0; q < Q; ++q) {
                if (s_q[q] < 0) continue;
                const unsigned char* qb = a.q.data + a.q.off[s_q[q]] * a.q.width;
                for (int i = threadIdx.x; i < s_m[q]; i += blockDim.x) {
                    const u64 c = load_unit(qb, a.q.width, i);
                    /* a unit >= 256 here means one-byte choices, which never hold it */
                    if (c < 256) atomicOr((unsigned long long*)&rows[q * 257 + c], 1ull << i);
                }
            }
            __syncthreads();
            cur_g = gi;
        }
        int m[Q];
        int qn = 0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            m[q] = s_m[q];
            if (s_q[q] >= 0) qn = q + 1;
        }
        typedef typename std::conditional<HALF, MQRows32, MQRows>::type Rows;
        typedef typename std::conditional<HALF, uint32_t, u64>::type Word;
        const Rows pm{(decltype(Rows::rows))rows};
        const int64_t c0 = ch * a.chunk;
        const int64_t c1 = c0 + a.chunk < a.c.n ? c0 + a.chunk : a.c.n;
        for (int64_t s0 = c0; s0 < c1; s0 += a.stage) {
            const int64_t s1 = s0 + a.stage < c1 ? s0 + a.stage : c1;
            int64_t p = s0 + threadIdx.x;
            int64_t ci_n = 0, o_n = 0;
            int n_n = 0;
            if (p < s1) {
                ci_n = __ldg(a.perm + p);
                o_n = __ldg(a.poff + p);
                n_n = __ldg(a.plen + p);
            }
            for (; p < s1; p += blockDim.x) {
                const int64_t ci = ci_n, o0 = o_n;
                const int n = n_n;
                const int64_t pn = p + blockDim.x;
                if (pn < s1) {
                    ci_n = __ldg(a.perm + pn);
                    o_n = __ldg(a.poff + pn);
                    n_n = __ldg(a.plen + pn);
                }
                i64 d[Q], Kq[Q];
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if (!NORM) Kq[q] = K;
                    else {
                        u64 kd;
                        if (n <= a.tab_t) kd = kdt[q * tn + n];
                        else {
                            PairSpec sp;
                            sp.metric = a.metric;
                            sp.op = a.op;
                            sp.form = a.form;
                            sp.ci = a.ci;
                            sp.cf = a.cf;
                            sp.p = a.sp;
                            sp.l1 = (u64)m[q];
                            sp.l2 = (u64)n;
                            kd = chain_kd(sp);
                        }
                        Kq[q] = clamp_bound(kd);
                    }
                }
                group_word_dist<FAM, Q, Rows, MQText<CT>, Word>(pm, m, qn, MQText<CT>{(const CT*)a.c.data + o0}, n, Kq,
                                                                d);
                const int64_t i = ci - s0;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if (q >= qn) break;
                    const int64_t at = (int64_t)q * a.stage + i;
                    if (!NORM) {
                        switch (a.out_dtype) {
                        case 0: ((int32_t*)stage)[at] = (int32_t)d[q]; break;
                        case 1: ((int64_t*)stage)[at] = d[q]; break;
                        default: ((double*)stage)[at] = int_result_as_double(d[q]);
                        }
                    }
                    else {
                        /* the normalized chain over d with its integer cutoff Kq (finish_int) */
                        const u64 M = FAM == FAM_LCS ? (u64)m[q] + n : (u64)(m[q] > n ? m[q] : n);
                        const u64 Kc = (u64)Kq[q], du = (u64)d[q];
                        double vf = 0.0;
                        if (a.metric == RATIO)
                            vf = (M != 0 && du > Kc && abs_le_bits(a.cf, 200.0)) ? 0.0 : ratio_finish(M, du, a.cf, Kc);
                        else {
                            i64 vi = 0;
                            dist_chain_finish(a.op, M, du, a.ci, a.cf, &vi, &vf, Kc);
                        }
                        ((double*)stage)[at] = vf;
                    }
                }
            }
            __syncthreads();
            for (int q = 0; q < qn; ++q) {
                const int64_t base = s_q[q] * a.ld + s0, nn = s1 - s0;
                if (a.out_dtype == 0) {
                    const int32_t* src = (const int32_t*)stage + (int64_t)q * a.stage;
                    for (int64_t i = threadIdx.x; i < nn; i += blockDim.x) ((int32_t*)a.out)[base + i] = src[i];
                }
                else {
                    const unsigned long long* src = (const unsigned long long*)stage + (int64_t)q * a.stage;
                    for (int64_t i = threadIdx.x; i < nn; i += blockDim.x)
                        ((unsigned long long*)a.out)[base + i] = src[i];
                }
            }
            __syncthreads();
        }
    }
}

/* Jaro / Jaro-Winkler over one-word patterns with code units below 256, four queries
 * per thread: the per-query tables come from k_jaro_tables, the flagging of the four
 * patterns shares the text fetch (group_jaro_word); a pair outside the tables or with an
 * effective text end above 64 takes the one-query cores. */
#ifndef RFG_MINB_MQJ
#define RFG_MINB_MQJ 3
#endif

struct MQRow1 {
    const u64* rows;
    __device__ __forceinline__ u64 operator()(u64 c) const { return rows[c]; }
    __device__ __forceinline__ u64 operator()(u64 c, int) const { return rows[c]; }
};

template <typename CT, int Q>
__global__ void __launch_bounds__(256, RFG_MINB_MQJ) k_tiles_mq_jaro(const KParams a)
{
    extern __shared__ u64 smem[];
    u64* rows = smem;
    JaroTab* jt = (JaroTab*)(smem + Q * 257);
    unsigned char* stage = (unsigned char*)(jt + Q);
    __shared__ int64_t s_tile;
    __shared__ int64_t s_q[Q];
    __shared__ int s_m[Q];
    __shared__ u64 s_pre[Q][4];
    const int64_t ngroups = ((int64_t)a.nq + Q - 1) / Q;
    const int64_t ntiles = ngroups * a.nchunks;
    const int tw = (int)(sizeof(JaroTab) / 8);
    int64_t cur_g = -1;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(a.counter, 1);
        __syncthreads();
        const int64_t t = s_tile;
        if (t >= ntiles) break;
        const int64_t gi = t / a.nchunks, ch = t % a.nchunks;
        if (gi != cur_g) {
            for (int i = threadIdx.x; i < Q * 257; i += blockDim.x) rows[i] = 0;
            if (threadIdx.x < Q) {
                const int64_t k = gi * Q + threadIdx.x;
                int64_t qi = -1;
                int m = 0;
                if (k < a.nq) {
                    qi = a.qlist[k];
                    m = (int)(a.q.off[qi + 1] - a.q.off[qi]);
                    if (m > 64) { /* the host classified this query into a smaller class */
                        atomicExch(a.err, 2);
                        m = 64;
                    }
                }
                s_q[threadIdx.x] = qi;
                s_m[threadIdx.x] = m;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < Q * tw; i += blockDim.x) {
                const int q = i / tw;
                if (s_q[q] >= 0) ((u64*)(jt + q))[i % tw] = __ldg((const u64*)(a.jtab + s_q[q]) + i % tw);
            }
            for (int q = 0; q < Q; ++q) {
                if (s_q[q] < 0) continue;
                const unsigned char* qb = a.q.data + a.q.off[s_q[q]] * a.q.width;
                for (int i = threadIdx.x; i < s_m[q]; i += blockDim.x) {
                    const u64 c = load_unit(qb, a.q.width, i);
                    /* a unit >= 256 here means one-byte choices, which never hold it */
                    if (c < 256) atomicOr((unsigned long long*)&rows[q * 257 + c], 1ull << i);
                }
                if (threadIdx.x < 4) s_pre[q][threadIdx.x] = (int)threadIdx.x < s_m[q] ? load_unit(qb, a.q.width, threadIdx.x) : 0;
            }
            __syncthreads();
            cur_g = gi;
        }
        int m[Q];
        int qn = 0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            m[q] = s_m[q];
            if (s_q[q] >= 0) qn = q + 1;
        }
        const MQRows pm{rows};
        const int64_t c0 = ch * a.chunk;
        const int64_t c1 = c0 + a.chunk < a.c.n ? c0 + a.chunk : a.c.n;
        for (int64_t s0 = c0; s0 < c1; s0 += a.stage) {
            const int64_t s1 = s0 + a.stage < c1 ? s0 + a.stage : c1;
            const int64_t bd = blockDim.x;
            int64_t p = s0 + threadIdx.x;
            PosMeta cur{0, 0, 0}, nxt{0, 0, 0};
            if (p < s1) cur = load_pos(a, p);
            if (p + bd < s1) nxt = load_pos(a, p + bd);
            for (; p < s1; p += bd) {
                const PosMeta pos = cur;
                cur = nxt;
                if (p + 2 * bd < s1) nxt = load_pos(a, p + 2 * bd);
                if (p + bd < s1) prefetch_text(a, cur);
                const int n = pos.n;
                const CT* s2 = (const CT*)a.c.data + pos.o;
                const MQText<CT> txt{s2};
                u64 t4[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) t4[k] = k < n ? (u64)__ldg(s2 + k) : ~0ull;
                PairSpec sp;
                sp.metric = a.metric;
                sp.op = a.op;
                sp.form = a.form;
                sp.ci = a.ci;
                sp.cf = a.cf;
                sp.p = a.sp;
                sp.l2 = (u64)n;
                int prefix[Q], need[Q], C[Q], Tr[Q];
                double vf[Q];
                unsigned active = 0, decided = 0;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    prefix[q] = 0;
                    need[q] = 0;
                    vf[q] = 0.0;
                    if (q >= qn) continue;
                    const int mx = (m[q] < n ? m[q] : n) < 4 ? (m[q] < n ? m[q] : n) : 4;
                    int pr = 0;
                    for (; pr < mx; ++pr)
                        if (t4[pr] != s_pre[q][pr]) break;
                    prefix[q] = pr;
                    sp.l1 = (u64)m[q];
                    int bound = (m[q] > n ? m[q] : n) / 2;
                    if (bound > 0) --bound;
                    const int te = n < m[q] + bound ? n : m[q] + bound;
                    if (n <= a.tab_t) {
                        const unsigned short mc = jt[q].minc[pr][n];
                        const int cmax = m[q] < n ? m[q] : n;
                        const bool one = m[q] == 1 && n == 1;
                        const bool fail = mc != 0 && !one && (mc == 0xffff || cmax < (int)mc);
                        if (fail) {
                            vf[q] = jt[q].vfail[pr];
                            decided |= 1u << q;
                        }
                        else if (mc == 0) {
                            /* counts never read: 0.0 inside (the failing value) unless both empty */
                            vf[q] = (m[q] == 0 && n == 0) ? finish_jaro_tab(sp, jt[q], pr, 0, 0) : jt[q].vfail[pr];
                            decided |= 1u << q;
                        }
                        else if (te <= 64) {
                            need[q] = one ? 0 : (int)mc;
                            active |= 1u << q;
                        }
                        else {
                            int c = 0, tr = 0;
                            jaro_multi<1>(MQRow1{rows + q * 257}, m[q], txt, n, &c, &tr);
                            vf[q] = c < (one ? 0 : (int)mc) ? jt[q].vfail[pr] : finish_jaro_tab(sp, jt[q], pr, c, tr);
                            decided |= 1u << q;
                        }
                    }
                    else {
                        /* outside the tables: the reference's filters pair by pair */
                        int c = 0, tr = 0;
                        if (m[q] > 0 && n > 0 && jaro_pair_needs_counts(sp, pr)) {
                            if (te <= 64) jaro_word(MQRow1{rows + q * 257}, m[q], txt, n, &c, &tr);
                            else jaro_multi<1>(MQRow1{rows + q * 257}, m[q], txt, n, &c, &tr);
                        }
                        vf[q] = finish_jaro(sp, pr, c, tr);
                        decided |= 1u << q;
                    }
                }
                if (active) {
                    group_jaro_word<Q>(pm, m, active, txt, n, need, C, Tr);
#pragma unroll
                    for (int q = 0; q < Q; ++q) {
                        if (!((active >> q) & 1u)) continue;
                        sp.l1 = (u64)m[q];
                        vf[q] = C[q] < need[q] ? jt[q].vfail[prefix[q]] : finish_jaro_tab(sp, jt[q], prefix[q], C[q], Tr[q]);
                    }
                }
                (void)decided;
                const int64_t i = pos.ci - s0;
#pragma unroll
                for (int q = 0; q < Q; ++q)
                    if (q < qn) ((double*)stage)[(int64_t)q * a.stage + i] = vf[q];
            }
            __syncthreads();
            for (int q = 0; q < qn; ++q) {
                const int64_t base = s_q[q] * a.ld + s0, nn = s1 - s0;
                const unsigned long long* src = (const unsigned long long*)stage + (int64_t)q * a.stage;
                for (int64_t i = threadIdx.x; i < nn; i += blockDim.x) ((unsigned long long*)a.out)[base + i] = src[i];
            }
            __syncthreads();
        }
    }
}

inline size_t tiles_mq_jaro_smem_bytes(int64_t stage, int Q)
{
    return (size_t)Q * 257 * 8 + (size_t)Q * sizeof(JaroTab) + (size_t)Q * stage * 8;
}

inline size_t tiles_mq_smem_bytes(int64_t stage, int out_dtype, int kd_len, int Q)
{
    return ((size_t)Q * 257 + (size_t)Q * kd_len) * 8 + (size_t)Q * stage * (out_dtype == 0 ? 4 : 8);
}

/* Per query: the best topk of all its tiles' candidates, best first; scores as doubles
 * (integer results convert exactly).  One CTA per query. */
/* One CTA per query: its JaroTab over text lengths 0..tab_t (the double-precision
 * filters once per query instead of once per tile). */
static __global__ void __launch_bounds__(256) k_jaro_tables(const KParams a, JaroTab* out)
{
    const int64_t qi = blockIdx.x;
    if (qi >= a.q.n) return;
    const int m = (int)(a.q.off[qi + 1] - a.q.off[qi]);
    PairSpec s;
    s.metric = a.metric;
    s.op = a.op;
    s.form = a.form;
    s.l1 = (u64)m;
    s.ci = a.ci;
    s.cf = a.cf;
    s.p = a.sp;
    JaroTab& t = out[qi];
    if (threadIdx.x == 0) jaro_tab_head(t, s);
    for (int i = threadIdx.x; i < 5 * (a.tab_t + 1); i += blockDim.x) {
        const int p = i / (a.tab_t + 1), tl = i % (a.tab_t + 1);
        t.minc[p][tl] = jaro_tab_minc(s, m, p, tl);
    }
}

static __global__ void __launch_bounds__(256) k_topk_merge(const u64* cand_key, const int64_t* cand_idx, int64_t nchunks,
                                                     int k, int tie_last, int better_high, int is_int,
                                                     int64_t* out_idx, double* out_score, int32_t* out_count)
{
    __shared__ u64 s_key[32];
    __shared__ int64_t s_idx[32];
    __shared__ int64_t s_win;
    __shared__ u64 s_wkey;
    const int64_t q = blockIdx.x;
    const int64_t n = nchunks * k;
    const u64* ck = cand_key + q * n;
    const int64_t* ci = cand_idx + q * n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int count = 0;
    for (int r = 0; r < k; ++r) {
        u64 bk = 0;
        int64_t bi = -1;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
            if (cand_better(ck[i], ci[i], bk, bi, tie_last)) {
                bk = ck[i];
                bi = ci[i];
            }
        for (int o = 16; o > 0; o >>= 1) {
            const u64 ok = __shfl_down_sync(0xffffffffu, bk, o);
            const int64_t oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (cand_better(ok, oi, bk, bi, tie_last)) {
                bk = ok;
                bi = oi;
            }
        }
        if (lane == 0) {
            s_key[warp] = bk;
            s_idx[warp] = bi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            u64 wk = s_key[0];
            int64_t wi = s_idx[0];
            for (int w = 1; w < nw; ++w)
                if (cand_better(s_key[w], s_idx[w], wk, wi, tie_last)) {
                    wk = s_key[w];
                    wi = s_idx[w];
                }
            s_win = wi;
            s_wkey = wk;
        }
        __syncthreads();
        const int64_t win = s_win;
        if (win < 0) break;
        /* remove the winner (its choice index is unique within the query) */
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
            if (ci[i] == win) ((int64_t*)ci)[i] = -1;
        if (threadIdx.x == 0) {
            const u64 raw = better_high ? s_wkey : ~s_wkey;
            out_idx[q * k + r] = win;
            out_score[q * k + r] = is_int ? (double)(int64_t)raw : __longlong_as_double((long long)raw);
        }
        ++count;
        __syncthreads();
    }
    if (threadIdx.x == 0) out_count[q] = count;
}

/* shared memory of k_tiles<.., W> */
inline size_t tiles_smem_bytes(int W, int hcap) { return ((size_t)(256 + hcap + 1) * W + (size_t)hcap) * 8; }

} // namespace rfg
