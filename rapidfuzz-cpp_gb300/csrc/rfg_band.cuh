/*
 * rfg_band.cuh -- banded Levenshtein (weights 1/1/1) and banded LCS (Indel, LCSseq,
 * ratio) for queries whose every passing pair needs a diagonal band narrower than the
 * pattern: the reference's levenshtein_hyrroe2003_small_band / the band of
 * levenshtein_hyrroe2003_block (Levenshtein_impl.hpp:419-505, 641-850) and the band of
 * lcs_blockwise (LCSseq_impl.hpp:262-333, chosen at :349), on Ukkonen's band of about
 * K + 2 diagonals (lev_band32, lcs_band32; K the Levenshtein bound, or for the LCS
 * families the Indel-distance bound their plans carry), chosen when that band is
 * narrower than the pattern for the largest bound K any pair of the query can reach (the
 * length filters Levenshtein_impl.hpp:863, LCSseq_impl.hpp:389 cap it).
 *
 * Whether a pair passes the length filter depends on its two lengths alone, and the
 * passing choice lengths of a query form one interval [nlo, nhi] (band_range).  With the
 * choices in one global length order (records {offset, length, index}), a query's passing
 * pairs are one contiguous run [plo, phi) of that order.  A launch holds two kinds of
 * warp task, both taken from one counter:
 *   - units: `rounds` groups of 32 consecutive passing pairs of one query, one pair per
 *     lane on B 32-bit words (band_run8; registers sized by the band, not by the
 *     pattern); lanes of a group meet choices of nearly one length;
 *   - fills: 1024 consecutive choices of one query's result row in the caller's order,
 *     storing the value of every pair outside [nlo, nhi] (band_reject_value: the chain's
 *     value of a pruned pair, the same for every such pair) with coalesced stores.
 * Every warp is its own worker (no barrier of the CTA): it keeps in its own slice of
 * shared memory the table of the query it last scored and rebuilds it when a unit of
 * another query comes --
 *   - a compact pattern table: one row of ceil(m/32) 32-bit words for each code unit
 *     the query holds (plus the all-zero row), each row with zero words on either side
 *     so the band's window is loaded without range tests; rmap[c] = the word offset of
 *     unit c's row;
 *   - for the normalized ops, the integer cutoff chain_kd(m, m + j) so that no pair
 *     evaluates the double-precision chain: Levenshtein j = 0..32B (the cutoff depends
 *     on max(m, n) only, so j = 0 serves every n <= m); the LCS families, whose Indel
 *     maximum m + n depends on n on both sides, j = -32B..32B (no passing pair has
 *     |n - m| > K, and K < 32B).
 * One-byte choices only (a wider unit has no row: the zero row would do, but the host
 * keeps wide alphabets on the general kernels).
 */
#pragma once
#include "rfg_device.cuh"

namespace rfg {

/* words of one compact row of a query of m units and band B: the pattern's words, B + 1
 * zero words before and 2B + 2 after (the window of a pair with n up to m + K reads that
 * far past the pattern's last word) */
__host__ __device__ inline int band_row_stride(int m, int B) { return (m + 31) / 32 + 3 * (B + 1); }

/* choices a fill task covers */
#define RFG_BAND_FILL 1024

/* bytes of one warp's slice: rmap (256 ints), the cutoff table (tab_t + 1 entries, or
 * none when tab_t < 0), then `words` 32-bit words of rows */
__host__ __device__ inline size_t band_kd_bytes(int tab_t) { return tab_t >= 0 ? ((((size_t)tab_t + 1) * 4 + 15) & ~(size_t)15) : 0; }
__host__ __device__ inline size_t band_warp_bytes(int tab_t, int64_t words)
{
    return 1024 + band_kd_bytes(tab_t) + (((size_t)words * 4 + 15) & ~(size_t)15);
}

struct BandRows {
    const u32* base;
    const int* rmap;
    __device__ __forceinline__ const u32* operator()(u64 c) const { return base + rmap[c]; }
};

template <typename CT>
struct BandText {
    const CT* p;
    __device__ __forceinline__ u64 operator[](int j) const { return (u64)__ldg(p + j); }
};

/* the query whose units hold unit t: the last j in [0, nq) with ustart[j] <= t (ustart
 * ascends and ustart[nq] > t), by the whole warp, 32 samples per round */
__device__ __forceinline__ int band_query_of(const BandQuery* bq, int nq, int t, int lane)
{
    int lo = 0, hi = nq;
    while (hi - lo > 1) {
        const int S = (hi - lo + 31) >> 5;
        const int k = lo + lane * S;
        const bool le = k < hi && __ldg(&bq[k].ustart) <= t;
        const int c = __popc(__ballot_sync(0xffffffffu, le)); /* sample 0 (lo) always passes */
        lo += (c - 1) * S;
        hi = lo + S < hi ? lo + S : hi;
    }
    return lo;
}

/* a pair's chain as the band kernel plans it: the cutoff of a normalized op from the
 * warp's table (Levenshtein: kd[n - m], kd[0] for every n <= m; the LCS families:
 * kd[n - m + tab_t / 2]), else from the double chain */
template <bool LCS>
__device__ __forceinline__ PairSpec band_pair_spec(const KParams& a, const u32* kd, int tab_t, int m, int n)
{
    PairSpec s;
    s.metric = a.metric;
    s.op = a.op;
    s.form = a.form;
    s.l1 = (u64)m;
    s.l2 = (u64)n;
    s.ci = a.ci;
    s.cf = a.cf;
    s.p = a.sp;
    if (tab_t >= 0) {
        if constexpr (LCS) {
            const int h = tab_t >> 1, jj = n - m + h;
            if (jj >= 0 && jj <= tab_t) {
                const u32 v = kd[jj];
                s.kd_pre = v == 0xffffffffu ? ~0ull : (u64)v;
            }
        }
        else {
            const int jj = n - m;
            if (jj <= tab_t) {
                const u32 v = kd[jj > 0 ? jj : 0];
                s.kd_pre = v == 0xffffffffu ? ~0ull : (u64)v;
            }
        }
    }
    return s;
}

/* a pair's result from the core's raw distance (Levenshtein, or for the LCS families
 * the Indel distance m + n - 2 LCS; any value > K when pruned) */
template <bool LCS>
__device__ __forceinline__ void band_store(const KParams& a, const PairSpec& s, const Plan& pl, i64 K, i64 raw,
                                           int m, int n, int64_t qi, int64_t ci, bool is_int)
{
    i64 vi = 0;
    double vf = 0.0;
    if (a.fast) vi = raw <= K ? raw : K + 1;
    else if constexpr (LCS) finish_int(s, pl, raw <= K ? ((i64)m + n - raw) >> 1 : -1, &vi, &vf); /* the LCS length, or -1 */
    else finish_int(s, pl, raw, &vi, &vf);
    store_result(a, qi, ci, vi, vf, is_int);
}

#ifndef RFG_BAND_MINB
#define RFG_BAND_MINB 3 /* CTAs of 256 threads per SM the register budget of bands up to 4 words is sized for (85 registers) */
#endif

template <typename CT, int B, bool LCS>
__global__ void __launch_bounds__(256, B <= 4 ? RFG_BAND_MINB : B <= 8 ? 2 : 1) k_band(const KParams a)
{
    extern __shared__ u64 smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tab_t = a.tab_t; /* cutoffs of n = m .. m + tab_t (LCS: m - tab_t/2 .. m + tab_t/2; -1: not used) */
    const int64_t words = a.scratch_per_thread; /* row words a slice holds */
    unsigned char* slice = (unsigned char*)smem + (size_t)warp * band_warp_bytes(tab_t, words);
    int* rmap = (int*)slice;
    u32* kd = (u32*)(slice + 1024);
    u32* rows = (u32*)(slice + 1024 + band_kd_bytes(tab_t));
    const BandQuery* bq = a.band_q;
    const int nq = a.nq;
    const int rounds = (int)a.chunk;
    const int nunits = (int)a.nchunks;
    const int fch = (int)((a.c.n + RFG_BAND_FILL - 1) / RFG_BAND_FILL);
    /* the host keeps units + fills below 2^31 */
    const int ntasks = nunits + nq * fch;
    const bool is_int = result_is_int(a.metric, a.op);
    const bool use_kd = tab_t >= 0;
    i64 rej_i;
    double rej_f;
    band_reject_value(a.metric, a.op, a.ci, a.fast, a.fast_k, &rej_i, &rej_f);
    int cur = -1, m = 0, S = 0;
    int64_t qi = 0;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(a.counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntasks) break;
        if (t >= nunits) {
            /* fill: the pairs outside [nlo, nhi] of 1024 choices of one row */
            const int f = t - nunits, j = f / fch;
            const int64_t c0 = (int64_t)(f - j * fch) * RFG_BAND_FILL;
            const int64_t c1 = c0 + RFG_BAND_FILL < a.c.n ? c0 + RFG_BAND_FILL : a.c.n;
            const int64_t nlo = __ldg(&bq[j].nlo), nhi = __ldg(&bq[j].nhi), fq = __ldg(&bq[j].qi);
            for (int64_t cc = c0; cc < c1; cc += 32) {
                const int64_t c = cc + lane;
                /* off has n + 1 entries: lanes up to c = n load, the last lane its successor */
                const int64_t o = c <= a.c.n ? __ldg(a.c.off + c) : 0;
                const int64_t nx = __shfl_down_sync(0xffffffffu, o, 1);
                const int64_t o1 = lane == 31 ? (c + 1 <= a.c.n ? __ldg(a.c.off + c + 1) : 0) : nx;
                const int64_t n = o1 - o;
                if (c < c1 && (n < nlo || n > nhi)) store_result(a, fq, c, rej_i, rej_f, is_int);
            }
            continue;
        }
        const int j = band_query_of(bq, nq, t, lane);
        if (j != cur) {
            /* this warp's table for query j */
            qi = __ldg(&bq[j].qi);
            const int64_t q0 = a.q.off[qi];
            m = (int)(a.q.off[qi + 1] - q0);
            S = band_row_stride(m, B);
            const unsigned char* qb = a.q.data + q0 * a.q.width;
            for (int i = lane; i < 256; i += 32) rmap[i] = 0;
            __syncwarp();
            for (int i = lane; i < m; i += 32) {
                const u64 c = load_unit(qb, a.q.width, i);
                if (c < 256) rmap[c] = 1;
            }
            __syncwarp();
            /* row ids in code-unit order (row 0 is the zero row) */
            int total = 0;
            for (int c0 = 0; c0 < 256; c0 += 32) {
                const bool present = rmap[c0 + lane] != 0;
                const unsigned bal = __ballot_sync(0xffffffffu, present);
                int id = present ? total + __popc(bal & ((1u << lane) - 1)) + 1 : 0;
                if ((int64_t)(id + 1) * S > words) id = 0; /* the host sized the slice too small */
                rmap[c0 + lane] = id * S + (B + 1);
                total += __popc(bal);
            }
            if ((int64_t)(total + 1) * S > words && lane == 0) atomicExch(a.err, 5);
            const int nrow = (int64_t)(total + 1) * S <= words ? (total + 1) * S : (int)words;
            for (int i = lane; i < nrow; i += 32) rows[i] = 0;
            __syncwarp();
            /* lanes holding one code unit in a 32-unit block find each other; the lowest
             * writes that word of the unit's row */
            for (int i0 = 0; i0 < m; i0 += 32) {
                const int i = i0 + lane;
                int r = -1;
                if (i < m) {
                    const u64 c = load_unit(qb, a.q.width, i);
                    if (c < 256) r = (int)c;
                }
                const unsigned same = __match_any_sync(0xffffffffu, r);
                if (r >= 0 && lane == __ffs(same) - 1 && rmap[r] != B + 1) rows[rmap[r] + (i0 >> 5)] = same;
            }
            if (use_kd) {
                PairSpec s;
                s.metric = a.metric;
                s.op = a.op;
                s.form = a.form;
                s.l1 = (u64)m;
                s.ci = a.ci;
                s.cf = a.cf;
                s.p = a.sp;
                const int j0 = LCS ? -(tab_t >> 1) : 0;
                for (int jj = lane; jj <= tab_t; jj += 32) {
                    s.l2 = (u64)(m + j0 + jj > 0 ? m + j0 + jj : 0);
                    const u64 v = chain_kd(s);
                    kd[jj] = v >= 0xffffffffull ? 0xffffffffu : (u32)v;
                }
            }
            __syncwarp();
            cur = j;
        }
        /* the unit: `rounds` groups of 32 consecutive pairs of the query, one pair per
         * lane; a group's lanes start together, step until every lane's pair has ended,
         * and then finish and store together (the per-pair plan and finish run with the
         * whole warp, not once for each block in which some lane's pair ends) */
        const int64_t phi = __ldg(&bq[j].phi);
        const int64_t u0 = __ldg(&bq[j].plo) + (int64_t)(t - __ldg(&bq[j].ustart)) * 32 * rounds;
        const BandRows pm{rows, rmap};
        for (int r = 0; r < rounds; ++r) {
            const int64_t g0 = u0 + (int64_t)r * 32;
            if (g0 >= phi) break;
            const int64_t p = g0 + lane;
            const bool mine = p < phi;
            int4 rec = make_int4(0, 0, 0, 0);
            if (mine) rec = __ldg(a.prec + p);
            const int n = rec.z;
            const BandText<CT> tx{(const CT*)a.c.data + (int64_t)(((uint64_t)(uint32_t)rec.y << 32) | (uint32_t)rec.x)};
            const PairSpec s = band_pair_spec<LCS>(a, kd, tab_t, m, n);
            Plan pl;
            i64 K;
            if (a.fast) K = a.fast_k;
            else {
                pl = plan_int(s);
                K = pl.run ? pl.K : -1;
            }
            const i64 diff = m > n ? m - n : n - m;
            const bool passes = mine && K >= 0 && m > 0 && n > 0 && K >= diff;
            const bool run = passes && K < m && band_bits((int)K, m - n) <= 32 * B;
            i64 raw = 0;
            if (passes && !run) { /* outside the class the host computed */
                atomicExch(a.err, 6);
                raw = K + 1;
            }
            else if (!passes && K >= 0)
                raw = m == 0 ? n : n == 0 ? m : K + 1;
            bool act = run;
            if constexpr (LCS) {
                LcsBandLane<B> L;
                if (run) lcs_band_init<B>(L, m, tx, n, (int)K);
                while (__any_sync(0xffffffffu, act))
                    if (act && lcs_band_run8<B>(L, pm, tx, &raw)) act = false;
            }
            else {
                BandLane<B> L;
                if (run) band_init<B>(L, m, tx, n, (int)K);
                while (__any_sync(0xffffffffu, act))
                    if (act && band_run8<B>(L, pm, tx, &raw)) act = false;
            }
            if (mine) band_store<LCS>(a, s, pl, K, raw, m, n, qi, rec.w, is_int);
        }
    }
}

} // namespace rfg
