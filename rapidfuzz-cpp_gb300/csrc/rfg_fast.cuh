/*
 * rfg_fast.cuh -- warp tiles for the unit-weight distances of one-word patterns:
 * Levenshtein 1/1/1, Indel and OSA with the chain d <= K ? d : K + 1 (cdist with a
 * distance cutoff, the reference's Cached*::distance over many choices,
 * Levenshtein.hpp:421-482, Indel.hpp:148-183, OSA.hpp:232-271).
 *
 * Every warp is its own worker: it pulls a task (a group of Q queries, one window of
 * choices) from the launch's counter, builds the group's pattern tables in its own
 * slice of shared memory, and for the window
 *   1. fills its result stage with K + 1, the value of every pair that fails the length
 *      filter |m - n| <= K (Levenshtein_impl.hpp:863, LCSseq_impl.hpp:389);
 *   2. finds, with two warp-wide votes, the visiting positions whose lengths can pass for
 *      some query of the group -- windows are sorted by choice length, so they form one
 *      run -- puts them through the length filter and the count filter
 *      (hist_lower_bound, below cutoffs where it can prune), and scores the survivors
 *      gathered 32 at a time, one choice per lane against the Q queries (fast_group);
 *   3. writes the window's Q result rows with 16-byte stores.
 * No barrier of the whole CTA is ever taken (only __syncwarp), so a warp that meets
 * short or quickly pruned choices moves on to the next task at once.
 *
 * Layout (per warp, in dynamic shared memory): Q pattern tables of 257 rows (code units
 * 0..255, then an all-zero row for units the patterns lack), 64-bit rows for patterns
 * of up to 64 units or 32-bit rows for patterns of up to 32 units (whose recurrence runs
 * on 32-bit words, the ALU width); then Q x window results, 16 bits wide when the cutoff
 * allows (every value of the chain is at most K + 1), converted to the output type when
 * the window's rows are written.
 */
#pragma once
#include "rfg_device.cuh"

namespace rfg {

#ifndef RFG_FAST_WARPS
#define RFG_FAST_WARPS 4 /* warps per CTA (the CTA only packs independent warps) */
#endif
/* CTAs per SM the register budget is sized for: as many as the shared memory of the
 * default 512-position window lets reside, at most 8 (64 registers; 7 for OSA on 64-bit
 * words, whose recurrence holds two more words a pattern) */
template <int FAM, int Q, bool HALF>
constexpr int fast_min_blocks()
{
    return (227 * 1024) / (RFG_FAST_WARPS * (Q * 257 * (HALF ? 4 : 8) + Q * 32 + Q * 512 * 2)) <
                   (FAM == FAM_OSA && !HALF ? 7 : 8)
               ? (227 * 1024) / (RFG_FAST_WARPS * (Q * 257 * (HALF ? 4 : 8) + Q * 32 + Q * 512 * 2))
               : (FAM == FAM_OSA && !HALF ? 7 : 8);
}

/* bytes of one warp's slice: tables, the patterns' count histograms (32 bytes each),
 * then the result stage (16-bit results when every value the chain can give, at most
 * K + 1, fits in 16 bits; else 32-bit) */
__host__ __device__ inline size_t fast_pm_bytes(int Q, bool half) { return ((size_t)Q * 257 * (half ? 4 : 8) + 15) / 16 * 16; }
__host__ __device__ inline size_t fast_hist_bytes(int Q) { return (size_t)Q * 32; }
__host__ __device__ inline size_t fast_stage_bytes(int Q, int64_t window, bool s16) { return (size_t)Q * window * (s16 ? 2 : 4); }
inline size_t fast_smem_bytes(int Q, bool half, int64_t window, bool s16)
{
    return (size_t)RFG_FAST_WARPS * (fast_pm_bytes(Q, half) + fast_hist_bytes(Q) + fast_stage_bytes(Q, window, s16));
}

/* the count histograms of the choices in visiting order, before the warp tiles of a
 * launch: 32 buckets of one byte, for choices of at most RFG_HIST_MAXLEN units (longer
 * choices get zeros and are never filtered).  One warp a choice: lanes holding units of
 * one bucket find each other and the lowest adds their number to the bucket's byte. */
#define RFG_HIST_WARPS 8
static __global__ void __launch_bounds__(RFG_HIST_WARPS * 32) k_fast_hist(const KParams a, uint4* out)
{
    __shared__ u32 cnt[RFG_HIST_WARPS][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char* b = (unsigned char*)cnt[warp];
    for (int64_t p = (int64_t)blockIdx.x * RFG_HIST_WARPS + warp; p < a.c.n; p += (int64_t)gridDim.x * RFG_HIST_WARPS) {
        if (lane < 8) cnt[warp][lane] = 0;
        __syncwarp();
        const int4 r = __ldg(a.prec + p);
        const int64_t o0 = (int64_t)(((uint64_t)(uint32_t)r.y << 32) | (uint32_t)r.x);
        if (r.z <= RFG_HIST_MAXLEN) {
            const unsigned char* cb = a.c.data + o0 * a.c.width;
            for (int i0 = 0; i0 < r.z; i0 += 32) {
                const int i = i0 + lane;
                const int bkt = i < r.z ? (int)(load_unit(cb, a.c.width, i) & 31) : -1;
                const unsigned same = __match_any_sync(0xffffffffu, bkt);
                if (bkt >= 0 && lane == __ffs(same) - 1) b[bkt] += (unsigned char)__popc(same);
                __syncwarp();
            }
        }
        if (lane < 2)
            out[2 * p + lane] = make_uint4(cnt[warp][4 * lane], cnt[warp][4 * lane + 1], cnt[warp][4 * lane + 2],
                                           cnt[warp][4 * lane + 3]);
        __syncwarp();
    }
}

template <typename WT>
struct FastRows {
    const WT* rows;
    __device__ __forceinline__ WT operator()(int q, unsigned c) const { return rows[q * 257 + c]; }
};

/* the position of the n-th (from 0) set bit of m (n < popc(m)) */
__device__ __forceinline__ int select_bit(unsigned m, int n)
{
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const int c = __popc(m & ((1u << w) - 1u));
        if (n >= c) {
            n -= c;
            m >>= w;
            pos += w;
        }
    }
    return pos;
}

/* first position p of [0, nn) with lens[4 p] >= L (lens ascending; nn <= 4096), by the
 * whole warp: one sampled length per lane narrows the answer to one run of
 * S = ceil(nn / 32) positions, which 32-position votes then search */
__device__ __forceinline__ int first_at_least(const int* lens, int nn, int64_t L, int lane)
{
    const int S = (nn + 31) >> 5; /* sample stride */
    const int ps = lane * S;
    const unsigned below = __ballot_sync(0xffffffffu, ps < nn && (int64_t)__ldg(lens + 4 * ps) < L);
    const int c = __popc(below); /* samples 0..c-1 lie below L */
    if (c == 0) return 0;
    const int base = (c - 1) * S + 1;              /* the answer is in [base, end] */
    const int end = c * S < nn ? c * S : nn;       /* sample c (if any) is not below L */
    for (int b = base; b < end; b += 32) {
        const int pq = b + lane;
        const unsigned b2 = __ballot_sync(0xffffffffu, pq < end && (int64_t)__ldg(lens + 4 * pq) < L);
        if (b2 != 0xffffffffu) return b + __popc(b2); /* the lengths below L are a prefix */
    }
    return end;
}

/* set (SET) or clear the table rows of pattern q: lane l holds units l and l + 32;
 * lanes holding one code unit find each other by match and the lowest of them writes
 * that 32-bit half of the row */
template <typename WT, bool SET>
__device__ __forceinline__ void fast_rows(WT* rows, int q, const KParams& a, int qi, int m, int lane)
{
    const unsigned char* qb = a.q.data + a.q.off[qi] * a.q.width;
#pragma unroll
    for (int h = 0; h < (sizeof(WT) == 4 ? 1 : 2); ++h) {
        const int i = lane + 32 * h;
        int r = 256;
        if (i < m) {
            const u64 c = load_unit(qb, a.q.width, i);
            if (c < 256) r = (int)c; /* a wider unit never occurs in one-byte choices */
        }
        if (SET) {
            const unsigned same = __match_any_sync(0xffffffffu, r);
            if (r < 256 && lane == __ffs(same) - 1) ((uint32_t*)&rows[q * 257 + r])[h] = same;
        }
        else if (r < 256)
            rows[q * 257 + r] = 0;
    }
}

template <int FAM, typename CT, int Q, bool HALF>
__global__ void __launch_bounds__(RFG_FAST_WARPS * 32, (fast_min_blocks<FAM, Q, HALF>())) k_fast(const KParams a)
{
    typedef typename std::conditional<HALF, uint32_t, u64>::type WT;
    extern __shared__ u64 smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int win = (int)a.stage; /* positions per window (a multiple of 8, at most 2048) */
    const int K = (int)(a.fast_k < 0x7fffffff ? a.fast_k : 0x7fffffff);
    const bool s16 = K < 0xffff;
    const size_t pmb = fast_pm_bytes(Q, HALF);
    unsigned char* slice = (unsigned char*)smem + (size_t)warp * (pmb + fast_hist_bytes(Q) + fast_stage_bytes(Q, win, s16));
    WT* rows = (WT*)slice;
    u32* qh = (u32*)(slice + pmb); /* pattern q's histogram: words 8q .. 8q + 7 */
    unsigned char* stage = slice + pmb + fast_hist_bytes(Q);
    /* the host keeps tasks and windows below 2^31 */
    const int nwin = (int)a.nchunks;
    const int ntasks = (int)(((int64_t)a.nq + Q - 1) / Q * nwin);
    const int maxm = HALF ? 32 : 64;

    int cur_g = -1;
    bool tab_ok = false; /* the rows hold the current group's patterns */
    int m[Q], qi[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) m[q] = qi[q] = 0;
    int qn = 0, mmin = 0, mmax = 0;
    __syncwarp();

    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(a.counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntasks) break;
        const int g = t / nwin, w = t - g * nwin;
        if (g != cur_g) {
            /* the group's pattern tables are built when its first survivors are scored
             * (most tasks of a pruning cutoff have none) */
            tab_ok = false;
            qn = 0;
            mmin = 0x7fffffff;
            mmax = 0;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const int kq = g * Q + q;
                m[q] = 0;
                if (kq < a.nq) {
                    qi[q] = a.qlist[kq];
                    int mq = (int)(a.q.off[qi[q] + 1] - a.q.off[qi[q]]);
                    if (mq > maxm) { /* the host classified this query into a smaller class */
                        if (lane == 0) atomicExch(a.err, 2);
                        mq = maxm;
                    }
                    m[q] = mq;
                    qn = q + 1;
                    mmin = mq < mmin ? mq : mmin;
                    mmax = mq > mmax ? mq : mmax;
                }
            }
            if (a.cfilter) {
                /* the group's count histograms: lanes holding units of one bucket find
                 * each other; the lowest adds their number to the bucket's byte */
                for (int i = lane; i < Q * 8; i += 32) qh[i] = 0;
                __syncwarp();
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if (q >= qn) break;
                    const unsigned char* qb = a.q.data + a.q.off[qi[q]] * a.q.width;
#pragma unroll
                    for (int h = 0; h < (HALF ? 1 : 2); ++h) {
                        const int i = lane + 32 * h;
                        const int bkt = i < m[q] ? (int)(load_unit(qb, a.q.width, i) & 31) : -1;
                        const unsigned same = __match_any_sync(0xffffffffu, bkt);
                        if (bkt >= 0 && lane == __ffs(same) - 1) ((unsigned char*)qh)[32 * q + bkt] += (unsigned char)__popc(same);
                        __syncwarp();
                    }
                }
            }
            __syncwarp();
            cur_g = g;
        }
        const int64_t p0 = (int64_t)w * win;
        const int nn = (int)(p0 + win < a.c.n ? win : a.c.n - p0);
        /* visiting positions [lo, hi) of the window whose lengths lie in
         * [mmin - K, mmax + K] (lengths ascend within a window) */
        const int* lens = (const int*)(a.prec + p0) + 2;
        const int lo = first_at_least(lens, nn, (int64_t)mmin - K, lane);
        const int hi = first_at_least(lens, nn, (int64_t)mmax + K + 1, lane);
        /* the stage holds K + 1 for every pair the filter rejects */
        {
            const unsigned v = K < 0x7fffffff ? (unsigned)K + 1 : (unsigned)K;
            const unsigned w2 = s16 ? v * 0x10001u : v;
            const int4 f = make_int4((int)w2, (int)w2, (int)w2, (int)w2);
            const int words = Q * win / (s16 ? 2 : 1); /* 32-bit words of the stage */
            for (int i = lane * 4; i < words; i += 128) *(int4*)((unsigned*)stage + i) = f;
        }
        __syncwarp();
        /* every visiting position goes through the length and count filters; the pairs
         * that survive wait in a lane each (position and skip mask) and are scored
         * together once up to 32 wait, so the recurrence runs with full warps rather
         * than for the one or two survivors of each 32 positions. */
        int pend = -1;          /* this lane's waiting position, or -1 */
        unsigned pend_skip = 0; /* its patterns whose bound exceeds K */
        auto run_pending = [&]() {
            if (!__any_sync(0xffffffffu, pend >= 0)) return;
            if (!tab_ok) {
                /* all rows zeroed (the previous group's units among them), then the
                 * group's patterns set */
                u64* z = (u64*)rows;
                for (int i = lane; i < (int)(Q * 257 * sizeof(WT) / 8); i += 32) z[i] = 0;
                __syncwarp();
#pragma unroll
                for (int q = 0; q < Q; ++q)
                    if (q < qn) fast_rows<WT, true>(rows, q, a, qi[q], m[q], lane);
                __syncwarp();
                tab_ok = true;
            }
            if (pend >= 0) {
                const int4 r = __ldg(a.prec + p0 + pend);
                const int64_t o0 = (int64_t)(((uint64_t)(uint32_t)r.y << 32) | (uint32_t)r.x);
                int d[Q];
                fast_group<FAM, Q, FastRows<WT>, MQText<CT>, WT>(FastRows<WT>{rows}, m, qn,
                                                                 MQText<CT>{(const CT*)a.c.data + o0}, r.z, K, d,
                                                                 pend_skip);
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if (q >= qn) break;
                    const int at = q * win + r.w;
                    if (s16) ((unsigned short*)stage)[at] = (unsigned short)d[q];
                    else ((unsigned*)stage)[at] = (unsigned)d[q];
                }
            }
            pend = -1;
        };
        /* the filter needs a position's length and histogram only; the next iteration's
         * are loaded before this one is filtered */
        const bool hf = a.cfilter != 0;
        int zn = 0;
        uint4 hn0 = make_uint4(0, 0, 0, 0), hn1 = hn0;
        if (lo + lane < hi) {
            zn = __ldg(&a.prec[p0 + lo + lane].z);
            if (hf) {
                hn0 = __ldg(a.chist + 2 * (p0 + lo + lane));
                hn1 = __ldg(a.chist + 2 * (p0 + lo + lane) + 1);
            }
        }
        for (int b0 = lo; b0 < hi; b0 += 32) {
            const int p = b0 + lane;
            const int z = zn;
            const uint4 h0 = hn0, h1 = hn1;
            if (p + 32 < hi) {
                zn = __ldg(&a.prec[p0 + p + 32].z);
                if (hf) {
                    hn0 = __ldg(a.chist + 2 * (p0 + p + 32));
                    hn1 = __ldg(a.chist + 2 * (p0 + p + 32) + 1);
                }
            }
            bool surv = false;
            unsigned skip = 0;
            if (p < hi) {
                /* patterns the length filter lets through, less those whose count bound
                 * exceeds K (they keep the stage's K + 1) */
                unsigned live = 0;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const int diff = m[q] > z ? m[q] - z : z - m[q];
                    if (q < qn && diff <= K) live |= 1u << q;
                }
                if (hf && live && z <= RFG_HIST_MAXLEN) {
                    const u32 hc[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
#pragma unroll
                    for (int q = 0; q < Q; ++q) {
                        if (!((live >> q) & 1u)) continue;
                        const uint4 g0 = *(const uint4*)(qh + 8 * q), g1 = *(const uint4*)(qh + 8 * q + 4);
                        const u32 hq[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
                        if (hist_lower_bound(FAM, hq, hc, m[q], z) > K) skip |= 1u << q;
                    }
                }
                surv = (live & ~skip) != 0;
            }
            const unsigned sm = __ballot_sync(0xffffffffu, surv);
            if (!sm) continue;
            unsigned idle = __ballot_sync(0xffffffffu, pend < 0);
            if (__popc(sm) > __popc(idle)) {
                run_pending();
                idle = 0xffffffffu;
            }
            /* the k-th survivor waits in the k-th idle lane */
            const int rank = __popc(idle & ((1u << lane) - 1));
            const bool take = ((idle >> lane) & 1u) && rank < __popc(sm);
            const int src = take ? select_bit(sm, rank) : lane;
            const int sp = __shfl_sync(0xffffffffu, p, src);
            const unsigned ss = __shfl_sync(0xffffffffu, skip, src);
            if (take) {
                pend = sp;
                pend_skip = ss;
            }
        }
        run_pending();
        __syncwarp();
        /* the window's rows, converted to the output type: 16-byte stores where the row
         * segment is aligned */
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            if (q >= qn) break;
            const int64_t base = (int64_t)qi[q] * a.ld + p0;
            const unsigned short* s1 = (const unsigned short*)stage + q * win;
            const unsigned* s2 = (const unsigned*)stage + q * win;
            if (a.out_dtype == 0) {
                int* dst = (int*)a.out + base;
                const int nv = a.vec ? nn & ~3 : 0;
                for (int i = lane * 4; i < nv; i += 128) {
                    int4 o;
                    if (s16) {
                        const uint2 u = *(const uint2*)(s1 + i);
                        o = make_int4((int)(u.x & 0xffff), (int)(u.x >> 16), (int)(u.y & 0xffff), (int)(u.y >> 16));
                    }
                    else
                        o = *(const int4*)(s2 + i);
                    *(int4*)(dst + i) = o;
                }
                for (int i = nv + lane; i < nn; i += 32) dst[i] = s16 ? (int)s1[i] : (int)s2[i];
            }
            else {
                long long* dst = (long long*)a.out + base;
                const bool dbl = a.out_dtype == 2;
                auto conv = [&](unsigned x) -> long long {
                    return dbl ? (long long)__double_as_longlong(int_result_as_double((i64)x)) : (long long)x;
                };
                const int nv = a.vec ? nn & ~1 : 0;
                for (int i = lane * 2; i < nv; i += 64) {
                    const unsigned x0 = s16 ? s1[i] : s2[i], x1 = s16 ? s1[i + 1] : s2[i + 1];
                    *(longlong2*)(dst + i) = make_longlong2(conv(x0), conv(x1));
                }
                for (int i = nv + lane; i < nn; i += 32) dst[i] = conv(s16 ? s1[i] : s2[i]);
            }
        }
        __syncwarp();
    }
}

} // namespace rfg
