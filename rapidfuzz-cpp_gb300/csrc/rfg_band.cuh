/*
 * rfg_band.cuh -- banded Levenshtein (weights 1/1/1) for queries whose every passing pair
 * needs a diagonal band narrower than the pattern: the reference's
 * levenshtein_hyrroe2003_small_band / the band of levenshtein_hyrroe2003_block
 * (Levenshtein_impl.hpp:419-505, 641-850), on Ukkonen's band of about K + 2 diagonals
 * (lev_band32), chosen when that band is narrower than the pattern for the largest bound
 * K any pair of the query can reach (the length filter Levenshtein_impl.hpp:863 caps it).
 *
 * A CTA takes (query, chunk of choices) tiles from the launch's counter; its warps take
 * runs of 32 length-ordered positions of the tile from a counter of the CTA and score one
 * pair per lane with lev_band32<B> on B 32-bit words (the kernel's registers are sized by
 * the band, not by the pattern's length).  Only a few pairs of a chunk pass the length
 * filter and those run hundreds of steps, so no barrier is taken between runs: a warp
 * whose pairs were rejected takes the next run at once.  Results are stored where they
 * belong.  Per query the CTA builds in shared memory
 *   - a compact pattern table: one row of ceil(m/32) 32-bit words for each code unit
 *     the query holds (plus the all-zero row), each row with zero words on either side
 *     so the band's window is loaded without range tests, and rmap[c] = the word offset
 *     of unit c's row;
 *   - for the normalized ops, the integer cutoff chain_kd of every choice length up to
 *     tab_t (32-bit; 0xffffffff: none), so no pair evaluates the double-precision chain
 *     to find its bound.
 * One-byte choices only (a wider unit has no row: the zero row would do, but the host
 * keeps wide alphabets on the general kernels).
 */
#pragma once
#include "rfg_device.cuh"

namespace rfg {

/* words of one compact row for a class of queries of at most m units and band B: the
 * pattern's words, B + 1 zero words before and 2B + 2 after (the window of a pair with
 * n up to m + K reads that far past the pattern's last word) */
__host__ __device__ inline int band_row_stride(int m, int B) { return (m + 31) / 32 + 3 * (B + 1); }

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

/* shared-memory bytes of a band launch: kd table, rmap, rows */
inline size_t band_smem_bytes(int tab_t, int rows, int stride)
{
    const size_t kd = tab_t >= 0 ? ((size_t)tab_t + 1) * 4 : 0;
    const size_t head = (kd + 1024 + 15) / 16 * 16;
    return head + ((size_t)rows * stride * 4 + 15) / 16 * 16;
}

template <typename CT, int B>
__global__ void __launch_bounds__(256, B <= 4 ? 4 : B <= 8 ? 2 : 1) k_band(const KParams a)
{
    extern __shared__ u64 smem[];
    const int tab_t = a.tab_t;          /* kd covers choice lengths 0..tab_t (-1: not used) */
    const int R = (int)a.scratch_per_thread; /* rows the table holds (the class maximum) */
    const int S = a.wmax;               /* words per row */
    u32* kd = (u32*)smem;
    const size_t kdb = tab_t >= 0 ? ((size_t)tab_t + 1) * 4 : 0;
    int* rmap = (int*)((unsigned char*)smem + kdb);
    u32* rows = (u32*)((unsigned char*)smem + (kdb + 1024 + 15) / 16 * 16);
    __shared__ int64_t s_tile;
    __shared__ int s_sub;
    __shared__ int s_warp_cnt[8];
    int64_t cur_q = -1;
    int m = 0;
    const int64_t ntiles = (int64_t)a.nq * a.nchunks;
    const bool is_int = result_is_int(a.metric, a.op);
    const bool use_kd = tab_t >= 0;
    for (;;) {
        if (threadIdx.x == 0) {
            s_tile = atomicAdd(a.counter, 1);
            s_sub = 0;
        }
        __syncthreads();
        const int64_t t = s_tile;
        if (t >= ntiles) break;
        const int64_t qi = a.qlist[t / a.nchunks];
        const int64_t ch = t % a.nchunks;
        if (qi != cur_q) {
            const int64_t q0 = a.q.off[qi];
            m = (int)(a.q.off[qi + 1] - q0);
            const unsigned char* qb = a.q.data + q0 * a.q.width;
            /* which code units below 256 the query holds */
            for (int i = threadIdx.x; i < 256; i += blockDim.x) rmap[i] = 0;
            __syncthreads();
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                const u64 c = load_unit(qb, a.q.width, i);
                if (c < 256) rmap[c] = 1;
            }
            __syncthreads();
            /* row ids in code-unit order: a CTA-wide exclusive count of the present units
             * (row 0 is the zero row) */
            const int c = threadIdx.x; /* blockDim.x == 256: one code unit per thread */
            const bool present = rmap[c] != 0;
            const unsigned bal = __ballot_sync(0xffffffffu, present);
            const int lane = c & 31, wid = c >> 5;
            if (lane == 0) s_warp_cnt[wid] = __popc(bal);
            __syncthreads();
            int before = 0;
            for (int w = 0; w < wid; ++w) before += s_warp_cnt[w];
            const int id = present ? before + __popc(bal & ((1u << lane) - 1)) + 1 : 0;
            int total = 0;
            for (int w = 0; w < 8; ++w) total += s_warp_cnt[w];
            if (total + 1 > R && threadIdx.x == 0) atomicExch(a.err, 5); /* the host sized the table too small */
            __syncthreads();
            rmap[c] = (id < R ? id : 0) * S + (B + 1);
            for (int i = threadIdx.x; i < R * S; i += blockDim.x) rows[i] = 0;
            __syncthreads();
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                const u64 cu = load_unit(qb, a.q.width, i);
                if (cu < 256) atomicOr(&rows[rmap[cu] + (i >> 5)], 1u << (i & 31));
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
                for (int n = threadIdx.x; n <= tab_t; n += blockDim.x) {
                    s.l2 = (u64)n;
                    const u64 v = chain_kd(s);
                    kd[n] = v >= 0xffffffffull ? 0xffffffffu : (u32)v;
                }
            }
            __syncthreads();
            cur_q = qi;
        }
        /* the tile's positions go out in runs of 32 that warps take from a counter of
         * the CTA: a warp that meets pairs the length filter rejects moves on at once,
         * and the CTA waits for its slowest warp only at the end of the tile */
        const int64_t c0 = ch * a.chunk;
        const int64_t c1 = c0 + a.chunk < a.c.n ? c0 + a.chunk : a.c.n;
        const int nsub = (int)((c1 - c0 + 31) / 32);
        const BandRows pm{rows, rmap};
        const int lane = threadIdx.x & 31;
        for (;;) {
            int sub = 0;
            if (lane == 0) sub = atomicAdd(&s_sub, 1);
            sub = __shfl_sync(0xffffffffu, sub, 0);
            if (sub >= nsub) break;
            const int64_t p = c0 + (int64_t)sub * 32 + lane;
            if (p < c1) {
                const int64_t ci = __ldg(a.perm + p);
                const int64_t o0 = __ldg(a.poff + p);
                const int n = __ldg(a.plen + p);
                PairSpec s;
                s.metric = a.metric;
                s.op = a.op;
                s.form = a.form;
                s.l1 = (u64)m;
                s.l2 = (u64)n;
                s.ci = a.ci;
                s.cf = a.cf;
                s.p = a.sp;
                i64 vi = 0;
                double vf = 0.0;
                i64 K;
                Plan pl;
                if (a.fast) K = a.fast_k;
                else {
                    if (use_kd && n <= tab_t) s.kd_pre = kd[n] == 0xffffffffu ? ~0ull : (u64)kd[n];
                    pl = plan_int(s);
                    K = pl.run ? pl.K : -1;
                }
                i64 raw = 0;
                if (K >= 0) {
                    const i64 diff = m > n ? m - n : n - m;
                    if (m == 0) raw = n;
                    else if (K < diff) raw = K + 1;
                    else if (n == 0) raw = m;
                    else if (K >= m || band_bits((int)K, m - n) > 32 * B) { /* outside the class the host computed */
                        atomicExch(a.err, 6);
                        raw = K + 1;
                    }
                    else
                        raw = lev_band32<B>(pm, m, BandText<CT>{(const CT*)a.c.data + o0}, n, (int)K);
                }
                if (a.fast) {
                    vi = raw <= K ? raw : K + 1;
                    vf = 0.0;
                }
                else
                    finish_int(s, pl, raw, &vi, &vf);
                store_result(a, qi, ci, vi, vf, is_int);
            }
        }
        __syncthreads();
    }
}

} // namespace rfg
