/*
 * rfg_core.cuh -- bit-parallel scorer cores and the reference's formula chains.
 *
 * Every device result of this library is "formula chain over an exact integer":
 *   Levenshtein    exact (weighted) distance        rapidfuzz/distance/Levenshtein_impl.hpp:1056-1089
 *   Indel/LCSseq   exact LCS length                 rapidfuzz/distance/LCSseq_impl.hpp:205-403
 *   OSA            exact OSA distance               rapidfuzz/distance/OSA_impl.hpp:34-273
 *   Jaro / JW      common chars + transpositions    rapidfuzz/distance/Jaro_impl.hpp:94-454
 * The chains (distance <-> similarity <-> normalized, cutoff translation) follow
 * rapidfuzz/details/distance.hpp literally, so integers are bit-exact and doubles are
 * bit-identical: every double operation below is an explicit round-to-nearest
 * operation (no FMA contraction on the device).
 *
 * A core may stop early once the value it computes is known to exceed the pruning bound
 * K it was given; it then returns any value > K.  The chains only ever look at
 * "d <= K ? d : K+1", so pruning never changes a result.
 *
 * Early stop bound (all distance-type cores): after column j of an m x n DP, every
 * alignment path crosses column j at some row i and still needs |(m-i)-(n-j)| unit
 * operations, so dist >= min_i D[i][j] + |(m-i)-(n-j)|.  Because neighbouring cells of
 * a column differ by at most 1, that minimum sits at the row i* = m-n+j on the diagonal
 * through (m, n) (clamped to row 0, where it equals n-m).  D[i*][j] is j plus the
 * masked popcounts of the vertical-delta vectors, so the bound costs a few popcounts.
 * The same identity gives the final distance: D[m][n] = n + popc(VP) - popc(VN) over the
 * m pattern bits, so no per-character score tracking is needed.
 *
 * This header compiles for the device (nvcc) and, for the CPU self-checks of the
 * algorithms, for the host as well.
 */
#pragma once
#include <stdint.h>

#include <type_traits>

#ifdef __CUDACC__
#define RFG_HD __host__ __device__ __forceinline__
/* double-precision tails of the chains: kept out of line so the integer launches never
 * evaluate them speculatively (the FP64 pipe is a small fraction of the INT32 rate) */
#define RFG_COLD static __host__ __device__ __noinline__
/* large device routines called from several places: one out-of-line copy each */
#define RFG_NOINL __host__ __device__ __noinline__
#else
#define RFG_HD inline
#define RFG_COLD static inline
#define RFG_NOINL inline
#endif

namespace rfg {

typedef uint64_t u64;
typedef int64_t i64;
typedef uint32_t u32;

/* ---------------------------------------------------------------- bit helpers */

RFG_HD int popc64(u64 x)
{
#ifdef __CUDA_ARCH__
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}

RFG_HD int ctz64(u64 x)
{
#ifdef __CUDA_ARCH__
    return __ffsll((long long)x) - 1;
#else
    return __builtin_ctzll(x);
#endif
}

RFG_HD u64 blsi(u64 x) { return x & (0ull - x); }
RFG_HD u64 blsr(u64 x) { return x & (x - 1); }
/* bits [0, n), n in [0, 64] */
RFG_HD u64 low_mask(int n) { return n >= 64 ? ~0ull : ((1ull << n) - 1); }
/* bits [a, b] of a 64-bit word, clipped to [0, 63]; empty when b < a */
RFG_HD u64 range_mask(int a, int b)
{
    if (a < 0) a = 0;
    if (b > 63) b = 63;
    if (b < a) return 0;
    return low_mask(b + 1) & ~low_mask(a);
}

/* a + b + carry_in over 64 bits, carry out */
RFG_HD u64 add_carry(u64 a, u64 b, u32 cin, u32* cout)
{
#ifdef __CUDA_ARCH__
    u32 al = (u32)a, ah = (u32)(a >> 32), bl = (u32)b, bh = (u32)(b >> 32);
    u32 rl, rh, c;
    asm("add.cc.u32 %0, %4, %5;\n\t"
        "addc.cc.u32 %1, %6, %7;\n\t"
        "addc.u32 %2, 0, 0;\n\t"
        : "=r"(rl), "=r"(rh), "=r"(c)
        : "r"(0), "r"(al), "r"(bl), "r"(ah), "r"(bh));
    /* add the incoming carry separately: (a+b) + cin can carry only when a+b == ~0 */
    u64 r = ((u64)rh << 32) | rl;
    u64 r2 = r + cin;
    *cout = c | (u32)(r2 < r);
    return r2;
#else
    u64 r = a + b;
    u32 c1 = r < a;
    u64 r2 = r + cin;
    u32 c2 = r2 < r;
    *cout = c1 | c2;
    return r2;
#endif
}

/* -------------------------------------------------------------- exact doubles */

/* |x| <= lim for lim >= 0 on the bit patterns (no FP64 instruction; NaN compares false):
 * non-negative doubles order like their bit patterns */
RFG_HD bool abs_le_bits(double x, double lim)
{
#ifdef __CUDA_ARCH__
    const u64 bx = (u64)__double_as_longlong(x), bl = (u64)__double_as_longlong(lim);
#else
    u64 bx, bl;
    __builtin_memcpy(&bx, &x, 8);
    __builtin_memcpy(&bl, &lim, 8);
#endif
    return (bx & 0x7fffffffffffffffull) <= bl;
}

RFG_HD double dadd(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
RFG_HD double dsub(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
RFG_HD double dmul(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
RFG_HD double ddiv(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
RFG_HD double dceil(double x)
{
#ifdef __CUDA_ARCH__
    return ceil(x);
#else
    return __builtin_ceil(x);
#endif
}
/* std::min / std::max semantics (first argument kept on ties) */
RFG_HD double dmin(double a, double b) { return (b < a) ? b : a; }
RFG_HD double dmax(double a, double b) { return (a < b) ? b : a; }

/* ----------------------------------------------------------- metric/op enums */

enum Metric {
    LEVENSHTEIN = 0,
    INDEL = 1,
    LCSSEQ = 2,
    OSA = 3,
    JARO = 4,
    JARO_WINKLER = 5,
    RATIO = 6,
    PARTIAL_RATIO = 7,
    TOKEN_SORT_RATIO = 8,
    PARTIAL_TOKEN_SORT_RATIO = 9,
    QRATIO = 10,
    TOKEN_SET_RATIO = 11,
    PARTIAL_TOKEN_SET_RATIO = 12,
    TOKEN_RATIO = 13,
    PARTIAL_TOKEN_RATIO = 14,
    WRATIO = 15
};
enum Op { DISTANCE = 0, SIMILARITY = 1, NORM_DISTANCE = 2, NORM_SIMILARITY = 3 };
enum Form { FORM_FREE = 0, FORM_CACHED = 1, FORM_MULTI = 2 };

/* bit-parallel core family a (metric, weights) pair runs on */
enum Family { FAM_LEV = 0, FAM_LCS = 1, FAM_OSA = 2, FAM_JARO = 3, FAM_WF = 4, FAM_NONE = 5, FAM_PARTIAL = 6, FAM_TOKEN = 7 };

struct ScoreParams {
    i64 ins, del, rep;     /* Levenshtein weights */
    double prefix_weight;  /* Jaro-Winkler */
};

/* ======================================================== single-word cores
 * PM: pattern-match table of s1 (pm(c) = bit i set when s1[i] == c), pattern length
 * m in 1..64.  TXT: t[j] yields the j-th code unit of s2.  K: pruning bound. */

/* The single-word cores fetch the text eight characters at a time: the eight loads and
 * pattern-row lookups are independent of each other and of the recurrence, so their
 * latencies overlap.  The lower-bound check runs every 8th character. */
#ifndef RFG_FETCH
#define RFG_FETCH 8
#endif

/* Hyyro 2003 (Levenshtein_impl.hpp:259-322) */
template <typename PMF, typename TXT>
RFG_HD i64 lev_word(const PMF& pm, int m, const TXT& t, int n, i64 K)
{
    u64 VP = ~0ull, VN = 0;
    const bool check = K < (i64)(m > n ? m : n);
    /* full blocks of RFG_FETCH units without per-unit bounds tests, then the tail;
     * returns true once the bound is passed */
    auto block = [&](int j0, auto full) -> bool {
        constexpr bool FULL = decltype(full)::value;
        u64 Xb[RFG_FETCH];
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) Xb[k] = (FULL || j0 + k < n) ? pm(t[j0 + k]) : 0;
        const int kn = FULL ? RFG_FETCH : n - j0;
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) {
            if (FULL || k < kn) {
                const u64 X = Xb[k];
                const u64 D0 = (((X & VP) + VP) ^ VP) | X | VN;
                u64 HP = VN | ~(D0 | VP);
                u64 HN = D0 & VP;
                HP = (HP << 1) | 1;
                HN = HN << 1;
                VP = HN | ~(D0 | HP);
                VN = HP & D0;
            }
        }
        if (FULL && check && ((j0 + RFG_FETCH) & 7) == 0) {
            const int jj = j0 + RFG_FETCH, is = m - n + jj;
            if (is >= 0) {
                const u64 lm = low_mask(is);
                const i64 lb = (i64)jj + popc64(VP & lm) - popc64(VN & lm);
                if (lb > K) return true;
            }
        }
        return false;
    };
    int j0 = 0;
    for (; j0 + RFG_FETCH <= n; j0 += RFG_FETCH)
        if (block(j0, std::integral_constant<bool, true>())) return K + 1;
    if (j0 < n) block(j0, std::integral_constant<bool, false>());
    const u64 mm = low_mask(m);
    return (i64)n + popc64(VP & mm) - popc64(VN & mm);
}

/* Hyyro 2004 LCS (LCSseq_impl.hpp:205-260).  Kd bounds the Indel distance m+n-2*LCS;
 * returns the exact LCS, or -1 once the Indel distance is known to exceed Kd. */
template <typename PMF, typename TXT>
RFG_HD i64 lcs_word(const PMF& pm, int m, const TXT& t, int n, i64 Kd)
{
    u64 S = ~0ull;
    const bool check = Kd < (i64)(m + n);
    /* full blocks of RFG_FETCH units without per-unit bounds tests, then the tail;
     * returns true once the bound is passed */
    auto block = [&](int j0, auto full) -> bool {
        constexpr bool FULL = decltype(full)::value;
        u64 Xb[RFG_FETCH];
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) Xb[k] = (FULL || j0 + k < n) ? pm(t[j0 + k]) : 0;
        const int kn = FULL ? RFG_FETCH : n - j0;
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) {
            if (FULL || k < kn) {
                const u64 u = S & Xb[k];
                S = (S + u) | (S - u);
            }
        }
        if (FULL && check && ((j0 + RFG_FETCH) & 7) == 0) {
            const int jj = j0 + RFG_FETCH, is = m - n + jj;
            if (is >= 0) {
                const i64 lcs_is = popc64(~S & low_mask(is));
                if ((i64)is + jj - 2 * lcs_is > Kd) return true;
            }
        }
        return false;
    };
    int j0 = 0;
    for (; j0 + RFG_FETCH <= n; j0 += RFG_FETCH)
        if (block(j0, std::integral_constant<bool, true>())) return -1;
    if (j0 < n) block(j0, std::integral_constant<bool, false>());
    return popc64(~S & low_mask(m));
}

/* Hyyro 2003 with the transposition term (OSA_impl.hpp:34-74) */
template <typename PMF, typename TXT>
RFG_HD i64 osa_word(const PMF& pm, int m, const TXT& t, int n, i64 K)
{
    u64 VP = ~0ull, VN = 0, D0 = 0, PMold = 0;
    const bool check = K < (i64)(m > n ? m : n);
    /* full blocks of RFG_FETCH units without per-unit bounds tests, then the tail;
     * returns true once the bound is passed */
    auto block = [&](int j0, auto full) -> bool {
        constexpr bool FULL = decltype(full)::value;
        u64 Xb[RFG_FETCH];
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) Xb[k] = (FULL || j0 + k < n) ? pm(t[j0 + k]) : 0;
        const int kn = FULL ? RFG_FETCH : n - j0;
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) {
            if (FULL || k < kn) {
                const u64 X = Xb[k];
                const u64 TR = (((~D0) & X) << 1) & PMold;
                D0 = (((X & VP) + VP) ^ VP) | X | VN | TR;
                u64 HP = VN | ~(D0 | VP);
                u64 HN = D0 & VP;
                HP = (HP << 1) | 1;
                HN = HN << 1;
                VP = HN | ~(D0 | HP);
                VN = HP & D0;
                PMold = X;
            }
        }
        if (FULL && check && ((j0 + RFG_FETCH) & 7) == 0) {
            const int jj = j0 + RFG_FETCH, is = m - n + jj;
            if (is >= 0) {
                const u64 lm = low_mask(is);
                const i64 lb = (i64)jj + popc64(VP & lm) - popc64(VN & lm);
                if (lb > K) return true;
            }
        }
        return false;
    };
    int j0 = 0;
    for (; j0 + RFG_FETCH <= n; j0 += RFG_FETCH)
        if (block(j0, std::integral_constant<bool, true>())) return K + 1;
    if (j0 < n) block(j0, std::integral_constant<bool, false>());
    const u64 mm = low_mask(m);
    return (i64)n + popc64(VP & mm) - popc64(VN & mm);
}

/* Q one-word patterns against one text, sharing each fetched block of text units:
 * for pattern q (q < qn) the unit-weight distance chain d <= K[q] ? d : K[q] + 1 of
 * Levenshtein / OSA (lev_word / osa_word) or Indel (lcs_word, d = m + n - 2 LCS),
 * with the same length filter, empty-string rules and lower-bound exits as those cores
 * behind the tile kernel's fast path, so every d equals the single-pair result.
 * pm(q, c): pattern-match word of pattern q for the table row c of a text unit (t[j]
 * gives rows, at most 256); m[q] <= 64. */
template <int FAM, int Q, typename PMQ, typename TXT, typename WT = u64>
RFG_HD void group_word_dist(const PMQ& pm, const int* m, int qn, const TXT& t, int n, const i64* Kq, i64* d)
{
    /* WT: the recurrence word, 64 bits, or 32 when every pattern has at most 32 units (the
     * GPU's ALU is 32 bits wide: half the instructions per step) */
    WT A[Q], B[Q], D0[Q], PO[Q]; /* Lev / OSA: VP, VN, D0, previous X; Indel: S in A */
    unsigned live = 0, chk = 0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        A[q] = (WT)~(WT)0;
        B[q] = D0[q] = PO[q] = 0;
        d[q] = 0;
        if (q >= qn) continue;
        const int mq = m[q];
        const i64 K = Kq[q];
        const i64 diff = mq > n ? mq - n : n - mq;
        if (FAM == FAM_LCS) {
            if (mq == 0 || n == 0) d[q] = (i64)mq + n;
            else if (K < diff) d[q] = K + 1;
            else {
                live |= 1u << q;
                if (K < (i64)mq + n) chk |= 1u << q;
            }
        }
        else {
            if (mq == 0) d[q] = n;
            else if (K < diff) d[q] = K + 1;
            else if (n == 0) d[q] = mq;
            else {
                live |= 1u << q;
                if (K < (i64)(mq > n ? mq : n)) chk |= 1u << q;
            }
        }
    }
    /* blocks of RFG_FETCH units: full blocks without per-unit bounds tests, then the tail */
    auto block = [&](int j0, auto full) {
        constexpr bool FULL = decltype(full)::value;
        unsigned c[RFG_FETCH]; /* the table row of each unit (at most 256) */
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) c[k] = (FULL || j0 + k < n) ? (unsigned)t[j0 + k] : 0u;
        const int kn = FULL ? RFG_FETCH : n - j0;
        const bool at_check = FULL && ((j0 + RFG_FETCH) & 7) == 0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            if (!((live >> q) & 1u)) continue;
#pragma unroll
            for (int k = 0; k < RFG_FETCH; ++k) {
                if (FULL || k < kn) {
                    const WT X = (WT)pm(q, c[k]);
                    if (FAM == FAM_LCS) {
                        const WT u = A[q] & X;
                        A[q] = (WT)(A[q] + u) | (WT)(A[q] - u);
                    }
                    else {
                        const WT VP = A[q], VN = B[q];
                        WT D = (WT)((WT)((X & VP) + VP) ^ VP) | X | VN;
                        if (FAM == FAM_OSA) {
                            D |= (WT)(((WT)~D0[q] & X) << 1) & PO[q];
                            D0[q] = D;
                            PO[q] = X;
                        }
                        WT HP = VN | (WT)~(D | VP);
                        WT HN = D & VP;
                        HP = (WT)(HP << 1) | (WT)1;
                        HN = (WT)(HN << 1);
                        A[q] = HN | (WT)~(D | HP);
                        B[q] = HP & D;
                    }
                }
            }
            if (at_check && ((chk >> q) & 1u)) {
                const i64 K = Kq[q];
                const int jj = j0 + RFG_FETCH, is = m[q] - n + jj;
                if (is >= 0) {
                    const WT lm = (WT)low_mask(is);
                    const bool out = FAM == FAM_LCS
                                         ? (i64)is + jj - 2 * (i64)popc64((u64)(WT)(~A[q] & lm)) > K
                                         : (i64)jj + popc64((u64)(A[q] & lm)) - popc64((u64)(B[q] & lm)) > K;
                    if (out) {
                        d[q] = K + 1;
                        live &= ~(1u << q);
                    }
                }
            }
        }
    };
    int j0 = 0;
    for (; j0 + RFG_FETCH <= n && live; j0 += RFG_FETCH) block(j0, std::integral_constant<bool, true>());
    if (j0 < n && live) block(j0, std::integral_constant<bool, false>());
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if ((live >> q) & 1u) {
            const WT mm = (WT)low_mask(m[q]);
            d[q] = FAM == FAM_LCS ? (i64)m[q] + n - 2 * (i64)popc64((u64)(WT)(~A[q] & mm))
                                  : (i64)n + popc64((u64)(A[q] & mm)) - popc64((u64)(B[q] & mm));
        }
        d[q] = d[q] <= Kq[q] ? d[q] : Kq[q] + 1;
    }
}

/* popcount of a recurrence word (one POPC for 32-bit words) */
RFG_HD int popc_w(u64 x) { return popc64(x); }
RFG_HD int popc_w(u32 x)
{
#ifdef __CUDA_ARCH__
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}

/* Count filter of the distance fast path.  A string's code units counted in 32 buckets
 * (unit & 31), one byte each, four to a 32-bit word (strings of at most 255 units).
 * Indel distance >= sum_b |cnt_a(b) - cnt_b(b)| (an insertion or a deletion changes one
 * count by one); Levenshtein and OSA distance >= (that sum + |m - n|) / 2 (a substitution
 * moves one unit between two counts, an insertion or deletion changes one count, a
 * transposition none: the units a must lose and gain are each at most d).  Merging units
 * into buckets only lowers the sum, so the bound holds for any code units.  A pair whose
 * bound exceeds the cutoff K has distance > K: the chain's value is K + 1, as the
 * recurrence would give. */
#define RFG_HIST_MAXLEN 255

RFG_HD u32 sad4(u32 a, u32 b)
{
#ifdef __CUDA_ARCH__
    return __vsadu4(a, b);
#else
    u32 s = 0;
    for (int k = 0; k < 4; ++k) {
        const int x = (int)((a >> (8 * k)) & 0xffu), y = (int)((b >> (8 * k)) & 0xffu);
        s += (u32)(x > y ? x - y : y - x);
    }
    return s;
#endif
}

RFG_HD int hist_lower_bound(int fam, const u32* ha, const u32* hb, int m, int n)
{
    int s = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) s += (int)sad4(ha[w], hb[w]);
    return fam == FAM_LCS ? s : (s + (m > n ? m - n : n - m)) >> 1;
}

/* The unit-weight distance chain d <= K ? d : K + 1 of Q one-word patterns against one
 * text, for the warp tiles of the distance fast path: Levenshtein 1/1/1 (Hyyro 2003,
 * Levenshtein_impl.hpp:259-322), OSA (OSA_impl.hpp:34-74) or Indel (d = m + n - 2 LCS,
 * LCSseq_impl.hpp:205-260), with the length filter and empty-string rules of those
 * functions (Levenshtein_impl.hpp:863, LCSseq_impl.hpp:389) and the diagonal lower-bound
 * exit every 8 text units, so every d equals the single-pair result; patterns in `skip`
 * (their count bound exceeds K: hist_lower_bound) take K + 1 without running.  Lengths and K are
 * below 2^31 (int bookkeeping: every 64-bit integer operation costs two ALU instructions
 * on the GPU).  pm(q, c): pattern word of pattern q for table row c (t[j] gives rows);
 * m[q] <= bits of WT.  The LCS step S' = (S + u) | (S - u) with u = S & X is written as
 * (S + u) | (S & ~X): u is a subset of S, so S - u = S & ~X, which a single three-input
 * logic instruction merges with the OR. */
template <int FAM, int Q, typename PMQ, typename TXT, typename WT>
RFG_HD void fast_group(const PMQ& pm, const int* m, int qn, const TXT& t, int n, int K, int* d, unsigned skip = 0)
{
    WT A[Q], B[Q], D0[Q], PO[Q]; /* Lev / OSA: VP, VN, D0, previous X; Indel: S in A */
    unsigned live = 0, chk = 0; /* chk: the cutoff is below the largest possible distance */
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        A[q] = (WT)~(WT)0;
        B[q] = D0[q] = PO[q] = 0;
        d[q] = 0;
        if (q >= qn) continue;
        const int mq = m[q];
        const int diff = mq > n ? mq - n : n - mq;
        if (FAM == FAM_LCS) {
            if (mq == 0 || n == 0) d[q] = mq + n;
            else if (K < diff || ((skip >> q) & 1u)) d[q] = K + 1;
            else {
                live |= 1u << q;
                if (K < mq + n) chk |= 1u << q;
            }
        }
        else {
            if (mq == 0) d[q] = n;
            else if (K < diff) d[q] = K + 1;
            else if (n == 0) d[q] = mq;
            else if ((skip >> q) & 1u) d[q] = K + 1;
            else {
                live |= 1u << q;
                if (K < (mq > n ? mq : n)) chk |= 1u << q;
            }
        }
    }
    auto block = [&](int j0, auto full) {
        constexpr bool FULL = decltype(full)::value;
        unsigned c[RFG_FETCH];
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) c[k] = (FULL || j0 + k < n) ? (unsigned)t[j0 + k] : 0u;
        const int kn = FULL ? RFG_FETCH : n - j0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            if (!((live >> q) & 1u)) continue;
#pragma unroll
            for (int k = 0; k < RFG_FETCH; ++k) {
                if (FULL || k < kn) {
                    const WT X = (WT)pm(q, c[k]);
                    if (FAM == FAM_LCS) {
                        const WT S = A[q];
                        A[q] = (WT)(S + (WT)(S & X)) | (WT)(S & (WT)~X);
                    }
                    else {
                        const WT VP = A[q], VN = B[q];
                        WT D = (WT)((WT)((X & VP) + VP) ^ VP) | X | VN;
                        if (FAM == FAM_OSA) {
                            D |= (WT)(((WT)~D0[q] & X) << 1) & PO[q];
                            D0[q] = D;
                            PO[q] = X;
                        }
                        WT HP = VN | (WT)~(D | VP);
                        const WT HN = D & VP;
                        HP = (WT)(HP << 1) | (WT)1;
                        const WT HNs = (WT)(HN << 1);
                        A[q] = HNs | (WT)~(D | HP);
                        B[q] = HP & D;
                    }
                }
            }
            if (FULL && ((chk >> q) & 1u)) {
                /* lower bound at column jj on the diagonal through (m, n) */
                const int jj = j0 + RFG_FETCH, is = m[q] - n + jj;
                if (is >= 0) {
                    const WT lm = (WT)low_mask(is);
                    const int lb = FAM == FAM_LCS ? is + jj - 2 * popc_w((WT)(~A[q] & lm))
                                                  : jj + popc_w((WT)(A[q] & lm)) - popc_w((WT)(B[q] & lm));
                    if (lb > K) {
                        d[q] = K + 1;
                        live &= ~(1u << q);
                    }
                }
            }
        }
    };
    int j0 = 0;
    for (; j0 + RFG_FETCH <= n && live; j0 += RFG_FETCH) block(j0, std::integral_constant<bool, true>());
    if (j0 < n && live) block(j0, std::integral_constant<bool, false>());
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if ((live >> q) & 1u) {
            const WT mm = (WT)low_mask(m[q]);
            d[q] = FAM == FAM_LCS ? m[q] + n - 2 * popc_w((WT)(~A[q] & mm))
                                  : n + popc_w((WT)(A[q] & mm)) - popc_w((WT)(B[q] & mm));
        }
        d[q] = d[q] <= K ? d[q] : K + 1;
    }
}

/* Jaro flagging, P (= s1) 1..64 chars, effective text length <= 64
 * (Jaro_impl.hpp:94-132, 258-276).  Returns common chars, transpositions (unhalved). */
template <typename PMF, typename TXT>
RFG_HD void jaro_word(const PMF& pm, int pl, const TXT& t, int tl, int* common, int* transp, int need = 0)
{
    int bound = (pl > tl ? pl : tl) / 2;
    if (bound > 0) --bound;
    int te = tl;
    if (te > pl + bound) te = pl + bound; /* text beyond the last window never matches */
    u64 pflag = 0, tflag = 0;
    u64 bmask = low_mask(bound + 1);
    const int lead = bound < te ? bound : te;
    /* text units fetched RFG_FETCH at a time (independent loads), as in the edit cores */
    for (int j0 = 0; j0 < te; j0 += RFG_FETCH) {
        u64 X[RFG_FETCH];
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) X[k] = j0 + k < te ? pm(t[j0 + k]) : 0;
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) {
            const int j = j0 + k;
            if (j < te) {
                const u64 x = X[k] & bmask & ~pflag;
                pflag |= blsi(x);
                tflag |= (u64)(x != 0) << j;
                bmask = j < lead ? (bmask << 1) | 1 : bmask << 1;
                /* each remaining text character adds at most one common character: a
                 * caller that only needs to know whether `need` is reached stops here */
                if ((j & 3) == 3 && popc64(pflag) + (te - 1 - j) < need) {
                    *common = 0;
                    *transp = 0;
                    return;
                }
            }
        }
    }
    *common = popc64(pflag);
    if (*common < need) {
        *transp = 0;
        return;
    }
    int tr = 0;
    while (tflag) {
        const u64 pbit = blsi(pflag);
        tr += (pm(t[ctz64(tflag)]) & pbit) == 0;
        tflag = blsr(tflag);
        pflag ^= pbit;
    }
    *transp = tr;
}

/* Jaro flagging of Q one-word patterns against one text, sharing each fetched block of
 * text units.  For every pattern q in `active`: the common and (unhalved)
 * transposition counts of jaro_word(pm_q, pl[q], t, tl, need[q]) -- a pattern whose
 * count can no longer reach need[q] stops early with both counts 0, and one that ends
 * below need[q] skips the transpositions.  Every active pattern
 * must have its effective text end (jaro_bounds) at or below 64. */
template <int Q, typename PMQ, typename TXT>
RFG_HD void group_jaro_word(const PMQ& pm, const int* pl, unsigned active, const TXT& t, int tl, const int* need,
                            int* common, int* transp)
{
    u64 pflag[Q], tflag[Q], bmask[Q];
    int te[Q], lead[Q];
    unsigned live = active;
    int temax = 0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        pflag[q] = tflag[q] = bmask[q] = 0;
        te[q] = lead[q] = 0;
        common[q] = transp[q] = 0;
        if (!((active >> q) & 1u)) continue;
        int bound = (pl[q] > tl ? pl[q] : tl) / 2;
        if (bound > 0) --bound;
        te[q] = tl < pl[q] + bound ? tl : pl[q] + bound;
        bmask[q] = low_mask(bound + 1);
        lead[q] = bound < te[q] ? bound : te[q];
        temax = te[q] > temax ? te[q] : temax;
    }
    for (int j0 = 0; j0 < temax && live; j0 += RFG_FETCH) {
        u64 c[RFG_FETCH];
#pragma unroll
        for (int k = 0; k < RFG_FETCH; ++k) c[k] = j0 + k < temax ? t[j0 + k] : 0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            if (!((live >> q) & 1u)) continue;
            if (j0 + RFG_FETCH <= te[q]) {
                /* a full block for this pattern: no per-unit bounds tests, the exit test at
                 * units 3 and 7 of the block (j0 is a multiple of RFG_FETCH) */
#pragma unroll
                for (int k = 0; k < RFG_FETCH; ++k) {
                    const int j = j0 + k;
                    const u64 x = pm(q, c[k]) & bmask[q] & ~pflag[q];
                    pflag[q] |= blsi(x);
                    tflag[q] |= (u64)(x != 0) << j;
                    bmask[q] = j < lead[q] ? (bmask[q] << 1) | 1 : bmask[q] << 1;
                    if ((k & 3) == 3 && popc64(pflag[q]) + (te[q] - 1 - j) < need[q]) live &= ~(1u << q);
                }
                continue;
            }
#pragma unroll
            for (int k = 0; k < RFG_FETCH; ++k) {
                const int j = j0 + k;
                if (j < te[q]) {
                    const u64 x = pm(q, c[k]) & bmask[q] & ~pflag[q];
                    pflag[q] |= blsi(x);
                    tflag[q] |= (u64)(x != 0) << j;
                    bmask[q] = j < lead[q] ? (bmask[q] << 1) | 1 : bmask[q] << 1;
                    if ((j & 3) == 3 && popc64(pflag[q]) + (te[q] - 1 - j) < need[q]) live &= ~(1u << q);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (!((live >> q) & 1u)) continue;
        common[q] = popc64(pflag[q]);
        if (common[q] < need[q]) continue;
        int tr = 0;
        u64 pf = pflag[q], tf = tflag[q];
        while (tf) {
            const u64 pbit = blsi(pf);
            tr += (pm(q, t[ctz64(tf)]) & pbit) == 0;
            tf = blsr(tf);
            pf ^= pbit;
        }
        transp[q] = tr;
    }
}

/* ========================================================= multi-word cores
 * PMW: pm(c, w) = word w of the pattern-match vector of c.  W words in registers,
 * pattern length m in (64*(W-1), 64*W] (smaller m works: the extra words stay zero). */

/* Myers/Hyyro blocks (Levenshtein_impl.hpp:641-850 without the band) */
template <int W, typename PMW, typename TXT>
RFG_HD i64 lev_multi(const PMW& pm, int m, const TXT& t, int n, i64 K)
{
    u64 VP[W], VN[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        VP[w] = ~0ull;
        VN[w] = 0;
    }
    const bool check = K < (i64)(m > n ? m : n);
    u64 c_next = n > 0 ? t[0] : 0; /* the next unit, loaded one step ahead */
    for (int j = 0; j < n; ++j) {
        const u64 c = c_next;
        if (j + 1 < n) c_next = t[j + 1];
        u64 hp_c = 1, hn_c = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const u64 X = pm(c, w) | hn_c;
            const u64 vp = VP[w], vn = VN[w];
            const u64 D0 = (((X & vp) + vp) ^ vp) | X | vn;
            u64 HP = vn | ~(D0 | vp);
            u64 HN = D0 & vp;
            const u64 hp_o = HP >> 63, hn_o = HN >> 63;
            HP = (HP << 1) | hp_c;
            HN = (HN << 1) | hn_c;
            hp_c = hp_o;
            hn_c = hn_o;
            VP[w] = HN | ~(D0 | HP);
            VN[w] = HP & D0;
        }
        if (check && (j & 7) == 7) {
            const int jj = j + 1, is = m - n + jj;
            if (is >= 0) {
                i64 lb = jj;
#pragma unroll
                for (int w = 0; w < W; ++w) {
                    const int b = is - 64 * w;
                    const u64 lm = b <= 0 ? 0 : low_mask(b);
                    lb += popc64(VP[w] & lm) - popc64(VN[w] & lm);
                }
                if (lb > K) return K + 1;
            }
        }
    }
    i64 d = n;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const int b = m - 64 * w;
        const u64 lm = b <= 0 ? 0 : low_mask(b);
        d += popc64(VP[w] & lm) - popc64(VN[w] & lm);
    }
    return d;
}

/* Hyyro 2004 over words with the add carry chained (LCSseq_impl.hpp:205-260) */
template <int W, typename PMW, typename TXT>
RFG_HD i64 lcs_multi(const PMW& pm, int m, const TXT& t, int n, i64 Kd)
{
    u64 S[W];
#pragma unroll
    for (int w = 0; w < W; ++w) S[w] = ~0ull;
    const bool check = Kd < (i64)(m + n);
    u64 c_next = n > 0 ? t[0] : 0; /* the next unit, loaded one step ahead */
    for (int j = 0; j < n; ++j) {
        const u64 c = c_next;
        if (j + 1 < n) c_next = t[j + 1];
        u32 carry = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const u64 X = pm(c, w);
            const u64 s = S[w];
            const u64 u = s & X;
            const u64 x = add_carry(s, u, carry, &carry);
            S[w] = x | (s - u);
        }
        if (check && (j & 7) == 7) {
            const int jj = j + 1, is = m - n + jj;
            if (is >= 0) {
                i64 lcs_is = 0;
#pragma unroll
                for (int w = 0; w < W; ++w) {
                    const int b = is - 64 * w;
                    lcs_is += popc64(~S[w] & (b <= 0 ? 0 : low_mask(b)));
                }
                if ((i64)is + jj - 2 * lcs_is > Kd) return -1;
            }
        }
    }
    i64 l = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const int b = m - 64 * w;
        l += popc64(~S[w] & (b <= 0 ? 0 : low_mask(b)));
    }
    return l;
}

/* OSA over words (OSA_impl.hpp:176-249): the transposition term of word w needs the
 * previous column's D0 and the current column's match vector of word w-1 */
template <int W, typename PMW, typename TXT>
RFG_HD i64 osa_multi(const PMW& pm, int m, const TXT& t, int n, i64 K)
{
    u64 VP[W], VN[W], D0v[W], PMo[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        VP[w] = ~0ull;
        VN[w] = 0;
        D0v[w] = 0;
        PMo[w] = 0;
    }
    const bool check = K < (i64)(m > n ? m : n);
    u64 c_next = n > 0 ? t[0] : 0; /* the next unit, loaded one step ahead */
    for (int j = 0; j < n; ++j) {
        const u64 c = c_next;
        if (j + 1 < n) c_next = t[j + 1];
        u64 hp_c = 1, hn_c = 0;
        u64 d0_prev_word = 0; /* previous column's D0 of word w-1 */
        u64 pm_prev_word = 0; /* this column's match vector of word w-1 */
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const u64 X = pm(c, w);
            const u64 vp = VP[w], vn = VN[w], d0_old = D0v[w];
            const u64 TR = ((((~d0_old) & X) << 1) | (((~d0_prev_word) & pm_prev_word) >> 63)) & PMo[w];
            const u64 Xc = X | hn_c;
            const u64 D0 = (((Xc & vp) + vp) ^ vp) | Xc | vn | TR;
            u64 HP = vn | ~(D0 | vp);
            u64 HN = D0 & vp;
            const u64 hp_o = HP >> 63, hn_o = HN >> 63;
            HP = (HP << 1) | hp_c;
            HN = (HN << 1) | hn_c;
            hp_c = hp_o;
            hn_c = hn_o;
            VP[w] = HN | ~(D0 | HP);
            VN[w] = HP & D0;
            d0_prev_word = d0_old;
            pm_prev_word = X;
            D0v[w] = D0;
            PMo[w] = X;
        }
        if (check && (j & 7) == 7) {
            const int jj = j + 1, is = m - n + jj;
            if (is >= 0) {
                i64 lb = jj;
#pragma unroll
                for (int w = 0; w < W; ++w) {
                    const int b = is - 64 * w;
                    const u64 lm = b <= 0 ? 0 : low_mask(b);
                    lb += popc64(VP[w] & lm) - popc64(VN[w] & lm);
                }
                if (lb > K) return K + 1;
            }
        }
    }
    i64 d = n;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const int b = m - 64 * w;
        const u64 lm = b <= 0 ? 0 : low_mask(b);
        d += popc64(VP[w] & lm) - popc64(VN[w] & lm);
    }
    return d;
}

/* Banded Levenshtein over a diagonal window of 64*B bits, the multi-word form of
 * levenshtein_hyrroe2003_small_band (Levenshtein_impl.hpp:419-505).  Requires
 * 2K+1 <= 64*B and |m-n| <= K.  Window bit b of step j is pattern index
 * K+1-64B+j+b; the window moves down one row per text character (the D0 >> 1 frame
 * shift).  diag tracks D[K+j][j] on the lower band edge (rows past m are virtual rows
 * without matches; they never feed rows <= m).  D[m-n+j][j] = diag minus the vertical
 * deltas of a fixed bit range below the edge: the early-stop bound and, at j = n, the
 * distance. */
template <int B, typename PMW, typename TXT>
RFG_HD i64 lev_band(const PMW& pm, int pw, int m, const TXT& t, int n, int K)
{
    const int NB = 64 * B;
    u64 VP[B], VN[B], rmask[B];
    /* initial column: rows 1..K+1 (bits NB-1-K .. NB-1) have vertical delta +1 */
#pragma unroll
    for (int b = 0; b < B; ++b) {
        VP[b] = range_mask(NB - 1 - K - 64 * b, NB - 1 - 64 * b);
        VN[b] = 0;
        rmask[b] = range_mask(NB - 1 - K + (m - n) - 64 * b, NB - 2 - 64 * b);
    }
    i64 diag = K;
    int start = K + 1 - NB; /* pattern index of window bit 0 */
    u64 c_next = n > 0 ? t[0] : 0; /* the next unit, loaded one step ahead */
    for (int j = 0; j < n; ++j, ++start) {
        const u64 c = c_next;
        if (j + 1 < n) c_next = t[j + 1];
        /* window of match bits: pattern indices [start, start + NB) */
        u64 X[B];
        {
            const int w0 = start >> 6; /* floor division */
            const int sh = start & 63;
            u64 prev = (w0 >= 0 && w0 < pw) ? pm(c, w0) : 0;
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const int wn = w0 + b + 1;
                const u64 next = (wn >= 0 && wn < pw) ? pm(c, wn) : 0;
                X[b] = sh ? ((prev >> sh) | (next << (64 - sh))) : prev;
                prev = next;
            }
        }
        u64 D0[B];
        u32 carry = 0;
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const u64 sum = add_carry(X[b] & VP[b], VP[b], carry, &carry);
            D0[b] = (sum ^ VP[b]) | X[b] | VN[b];
        }
        diag += (D0[B - 1] >> 63) == 0;
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const u64 HP = VN[b] | ~(D0[b] | VP[b]);
            const u64 HN = D0[b] & VP[b];
            const u64 hi = (b + 1 < B) ? D0[b + 1 < B ? b + 1 : b] : 0;
            const u64 D0s = (D0[b] >> 1) | (hi << 63);
            VP[b] = HN | ~(D0s | HP);
            VN[b] = D0s & HP;
        }
        if ((j & 7) == 7 || j == n - 1) {
            i64 v = diag;
#pragma unroll
            for (int b = 0; b < B; ++b) v -= popc64(VP[b] & rmask[b]) - popc64(VN[b] & rmask[b]);
            if (j == n - 1) return v;
            if (v > K) return (i64)K + 1;
        }
    }
    return (i64)n; /* n == 0; callers never ask (|m-n| <= K < m) */
}

/* bits [a, b] of a 32-bit word, clipped to [0, 31]; empty when b < a */
RFG_HD u32 range_mask32(int a, int b)
{
    if (a < 0) a = 0;
    if (b > 31) b = 31;
    if (b < a) return 0;
    return (b >= 31 ? ~0u : ((1u << (b + 1)) - 1)) & ~(a >= 32 ? ~0u : ((1u << a) - 1));
}

/* bits [sh, sh + 32) of the 64-bit value hi:lo, sh in [0, 31] (one funnel shift) */
RFG_HD u32 funnel32(u32 lo, u32 hi, int sh)
{
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, sh);
#else
    return (u32)((((u64)hi << 32) | lo) >> sh);
#endif
}

/* Ukkonen's band of a pair (m, n) with bound K: a path of cost <= K to (m, n) only visits
 * diagonals d = i - j with |d| + |(m - n) - d| <= K (it needs |d| indels to reach d and
 * |(m - n) - d| to leave it), i.e. d in [band_lo, band_hi] =
 * [-ceil((K - (m-n)) / 2), ceil((K + (m-n)) / 2)]: at most K + 2 diagonals, about half of
 * the 2K + 1 of the symmetric band.  |m - n| <= K. */
RFG_HD int band_lo(int K, int delta) { return -((K - delta + 1) >> 1); }
RFG_HD int band_hi(int K, int delta) { return (K + delta + 1) >> 1; }
RFG_HD int band_bits(int K, int delta) { return band_hi(K, delta) - band_lo(K, delta) + 1; }

/* units of window loads run ahead of the band recurrence in a whole block (about 32
 * registers of windows) */
#define BAND_AHEAD(B) ((B) <= 4 ? 8 / ((B) + 1 >> 1) : (B) <= 8 ? 4 : 2)

/* a hint that text unit j will be read soon (the band kernel's texts override it with a
 * cache prefetch); j is a valid index */
template <typename TXT>
RFG_HD void text_prefetch(const TXT&, int)
{
}

/* s = a + b over B 32-bit words, the carry out of the top word dropped: on the GPU one
 * add.cc / addc chain (the carry passes in the condition code, one instruction a word) */
template <int B>
RFG_HD void add_chain(const u32* a, const u32* b, u32* s)
{
#ifdef __CUDA_ARCH__
    if constexpr (B == 1)
        s[0] = a[0] + b[0];
    else if constexpr (B == 2)
        asm("add.cc.u32 %0, %2, %4; addc.u32 %1, %3, %5;"
            : "=r"(s[0]), "=r"(s[1])
            : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]));
    else if constexpr (B == 3)
        asm("add.cc.u32 %0, %3, %6; addc.cc.u32 %1, %4, %7; addc.u32 %2, %5, %8;"
            : "=r"(s[0]), "=r"(s[1]), "=r"(s[2])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(b[0]), "r"(b[1]), "r"(b[2]));
    else if constexpr (B == 4)
        asm("add.cc.u32 %0, %4, %8; addc.cc.u32 %1, %5, %9; addc.cc.u32 %2, %6, %10; addc.u32 %3, %7, %11;"
            : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
    else if constexpr (B == 6)
        asm("add.cc.u32 %0, %6, %12; addc.cc.u32 %1, %7, %13; addc.cc.u32 %2, %8, %14; addc.cc.u32 %3, %9, %15; addc.cc.u32 %4, %10, %16; addc.u32 %5, %11, %17;"
            : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]));
    else if constexpr (B == 8)
        asm("add.cc.u32 %0, %8, %16; addc.cc.u32 %1, %9, %17; addc.cc.u32 %2, %10, %18; addc.cc.u32 %3, %11, %19; addc.cc.u32 %4, %12, %20; addc.cc.u32 %5, %13, %21; addc.cc.u32 %6, %14, %22; addc.u32 %7, %15, %23;"
            : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
    else if constexpr (B == 12)
        asm("add.cc.u32 %0, %12, %24; addc.cc.u32 %1, %13, %25; addc.cc.u32 %2, %14, %26; addc.cc.u32 %3, %15, %27; addc.cc.u32 %4, %16, %28; addc.cc.u32 %5, %17, %29; addc.cc.u32 %6, %18, %30; addc.cc.u32 %7, %19, %31; addc.cc.u32 %8, %20, %32; addc.cc.u32 %9, %21, %33; addc.cc.u32 %10, %22, %34; addc.u32 %11, %23, %35;"
            : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]));
    else if constexpr (B == 16)
        asm("add.cc.u32 %0, %16, %32; addc.cc.u32 %1, %17, %33; addc.cc.u32 %2, %18, %34; addc.cc.u32 %3, %19, %35; addc.cc.u32 %4, %20, %36; addc.cc.u32 %5, %21, %37; addc.cc.u32 %6, %22, %38; addc.cc.u32 %7, %23, %39; addc.cc.u32 %8, %24, %40; addc.cc.u32 %9, %25, %41; addc.cc.u32 %10, %26, %42; addc.cc.u32 %11, %27, %43; addc.cc.u32 %12, %28, %44; addc.cc.u32 %13, %29, %45; addc.cc.u32 %14, %30, %46; addc.u32 %15, %31, %47;"
            : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11]), "=r"(s[12]), "=r"(s[13]), "=r"(s[14]), "=r"(s[15])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(a[12]), "r"(a[13]), "r"(a[14]), "r"(a[15]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]), "r"(b[12]), "r"(b[13]), "r"(b[14]), "r"(b[15]));
    else
        static_assert(B == 1, "no add chain for this width");
#else
    u32 carry = 0;
    for (int i = 0; i < B; ++i) {
        const u64 t = (u64)a[i] + b[i] + carry;
        s[i] = (u32)t;
        carry = (u32)(t >> 32);
    }
#endif
}

/* the B-word window of a pattern row from pattern index `start` (any sign; the row has
 * B + 1 zero words before word 0): one funnel shift per word */
template <int B>
RFG_HD void band_window(const u32* row, int start, u32* X)
{
    const int w0 = start >> 5; /* floor division (arithmetic shift) */
    const int sh = start & 31;
    u32 prev = row[w0];
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const u32 next = row[w0 + b + 1];
        X[b] = funnel32(prev, next, sh);
        prev = next;
    }
}

/* Banded Levenshtein on B 32-bit words (a window of 32*B bits) over a pattern table of
 * 32-bit words, for one-byte texts: pm(c) gives the row of text unit c as a pointer to
 * its words, with at least B + 1 zero words before word 0 and 2B + 2 after the last, so
 * the window's words are loaded without range tests.  Window bit b covers diagonal
 * dlo + b (pattern index dlo + j + b at step j); dlo = band_lo(K, m - n) and
 * band_bits(K, m - n) <= 32*B.  The carry of (X & VP) + VP runs through the words; the
 * frame moves down one row per text unit (D0 >> 1), as in
 * levenshtein_hyrroe2003_small_band (Levenshtein_impl.hpp:419-505).  The band computes
 * the distance over paths inside it -- exact for every pair whose distance is at most K,
 * since those paths never leave Ukkonen's band -- and the lower bound on the diagonal
 * through (m, n) stops it after every 8 text units once it passes K.
 * A pair is a lane's state (BandLane) that band_run8 advances 8 text units at a time:
 * the band kernel gives a lane whose pair ended the next pair, and the text of the next
 * 8 units is loaded while the current 8 run.  Requires |m-n| <= K < m, n > 0. */
template <int B>
struct BandLane {
    u32 VP[B], VN[B], rmask[B];
    u32 cur[2]; /* the block's 8 text units, 4 to a word */
    int diag;   /* D on the window's bottom diagonal */
    int start;  /* pattern index of window bit 0 at the block's first unit */
    int j, n, K;
};

template <int B, typename TXT>
RFG_HD void band_init(BandLane<B>& L, int m, const TXT& t, int n, int K)
{
    const int NB = 32 * B;
    const int dlo = band_lo(K, m - n);
#pragma unroll
    for (int b = 0; b < B; ++b) {
        L.VP[b] = range_mask32(-dlo - 32 * b, NB - 1 - 32 * b); /* rows 1.. of column 0: delta +1 */
        L.VN[b] = 0;
        L.rmask[b] = range_mask32((m - n) - dlo - 32 * b, NB - 2 - 32 * b);
    }
    L.diag = dlo + NB - 1;
    L.start = dlo;
    L.j = 0;
    L.n = n;
    L.K = K;
    u32 u[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) u[s] = (u32)t[s < n - 1 ? s : n - 1];
    L.cur[0] = u[0] | u[1] << 8 | u[2] << 16 | u[3] << 24;
    L.cur[1] = u[4] | u[5] << 8 | u[6] << 16 | u[7] << 24;
}

/* one text unit whose window X is loaded */
template <int B>
RFG_HD void band_step(BandLane<B>& L, const u32* X)
{
    u32 U[B], S[B], D0[B];
#pragma unroll
    for (int b = 0; b < B; ++b) U[b] = X[b] & L.VP[b];
    add_chain<B>(U, L.VP, S);
#pragma unroll
    for (int b = 0; b < B; ++b) D0[b] = (S[b] ^ L.VP[b]) | X[b] | L.VN[b];
    L.diag += 1 - (int)(D0[B - 1] >> 31);
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const u32 HP = L.VN[b] | ~(D0[b] | L.VP[b]);
        const u32 HN = D0[b] & L.VP[b];
        const u32 D0s = b + 1 < B ? funnel32(D0[b], D0[b + 1 < B ? b + 1 : b], 1) : (D0[b] >> 1);
        L.VP[b] = HN | ~(D0s | HP);
        L.VN[b] = D0s & HP;
    }
}

/* the next 8 text units (fewer at the end); true when the pair is done, with *out = d,
 * or any value > K */
template <int B, typename PM32, typename TXT>
RFG_HD bool band_run8(BandLane<B>& L, const PM32& pm, const TXT& t, i64* out)
{
    const int last = L.n - 1;
    u32 nx[8];
    if (L.j + 16 <= L.n) {
#pragma unroll
        for (int s = 0; s < 8; ++s) nx[s] = (u32)t[L.j + 8 + s];
    }
    else {
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const int k = L.j + 8 + s;
            nx[s] = (u32)t[k < last ? k : last];
        }
    }
    text_prefetch(t, L.j + 64 < last ? L.j + 64 : last);
    const int rem = L.n - L.j;
    if (rem >= 8) {
        /* a whole block: straight-line code whose windows are loaded BAND_AHEAD units
         * before their step (they depend on the text alone, not on the recurrence) */
        constexpr int AH = BAND_AHEAD(B);
        u32 X[8][B];
#pragma unroll
        for (int s = 0; s < AH; ++s) band_window<B>(pm((L.cur[s >> 2] >> (8 * (s & 3))) & 0xffu), L.start + s, X[s]);
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            if (s + AH < 8)
                band_window<B>(pm((L.cur[(s + AH) >> 2] >> (8 * ((s + AH) & 3))) & 0xffu), L.start + s + AH,
                               X[s + AH < 8 ? s + AH : 0]);
            band_step<B>(L, X[s]);
        }
    }
    else {
#pragma unroll
        for (int s = 0; s < 8; ++s)
            if (s < rem) {
                const u32 c = (L.cur[s >> 2] >> (8 * (s & 3))) & 0xffu;
                u32 X[B];
                band_window<B>(pm(c), L.start + s, X);
                band_step<B>(L, X);
            }
    }
    L.j += 8;
    L.start += 8;
    int v = L.diag;
#pragma unroll
    for (int b = 0; b < B; ++b) v -= popc_w(L.VP[b] & L.rmask[b]) - popc_w(L.VN[b] & L.rmask[b]);
    if (L.j >= L.n) {
        *out = v;
        return true;
    }
    if (v > L.K) {
        *out = (i64)L.K + 1;
        return true;
    }
    L.cur[0] = nx[0] | nx[1] << 8 | nx[2] << 16 | nx[3] << 24;
    L.cur[1] = nx[4] | nx[5] << 8 | nx[6] << 16 | nx[7] << 24;
    return false;
}

/* one pair start to end; *steps (if given) = the text units run */
template <int B, typename PM32, typename TXT>
RFG_HD i64 lev_band32(const PM32& pm, int m, const TXT& t, int n, int K, int* steps = nullptr)
{
    BandLane<B> L;
    band_init<B>(L, m, t, n, K);
    i64 v = 0;
    while (!band_run8<B>(L, pm, t, &v)) {
    }
    if (steps) *steps = L.j < n ? L.j : n;
    return v;
}

/* Banded LCS on B 32-bit words, the band of lcs_blockwise (LCSseq_impl.hpp:262-333)
 * moved one row per text unit like the Levenshtein band above.  The LCS families reach
 * the core with an Indel-distance bound K (an LCS of at least (m + n - K) / 2), and a path
 * with at most K indels visits only the diagonals of Ukkonen's band for K -- the window
 * of band_lo / band_bits: bit b of the window is the difference bit (Hyyro's S, 0 = the
 * LCS rises at that pattern unit) of pattern index start + b.  Each text unit runs the
 * step S' = (S + (S & X)) | (S & ~X) (LCSseq_impl.hpp:226-229) over the window with no
 * carry into its bottom word, then moves the frame: the bottom bit leaves (a 0 adds one
 * to `base`, the LCS of the units below the window), and a 1 enters at the top.  Every
 * value the window then holds is the LCS of some real alignment (a pattern unit below
 * the window keeps its last value, one above it adds nothing), so the result never
 * exceeds the true LCS, and it equals it when the LCS is at least (m + n - K) / 2, since
 * those alignments never leave the band.  Indel distances along a diagonal never fall,
 * so after every 8 text units the cell on the diagonal of (m, n) (pattern index j + m - n
 * after j units: the window bits below m - n - dlo) gives a lower bound that stops the
 * pair once it passes K.  The lane reports the Indel distance m + n - 2 LCS, or any
 * value > K.  Requires |m - n| <= K, n > 0. */
template <int B>
struct LcsBandLane {
    u32 S[B], dmask[B];
    u32 cur[2]; /* the block's 8 text units, 4 to a word */
    u32 gone;   /* the bits that left the window in this block, the latest at bit 31 */
    int base;   /* LCS of the pattern units below the window */
    int start;  /* pattern index of window bit 0 at the block's first unit */
    int j, n, K, mn;
};

template <int B, typename TXT>
RFG_HD void lcs_band_init(LcsBandLane<B>& L, int m, const TXT& t, int n, int K)
{
    const int dlo = band_lo(K, m - n);
#pragma unroll
    for (int b = 0; b < B; ++b) {
        L.S[b] = ~0u;
        L.dmask[b] = range_mask32(-32 * b, (m - n) - dlo - 1 - 32 * b);
    }
    L.gone = ~0u;
    L.base = 0;
    L.start = dlo;
    L.j = 0;
    L.n = n;
    L.K = K;
    L.mn = m + n;
    u32 u[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) u[s] = (u32)t[s < n - 1 ? s : n - 1];
    L.cur[0] = u[0] | u[1] << 8 | u[2] << 16 | u[3] << 24;
    L.cur[1] = u[4] | u[5] << 8 | u[6] << 16 | u[7] << 24;
}

/* one text unit whose window X is loaded */
template <int B>
RFG_HD void lcs_band_step(LcsBandLane<B>& L, const u32* X)
{
    u32 U[B], T[B];
#pragma unroll
    for (int b = 0; b < B; ++b) U[b] = L.S[b] & X[b];
    add_chain<B>(L.S, U, T);
#pragma unroll
    for (int b = 0; b < B; ++b) T[b] = T[b] | (L.S[b] & ~X[b]);
    L.gone = funnel32(L.gone, T[0], 1);
#pragma unroll
    for (int b = 0; b < B; ++b) L.S[b] = funnel32(T[b], b + 1 < B ? T[b + 1 < B ? b + 1 : b] : ~0u, 1);
}

/* the next 8 text units (fewer at the end); true when the pair is done, with *out = the
 * Indel distance, or any value > K */
template <int B, typename PM32, typename TXT>
RFG_HD bool lcs_band_run8(LcsBandLane<B>& L, const PM32& pm, const TXT& t, i64* out)
{
    const int last = L.n - 1;
    u32 nx[8];
    if (L.j + 16 <= L.n) {
#pragma unroll
        for (int s = 0; s < 8; ++s) nx[s] = (u32)t[L.j + 8 + s];
    }
    else {
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const int k = L.j + 8 + s;
            nx[s] = (u32)t[k < last ? k : last];
        }
    }
    text_prefetch(t, L.j + 64 < last ? L.j + 64 : last);
    const int rem = L.n - L.j;
    if (rem >= 8) {
        constexpr int AH = BAND_AHEAD(B);
        u32 X[8][B];
#pragma unroll
        for (int s = 0; s < AH; ++s) band_window<B>(pm((L.cur[s >> 2] >> (8 * (s & 3))) & 0xffu), L.start + s, X[s]);
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            if (s + AH < 8)
                band_window<B>(pm((L.cur[(s + AH) >> 2] >> (8 * ((s + AH) & 3))) & 0xffu), L.start + s + AH,
                               X[s + AH < 8 ? s + AH : 0]);
            lcs_band_step<B>(L, X[s]);
        }
    }
    else {
#pragma unroll
        for (int s = 0; s < 8; ++s)
            if (s < rem) {
                const u32 c = (L.cur[s >> 2] >> (8 * (s & 3))) & 0xffu;
                u32 X[B];
                band_window<B>(pm(c), L.start + s, X);
                lcs_band_step<B>(L, X);
            }
            else L.gone = funnel32(L.gone, ~0u, 1);
    }
    /* the block's 8 leaving bits are the top byte of `gone` */
    L.base += 8 - popc_w(L.gone >> 24);
    L.j += 8;
    L.start += 8;
    if (L.j >= L.n) {
        int lcs = L.base;
#pragma unroll
        for (int b = 0; b < B; ++b) lcs += popc_w(~L.S[b]);
        *out = L.mn - 2 * lcs;
        return true;
    }
    int v = L.base;
#pragma unroll
    for (int b = 0; b < B; ++b) v += popc_w(~L.S[b] & L.dmask[b]);
    /* the cell (j + m - n, j): (j + m - n) + j - 2 v */
    if (2 * L.j + (L.mn - 2 * L.n) - 2 * v > L.K) {
        *out = (i64)L.K + 1;
        return true;
    }
    L.cur[0] = nx[0] | nx[1] << 8 | nx[2] << 16 | nx[3] << 24;
    L.cur[1] = nx[4] | nx[5] << 8 | nx[6] << 16 | nx[7] << 24;
    return false;
}

/* one pair start to end; *steps (if given) = the text units run */
template <int B, typename PM32, typename TXT>
RFG_HD i64 lcs_band32(const PM32& pm, int m, const TXT& t, int n, int K, int* steps = nullptr)
{
    LcsBandLane<B> L;
    lcs_band_init<B>(L, m, t, n, K);
    i64 v = 0;
    while (!lcs_band_run8<B>(L, pm, t, &v)) {
    }
    if (steps) *steps = L.j < n ? L.j : n;
    return v;
}

/* Jaro with P (= s1) of up to 64*W chars and a text of any length: the greedy
 * flagging of flag_similar_characters_block (Jaro_impl.hpp:134-256), with the window
 * masks built per word, and the transposition count of count_transpositions_block
 * (Jaro_impl.hpp:278-315), which pairs the k-th flagged text character with the k-th
 * flagged pattern position.  Up to 64 relevant text characters the text flags live in
 * one register; beyond that the flagging is run a second time and each newly flagged
 * text character is compared on the fly, so no per-text storage is needed. */
template <int W, typename PMW, typename TXT>
RFG_HD bool jaro_flag_step(const PMW& pm, u64* pflag, u64 c, int lo, int hi)
{
    bool found = false;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const u64 x = pm(c, w) & range_mask(lo - 64 * w, hi - 64 * w) & ~pflag[w];
        if (!found && x) {
            pflag[w] |= blsi(x);
            found = true;
        }
    }
    return found;
}

template <int W>
RFG_HD u64 select_word(const u64* v, int idx)
{
    u64 r = 0;
#pragma unroll
    for (int w = 0; w < W; ++w)
        if (w == idx) r = v[w];
    return r;
}

template <int W, typename PMW, typename TXT>
RFG_HD void jaro_multi(const PMW& pm, int pl, const TXT& t, int tl, int* common, int* transp)
{
    int bound = (pl > tl ? pl : tl) / 2;
    if (bound > 0) --bound;
    int te = tl;
    if (te > pl + bound) te = pl + bound;
    u64 pflag[W];
#pragma unroll
    for (int w = 0; w < W; ++w) pflag[w] = 0;
    u64 tflag = 0;
    for (int j = 0; j < te; ++j) {
        const bool f = jaro_flag_step<W, PMW, TXT>(pm, pflag, t[j], j - bound, j + bound);
        if (j < 64) tflag |= (u64)f << j;
    }
    int cc = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) cc += popc64(pflag[w]);
    *common = cc;
    int tr = 0, pwi = 0;
    u64 pf = select_word<W>(pflag, 0);
    auto next_pbit = [&]() -> u64 {
        while (!pf) pf = select_word<W>(pflag, ++pwi);
        const u64 b = blsi(pf);
        pf ^= b;
        return b;
    };
    if (te <= 64) {
        while (tflag) {
            const u64 pbit = next_pbit();
            tr += (pm(t[ctz64(tflag)], pwi) & pbit) == 0;
            tflag = blsr(tflag);
        }
    }
    else {
        u64 pflag2[W];
#pragma unroll
        for (int w = 0; w < W; ++w) pflag2[w] = 0;
        for (int j = 0; j < te; ++j) {
            const u64 r = t[j];
            if (jaro_flag_step<W, PMW, TXT>(pm, pflag2, r, j - bound, j + bound)) {
                const u64 pbit = next_pbit();
                tr += (pm(r, pwi) & pbit) == 0;
            }
        }
    }
    *transp = tr;
}

/* ======================================================= any-length cores
 * Runtime word count W, state in caller-provided memory (global scratch on the
 * device): the same recurrences as the register-resident cores above. */

template <typename PMW, typename TXT>
RFG_HD i64 lev_multi_rt(const PMW& pm, int W, int m, const TXT& t, int n, i64 K, u64* VP, u64* VN)
{
    for (int w = 0; w < W; ++w) {
        VP[w] = ~0ull;
        VN[w] = 0;
    }
    const bool check = K < (i64)(m > n ? m : n);
    for (int j = 0; j < n; ++j) {
        const u64 c = t[j];
        u64 hp_c = 1, hn_c = 0;
        for (int w = 0; w < W; ++w) {
            const u64 X = pm(c, w) | hn_c;
            const u64 vp = VP[w], vn = VN[w];
            const u64 D0 = (((X & vp) + vp) ^ vp) | X | vn;
            u64 HP = vn | ~(D0 | vp);
            u64 HN = D0 & vp;
            const u64 hp_o = HP >> 63, hn_o = HN >> 63;
            HP = (HP << 1) | hp_c;
            HN = (HN << 1) | hn_c;
            hp_c = hp_o;
            hn_c = hn_o;
            VP[w] = HN | ~(D0 | HP);
            VN[w] = HP & D0;
        }
        if (check && (j & 7) == 7) {
            const int jj = j + 1, is = m - n + jj;
            if (is >= 0) {
                i64 lb = jj;
                for (int w = 0; w * 64 < is; ++w) {
                    const u64 lm = low_mask(is - 64 * w);
                    lb += popc64(VP[w] & lm) - popc64(VN[w] & lm);
                }
                if (lb > K) return K + 1;
            }
        }
    }
    i64 d = n;
    for (int w = 0; w * 64 < m; ++w) {
        const u64 lm = low_mask(m - 64 * w);
        d += popc64(VP[w] & lm) - popc64(VN[w] & lm);
    }
    return d;
}

template <typename PMW, typename TXT>
RFG_HD i64 lcs_multi_rt(const PMW& pm, int W, int m, const TXT& t, int n, i64 Kd, u64* S)
{
    for (int w = 0; w < W; ++w) S[w] = ~0ull;
    const bool check = Kd < (i64)(m + n);
    for (int j = 0; j < n; ++j) {
        const u64 c = t[j];
        u32 carry = 0;
        for (int w = 0; w < W; ++w) {
            const u64 X = pm(c, w);
            const u64 sv = S[w];
            const u64 u = sv & X;
            const u64 x = add_carry(sv, u, carry, &carry);
            S[w] = x | (sv - u);
        }
        if (check && (j & 7) == 7) {
            const int jj = j + 1, is = m - n + jj;
            if (is >= 0) {
                i64 l = 0;
                for (int w = 0; w * 64 < is; ++w) l += popc64(~S[w] & low_mask(is - 64 * w));
                if ((i64)is + jj - 2 * l > Kd) return -1;
            }
        }
    }
    i64 l = 0;
    for (int w = 0; w * 64 < m; ++w) l += popc64(~S[w] & low_mask(m - 64 * w));
    return l;
}

template <typename PMW, typename TXT>
RFG_HD i64 osa_multi_rt(const PMW& pm, int W, int m, const TXT& t, int n, i64 K, u64* VP, u64* VN, u64* D0v,
                        u64* PMo)
{
    for (int w = 0; w < W; ++w) {
        VP[w] = ~0ull;
        VN[w] = 0;
        D0v[w] = 0;
        PMo[w] = 0;
    }
    const bool check = K < (i64)(m > n ? m : n);
    for (int j = 0; j < n; ++j) {
        const u64 c = t[j];
        u64 hp_c = 1, hn_c = 0, d0_prev_word = 0, pm_prev_word = 0;
        for (int w = 0; w < W; ++w) {
            const u64 X = pm(c, w);
            const u64 vp = VP[w], vn = VN[w], d0_old = D0v[w];
            const u64 TR = ((((~d0_old) & X) << 1) | (((~d0_prev_word) & pm_prev_word) >> 63)) & PMo[w];
            const u64 Xc = X | hn_c;
            const u64 D0 = (((Xc & vp) + vp) ^ vp) | Xc | vn | TR;
            u64 HP = vn | ~(D0 | vp);
            u64 HN = D0 & vp;
            const u64 hp_o = HP >> 63, hn_o = HN >> 63;
            HP = (HP << 1) | hp_c;
            HN = (HN << 1) | hn_c;
            hp_c = hp_o;
            hn_c = hn_o;
            VP[w] = HN | ~(D0 | HP);
            VN[w] = HP & D0;
            d0_prev_word = d0_old;
            pm_prev_word = X;
            D0v[w] = D0;
            PMo[w] = X;
        }
        if (check && (j & 7) == 7) {
            const int jj = j + 1, is = m - n + jj;
            if (is >= 0) {
                i64 lb = jj;
                for (int w = 0; w * 64 < is; ++w) {
                    const u64 lm = low_mask(is - 64 * w);
                    lb += popc64(VP[w] & lm) - popc64(VN[w] & lm);
                }
                if (lb > K) return K + 1;
            }
        }
    }
    i64 d = n;
    for (int w = 0; w * 64 < m; ++w) {
        const u64 lm = low_mask(m - 64 * w);
        d += popc64(VP[w] & lm) - popc64(VN[w] & lm);
    }
    return d;
}

/* Jaro with any pattern length: flags in caller memory (W words), two-pass
 * transposition count (see jaro_multi) */
template <typename PMW>
RFG_HD bool jaro_flag_step_rt(const PMW& pm, int W, u64* pflag, u64 c, int lo, int hi)
{
    int w0 = lo < 0 ? 0 : lo >> 6;
    const int w1 = hi >> 6;
    for (int w = w0; w <= w1 && w < W; ++w) {
        const u64 x = pm(c, w) & range_mask(lo - 64 * w, hi - 64 * w) & ~pflag[w];
        if (x) {
            pflag[w] |= blsi(x);
            return true;
        }
    }
    return false;
}

template <typename PMW, typename TXT>
RFG_HD void jaro_multi_rt(const PMW& pm, int W, int pl, const TXT& t, int tl, int* common, int* transp, u64* pflag,
                          u64* pflag2)
{
    int bound = (pl > tl ? pl : tl) / 2;
    if (bound > 0) --bound;
    int te = tl;
    if (te > pl + bound) te = pl + bound;
    for (int w = 0; w < W; ++w) {
        pflag[w] = 0;
        pflag2[w] = 0;
    }
    for (int j = 0; j < te; ++j) jaro_flag_step_rt(pm, W, pflag, t[j], j - bound, j + bound);
    int cc = 0;
    for (int w = 0; w < W; ++w) cc += popc64(pflag[w]);
    *common = cc;
    int tr = 0, pwi = 0;
    u64 pf = W > 0 ? pflag[0] : 0;
    for (int j = 0; j < te; ++j) {
        const u64 r = t[j];
        if (jaro_flag_step_rt(pm, W, pflag2, r, j - bound, j + bound)) {
            while (!pf) pf = pflag[++pwi];
            const u64 pbit = blsi(pf);
            pf ^= pbit;
            tr += (pm(r, pwi) & pbit) == 0;
        }
    }
    *transp = tr;
}

/* generalized Wagner-Fischer (Levenshtein_impl.hpp:85-155): weighted distance,
 * common affix stripped, `cache` holds m+1 entries; S1/S2 yield raw code units */
template <typename S1, typename S2>
RFG_HD u64 wf_distance(const S1& s1, int m, const S2& s2, int n, const ScoreParams& w, u64 max, u64* cache)
{
    const u64 ins = (u64)w.ins, del = (u64)w.del, rep = (u64)w.rep;
    const u64 min_edits = m > n ? (u64)(m - n) * del : (u64)(n - m) * ins;
    if (min_edits > max) return max + 1;
    int a0 = 0, a1 = m, b0 = 0, b1 = n;
    while (a0 < a1 && b0 < b1 && s1[a0] == s2[b0]) ++a0, ++b0;
    while (a0 < a1 && b0 < b1 && s1[a1 - 1] == s2[b1 - 1]) --a1, --b1;
    const int mm = a1 - a0;
    for (int i = 0; i <= mm; ++i) cache[i] = (u64)i * del;
    for (int j = b0; j < b1; ++j) {
        const u64 cj = s2[j];
        u64 temp = cache[0];
        cache[0] += ins;
        for (int i = 0; i < mm; ++i) {
            if (s1[a0 + i] != cj) {
                u64 v = cache[i] + del;
                const u64 v2 = cache[i + 1] + ins;
                const u64 v3 = temp + rep;
                v = v2 < v ? v2 : v;
                temp = v3 < v ? v3 : v;
            }
            const u64 nx = cache[i + 1];
            cache[i + 1] = temp;
            temp = nx;
        }
    }
    const u64 d = cache[mm];
    return d <= max ? d : max + 1;
}

/* ====================================================== formula chains
 * plan_*: the cutoff the reference passes to the metric's _distance/_similarity for
 *         (metric, op, form) -- the core's pruning bound is derived from it;
 * finish_*: the reference's arithmetic from that call's result to the API result. */

RFG_HD double norm_sim_to_norm_dist(double c) { return dmin(1.0, dadd(dsub(1.0, c), 0.00001)); } /* common.hpp:50-53 */

RFG_HD u64 ceil_div_u(u64 a, u64 d) { return a / d + (u64)(a % d != 0); }

/* (size_t)std::ceil((double)maximum * cutoff) */
RFG_HD u64 ceil_cut(u64 maximum, double c) { return (u64)dceil(dmul((double)maximum, c)); }

/* levenshtein_maximum (Levenshtein_impl.hpp:118-128) */
RFG_HD u64 lev_maximum(u64 l1, u64 l2, const ScoreParams& p)
{
    const u64 ins = (u64)p.ins, del = (u64)p.del, rep = (u64)p.rep;
    u64 mx = l1 * del + l2 * ins;
    u64 alt = (l1 >= l2) ? l2 * rep + (l1 - l2) * del : l1 * rep + (l2 - l1) * ins;
    return alt < mx ? alt : mx;
}

/* How a Levenshtein weight table maps onto a core (Levenshtein_impl.hpp:1061-1088) */
enum LevMode { LEV_ZERO = 0, LEV_UNIFORM = 1, LEV_INDEL = 2, LEV_GENERAL = 3 };
RFG_HD int lev_mode(const ScoreParams& p)
{
    if (p.ins == p.del) {
        if (p.ins == 0) return LEV_ZERO;
        if (p.ins == p.rep) return LEV_UNIFORM;
        if (p.rep >= p.ins + p.del) return LEV_INDEL;
    }
    return LEV_GENERAL;
}

/* Family of the bit-parallel core that (metric, weights, form) needs */
RFG_HD int metric_family(int metric, int form, const ScoreParams& p)
{
    switch (metric) {
    case LEVENSHTEIN:
        if (form == FORM_MULTI) return FAM_LEV; /* Multi ignores the replace weight (Levenshtein.hpp:391-398) */
        switch (lev_mode(p)) {
        case LEV_ZERO: return FAM_NONE;
        case LEV_UNIFORM: return FAM_LEV;
        case LEV_INDEL: return FAM_LCS;
        default: return FAM_WF;
        }
    case INDEL:
    case LCSSEQ:
    case RATIO: return FAM_LCS;
    case OSA: return FAM_OSA;
    case PARTIAL_RATIO: return FAM_PARTIAL;
    case TOKEN_SORT_RATIO:
    case PARTIAL_TOKEN_SORT_RATIO:
    case QRATIO:
    case TOKEN_SET_RATIO:
    case PARTIAL_TOKEN_SET_RATIO:
    case TOKEN_RATIO:
    case PARTIAL_TOKEN_RATIO:
    case WRATIO: return FAM_TOKEN;
    default: return FAM_JARO;
    }
}

/* A pair's plan: which core bound to run with (native units of the core) */
struct Plan {
    int run;     /* 0: the result needs no core */
    i64 K;       /* pruning bound: distance for LEV/OSA/WF, Indel distance for LCS */
    u64 Kchain;  /* the cutoff of the chain's single _distance/_similarity call */
    double jc;   /* Jaro cutoff (Jaro families) */
    u64 lcs_min; /* LCS families: the _similarity cutoff */
};

RFG_HD i64 clamp_bound(u64 k) { return k > (u64)0x3fffffffffffffffull ? (i64)0x3fffffffffffffffll : (i64)k; }

/* integer cutoff of a normalized op: ceil(M * c_nd) (distance.hpp:52-76); ratio: the
 * cutoff arrives in percent (fuzz_impl.hpp:28-32) */
RFG_COLD u64 norm_cut(int op, u64 M, double cf, int ratio)
{
    if (ratio) cf = ddiv(cf, 100.0);
    return op == NORM_DISTANCE ? ceil_cut(M, cf) : ceil_cut(M, norm_sim_to_norm_dist(cf));
}

/* _distance cutoff of a distance-type chain (distance.hpp:52-64, 120-133, 240-262, 304-317) */
RFG_HD bool dist_chain_cutoff(int op, u64 M, u64 ci, double cf, u64* K)
{
    switch (op) {
    case DISTANCE: *K = ci; return true;
    case SIMILARITY:
        if (ci > M) return false;
        *K = M - ci;
        return true;
    default: *K = norm_cut(op, M, cf, 0); return true;
    }
}

/* finish of a distance-type chain given d = _distance(K), K the chain's cutoff.
 * A pruned pair of a normalized op has d = K + 1 with K = ceil(M * c): then
 * (K+1)/M >= c(1 - 2^-53) + 1/M exceeds c by far more than one rounding step (M < 2^33,
 * c <= 2), so the reference returns exactly 1.0 (normalized distance) or 0.0
 * (normalized similarity) -- taken here without the double division. */
RFG_COLD double norm_finish(int op, u64 M, u64 d, double cf, u64 Kc)
{
    if (M != 0 && Kc != ~0ull && d > Kc && cf <= 2.0 && cf >= -2.0) return op == NORM_DISTANCE ? 1.0 : 0.0;
    if (op == NORM_DISTANCE) {
        const double nd = M != 0 ? ddiv((double)d, (double)M) : 0.0;
        return nd <= cf ? nd : 1.0;
    }
    const double cs = norm_sim_to_norm_dist(cf);
    double nd = M != 0 ? ddiv((double)d, (double)M) : 0.0;
    nd = nd <= cs ? nd : 1.0;
    const double ns = dsub(1.0, nd);
    return ns >= cf ? ns : 0.0;
}

RFG_HD void dist_chain_finish(int op, u64 M, u64 d, u64 ci, double cf, i64* oi, double* of, u64 Kc = ~0ull)
{
    if (op == DISTANCE) {
        *oi = (i64)d;
        return;
    }
    if (op == SIMILARITY) {
        const u64 s = M - d;
        *oi = s >= ci ? (i64)s : 0;
        return;
    }
    if (M != 0 && Kc != ~0ull && d > Kc && abs_le_bits(cf, 2.0)) {
        *of = op == NORM_DISTANCE ? 1.0 : 0.0; /* the shortcut of norm_finish, integer tests only */
        return;
    }
    *of = norm_finish(op, M, d, cf, Kc);
}

/* fuzz::ratio = indel_normalized_similarity(s1, s2, c / 100) * 100 (fuzz_impl.hpp:28-32) */
RFG_COLD double ratio_finish(u64 M, u64 d, double cf_percent, u64 Kc)
{
    const double r = norm_finish(NORM_SIMILARITY, M, d, ddiv(cf_percent, 100.0), Kc);
    return r == 0.0 ? 0.0 : dmul(r, 100.0);
}

/* Multi* chains (distance.hpp:421-460, 500-512, 552-563) over exact values */
RFG_HD void multi_dist_finish(int op, u64 M, u64 D, u64 ci, double cf, i64* oi, double* of)
{
    switch (op) {
    case DISTANCE: *oi = (i64)(D <= ci ? D : ci + 1); return;
    case SIMILARITY: {
        const u64 s = M - D;
        *oi = s >= ci ? (i64)s : 0;
        return;
    }
    case NORM_DISTANCE: {
        const double nd = M != 0 ? ddiv((double)D, (double)M) : 0.0;
        *of = nd <= cf ? nd : 1.0;
        return;
    }
    default: {
        double nd = M != 0 ? ddiv((double)D, (double)M) : 0.0;
        nd = nd <= 1.0 ? nd : 1.0;
        const double ns = dsub(1.0, nd);
        *of = ns >= cf ? ns : 0.0;
    }
    }
}

RFG_HD void multi_sim_finish(int op, u64 M, u64 S, u64 ci, double cf, i64* oi, double* of)
{
    switch (op) {
    case SIMILARITY: *oi = S >= ci ? (i64)S : 0; return;
    case DISTANCE: {
        const u64 d = M - S;
        *oi = (i64)(d <= ci ? d : ci + 1);
        return;
    }
    default: multi_dist_finish(op, M, M - S, ci, cf, oi, of);
    }
}

/* ------------------------------------------------------------------ Jaro */

RFG_HD double jaro_formula(i64 pl, i64 tl, i64 common, i64 transp) /* Jaro_impl.hpp:32-42 */
{
    transp /= 2;
    double sim = ddiv((double)common, (double)pl);
    sim = dadd(sim, ddiv((double)common, (double)tl));
    sim = dadd(sim, ddiv(dsub((double)common, (double)transp), (double)common));
    return ddiv(sim, 3.0);
}

RFG_HD bool jaro_length_filter(i64 pl, i64 tl, double c) /* Jaro_impl.hpp:47-55 */
{
    if (!tl || !pl) return false;
    const double mn = (double)(pl < tl ? pl : tl);
    double sim = dadd(dadd(ddiv(mn, (double)pl), ddiv(mn, (double)tl)), 1.0);
    sim = ddiv(sim, 3.0);
    return sim >= c;
}

RFG_HD bool jaro_common_filter(i64 pl, i64 tl, i64 common, double c) /* Jaro_impl.hpp:60-71 */
{
    if (!common) return false;
    double sim = ddiv((double)common, (double)pl);
    sim = dadd(sim, ddiv((double)common, (double)tl));
    sim = dadd(sim, 1.0);
    sim = ddiv(sim, 3.0);
    return sim >= c;
}

/* jaro_similarity (Jaro_impl.hpp:409-454) from exact counts; needs_counts() tells
 * whether the counts are read at all */
RFG_HD bool jaro_needs_counts(i64 pl, i64 tl, double c)
{
    if (c > 1.0) return false;
    if (!pl && !tl) return false;
    if (!jaro_length_filter(pl, tl, c)) return false;
    return true;
}

RFG_HD double jaro_from_counts(i64 pl, i64 tl, i64 common, i64 transp, double c)
{
    if (c > 1.0) return 0.0;
    if (!pl && !tl) return 1.0;
    if (!jaro_length_filter(pl, tl, c)) return 0.0;
    if (pl == 1 && tl == 1) return (double)(common == 1);
    if (!jaro_common_filter(pl, tl, common, c)) return 0.0;
    const double sim = jaro_formula(pl, tl, common, transp);
    return sim >= c ? sim : 0;
}

/* jaro_winkler_similarity's cutoff for the inner Jaro (JaroWinkler_impl.hpp:54-62) */
RFG_HD double jw_jaro_cutoff(i64 prefix, double pw, double c)
{
    double jc = c;
    if (jc > 0.7) {
        const double ps = dmul((double)prefix, pw);
        if (ps >= 1.0) jc = 0.7;
        else jc = dmax(0.7, ddiv(dsub(ps, jc), dsub(ps, 1.0)));
    }
    return jc;
}

/* the Winkler boost and final cutoff (JaroWinkler_impl.hpp:64-70) */
RFG_HD double jw_finish(double sim, i64 prefix, double pw, double c)
{
    if (sim > 0.7) {
        sim = dadd(sim, dmul(dmul((double)prefix, pw), dsub(1.0, sim)));
        sim = dmin(sim, 1.0);
    }
    return sim >= c ? sim : 0;
}

/* MultiJaro (jaro_similarity_simd, Jaro_impl.hpp:818-840, 666-709) */
RFG_HD double multi_jaro_from_counts(i64 pl, i64 tl, i64 common, i64 transp, double c)
{
    if (c > 1.0) return 0.0;
    if (tl == 0) return pl ? 0.0 : 1.0;
    if (!jaro_common_filter(pl, tl, common, c)) return 0.0;
    const double sim = jaro_formula(pl, tl, common, transp);
    return sim >= c ? sim : 0;
}

/* MultiJaroWinkler::_similarity (JaroWinkler.hpp:123-145) */
RFG_HD double multi_jw(double s, i64 prefix, double pw, double c)
{
    if (s > 0.7) {
        s = dadd(s, dmul(dmul((double)prefix, pw), dsub(1.0, s)));
        s = dmin(s, 1.0);
    }
    if (s < c) s = 0.0;
    return s;
}

/* the similarity cutoff that a double similarity-type chain passes on (maximum 1.0):
 * SimilarityBase::_distance and the normalized bases (distance.hpp:52-76, 177-190) */
RFG_HD double fsim_chain_cutoff(int op, double cf)
{
    switch (op) {
    case SIMILARITY: return cf;
    case DISTANCE: return 1.0 >= cf ? dsub(1.0, cf) : 0.0;
    case NORM_DISTANCE: {
        const double cd = dceil(dmul(1.0, cf));
        return 1.0 >= cd ? dsub(1.0, cd) : 0.0;
    }
    default: {
        const double cd = dceil(dmul(1.0, norm_sim_to_norm_dist(cf)));
        return 1.0 >= cd ? dsub(1.0, cd) : 0.0;
    }
    }
}

RFG_HD double fsim_chain_finish(int op, double s, double cf)
{
    switch (op) {
    case SIMILARITY: return s;
    case DISTANCE: {
        const double d = dsub(1.0, s);
        return d <= cf ? d : 1.0;
    }
    case NORM_DISTANCE: {
        const double cd = dceil(dmul(1.0, cf));
        double d = dsub(1.0, s);
        d = d <= cd ? d : 1.0;
        const double nd = ddiv(d, 1.0);
        return nd <= cf ? nd : 1.0;
    }
    default: {
        const double c2 = norm_sim_to_norm_dist(cf);
        const double cd = dceil(dmul(1.0, c2));
        double d = dsub(1.0, s);
        d = d <= cd ? d : 1.0;
        double nd = ddiv(d, 1.0);
        nd = nd <= c2 ? nd : 1.0;
        const double ns = dsub(1.0, nd);
        return ns >= cf ? ns : 0.0;
    }
    }
}

RFG_HD double multi_fsim_finish(int op, double s_at_cf, double s_at_0, double cf)
{
    switch (op) {
    case SIMILARITY: return s_at_cf;
    case DISTANCE: {
        const double d = dsub(1.0, s_at_0);
        return d <= cf ? d : 1.0;
    }
    case NORM_DISTANCE: {
        double d = dsub(1.0, s_at_0);
        d = d <= 1.0 ? d : 1.0;
        return d <= cf ? d : 1.0;
    }
    default: {
        double d = dsub(1.0, s_at_0);
        d = d <= 1.0 ? d : 1.0;
        const double ns = dsub(1.0, d);
        return ns >= cf ? ns : 0.0;
    }
    }
}

/* ================================================= per-pair plan and finish
 * Integer-valued metrics: the core result `raw` (a distance, or an LCS length, or -1
 * for "pruned") is turned into the API result.  l1/l2 are the string lengths. */

struct PairSpec {
    int metric, op, form;
    u64 l1, l2;
    u64 ci;
    double cf;
    ScoreParams p;
    u64 kd_pre = ~0ull; /* precomputed chain cutoff of a normalized op (chain_kd), or ~0 */
};

/* The internal distance cutoff of a normalized op's chain for (l1, l2): ceil(M * c)
 * with M the metric's maximum and c the cutoff the chain hands down.  Depends only on the
 * lengths, so kernels tabulate it per query.  ~0 for ops without one. */
RFG_HD u64 chain_kd(const PairSpec& s)
{
    if (s.form == FORM_MULTI) return ~0ull;
    const int op = s.metric == RATIO ? NORM_SIMILARITY : s.op;
    if (op != NORM_DISTANCE && op != NORM_SIMILARITY) return ~0ull;
    const double cf = s.metric == RATIO ? ddiv(s.cf, 100.0) : s.cf;
    const double c = op == NORM_DISTANCE ? cf : norm_sim_to_norm_dist(cf);
    u64 M;
    switch (s.metric) {
    case LEVENSHTEIN: M = lev_maximum(s.l1, s.l2, s.p); break;
    case INDEL:
    case RATIO: M = s.l1 + s.l2; break;
    case OSA:
    case LCSSEQ: M = s.l1 > s.l2 ? s.l1 : s.l2; break;
    default: return ~0ull;
    }
    return ceil_cut(M, c);
}

/* plan for integer families; returns the plan (run == 0: no core needed) */
RFG_HD Plan plan_int(const PairSpec& s)
{
    Plan pl;
    pl.run = 1;
    pl.K = 0;
    pl.Kchain = 0;
    pl.jc = 0;
    pl.lcs_min = 0;
    const u64 l1 = s.l1, l2 = s.l2;
    const u64 BIG = ~0ull;
    if (s.form == FORM_MULTI) {
        /* exact values; only the distance op carries its cutoff into the core */
        const u64 K = (s.op == DISTANCE && s.metric != LCSSEQ) ? s.ci : BIG;
        if (s.metric == LEVENSHTEIN || s.metric == OSA) pl.K = clamp_bound(K);
        else pl.K = clamp_bound(BIG); /* LCS families: exact LCS */
        return pl;
    }
    switch (s.metric) {
    case LEVENSHTEIN: {
        const u64 M = lev_maximum(l1, l2, s.p);
        u64 Kw;
        if (s.kd_pre != ~0ull && s.op >= NORM_DISTANCE) Kw = s.kd_pre;
        else if (!dist_chain_cutoff(s.op, M, s.ci, s.cf, &Kw)) {
            pl.run = 0;
            return pl;
        }
        pl.Kchain = Kw;
        switch (lev_mode(s.p)) {
        case LEV_ZERO: pl.run = 0; break;
        case LEV_UNIFORM:
        case LEV_INDEL: pl.K = clamp_bound(s.p.ins == 1 ? Kw : ceil_div_u(Kw, (u64)s.p.ins)); break;
        default: pl.K = clamp_bound(Kw);
        }
        return pl;
    }
    case INDEL:
    case RATIO: {
        const u64 M = l1 + l2;
        u64 K;
        const int op = s.metric == RATIO ? NORM_SIMILARITY : s.op;
        if (s.kd_pre != ~0ull && op >= NORM_DISTANCE) K = s.kd_pre;
        else if (op >= NORM_DISTANCE) K = norm_cut(op, M, s.cf, s.metric == RATIO);
        else if (!dist_chain_cutoff(op, M, s.ci, s.cf, &K)) {
            pl.run = 0;
            return pl;
        }
        pl.Kchain = K;
        pl.K = clamp_bound(K);
        return pl;
    }
    case OSA: {
        const u64 M = l1 > l2 ? l1 : l2;
        u64 K;
        if (s.kd_pre != ~0ull && s.op >= NORM_DISTANCE) K = s.kd_pre;
        else if (!dist_chain_cutoff(s.op, M, s.ci, s.cf, &K)) {
            pl.run = 0;
            return pl;
        }
        pl.Kchain = K;
        pl.K = clamp_bound(K);
        return pl;
    }
    case LCSSEQ: {
        const u64 M = l1 > l2 ? l1 : l2;
        u64 cs;
        switch (s.op) {
        case SIMILARITY: cs = s.ci; break;
        case DISTANCE: cs = M >= s.ci ? M - s.ci : 0; break;
        case NORM_DISTANCE: {
            const u64 Kd = s.kd_pre != ~0ull ? s.kd_pre : norm_cut(NORM_DISTANCE, M, s.cf, 0);
            pl.Kchain = Kd;
            cs = M >= Kd ? M - Kd : 0;
            break;
        }
        default: {
            const u64 Kd = s.kd_pre != ~0ull ? s.kd_pre : norm_cut(NORM_SIMILARITY, M, s.cf, 0);
            pl.Kchain = Kd;
            cs = M >= Kd ? M - Kd : 0;
        }
        }
        pl.lcs_min = cs;
        if (cs > l1 || cs > l2) {
            pl.run = 0; /* lcs_seq_similarity returns 0 (LCSseq_impl.hpp:382) */
            return pl;
        }
        pl.K = (i64)(l1 + l2 - 2 * cs);
        return pl;
    }
    }
    pl.run = 0;
    return pl;
}

/* The first band of the score-hint doubling for a unit-weight Levenshtein pair: the
 * caller's score_hint as a distance bound, converted by the op's chain the way the
 * reference's wrappers convert it (distance.hpp: similarity hint -> maximum - hint,
 * normalized hints -> ceil(maximum * hint) of the distance form).  Any value gives the
 * same results (a band whose distance exceeds its bound is discarded); the hint only
 * sets how much work the first band does. */
RFG_HD i64 lev_hint_bound(const PairSpec& s, u64 hint_i, double hint_f)
{
    const u64 M = lev_maximum(s.l1, s.l2, s.p);
    double c;
    switch (s.op) {
    case DISTANCE: return clamp_bound(hint_i);
    case SIMILARITY: return hint_i >= M ? 0 : (i64)(M - hint_i);
    case NORM_DISTANCE: c = hint_f; break;
    default: c = dsub(1.0, hint_f);
    }
    if (!(c >= 0.0)) return 0;
    if (!(c < 1.0)) return (i64)M;
    return (i64)ceil_cut(M, c);
}

/* Finish for integer families.  raw: LEV/OSA/WF -> distance (> K when pruned);
 * LCS -> LCS length, or -1 when pruned.  Ignored when plan.run == 0. */
RFG_HD void finish_int(const PairSpec& s, const Plan& pl, i64 raw, i64* oi, double* of)
{
    const u64 l1 = s.l1, l2 = s.l2;
    if (s.form == FORM_MULTI) {
        switch (s.metric) {
        case LEVENSHTEIN: multi_dist_finish(s.op, lev_maximum(l1, l2, s.p), (u64)raw, s.ci, s.cf, oi, of); return;
        case OSA: multi_dist_finish(s.op, l1 > l2 ? l1 : l2, (u64)raw, s.ci, s.cf, oi, of); return;
        case INDEL: multi_dist_finish(s.op, l1 + l2, l1 + l2 - 2 * (u64)raw, s.ci, s.cf, oi, of); return;
        case LCSSEQ: multi_sim_finish(s.op, l1 > l2 ? l1 : l2, (u64)raw, s.ci, s.cf, oi, of); return;
        case RATIO: {
            double r = 0;
            multi_dist_finish(NORM_SIMILARITY, l1 + l2, l1 + l2 - 2 * (u64)raw, 0, ddiv(s.cf, 100.0), oi, &r);
            *of = dmul(r, 100.0);
            return;
        }
        }
        return;
    }
    switch (s.metric) {
    case LEVENSHTEIN: {
        const u64 M = lev_maximum(l1, l2, s.p);
        if (!pl.run && lev_mode(s.p) != LEV_ZERO) { /* similarity with cutoff above the maximum */
            *oi = 0;
            return;
        }
        const u64 Kw = pl.Kchain;
        u64 d;
        switch (lev_mode(s.p)) {
        case LEV_ZERO: d = 0; break;
        case LEV_UNIFORM: {
            const u64 Kb = (u64)pl.K;
            u64 b = (raw >= 0 && (u64)raw <= Kb) ? (u64)raw : Kb + 1;
            d = b * (u64)s.p.ins;
            d = d <= Kw ? d : Kw + 1;
            break;
        }
        case LEV_INDEL: {
            /* raw is an LCS length (or -1): indel distance = l1 + l2 - 2 lcs */
            const u64 Kb = (u64)pl.K;
            u64 b = raw >= 0 ? l1 + l2 - 2 * (u64)raw : Kb + 1;
            b = b <= Kb ? b : Kb + 1;
            d = b * (u64)s.p.ins;
            d = d <= Kw ? d : Kw + 1;
            break;
        }
        default: d = (u64)raw <= Kw ? (u64)raw : Kw + 1;
        }
        if (lev_mode(s.p) == LEV_ZERO) {
            /* _distance returns 0 without a cutoff check; the chain still runs */
            u64 K2;
            if (!dist_chain_cutoff(s.op, M, s.ci, s.cf, &K2)) {
                *oi = 0;
                return;
            }
        }
        dist_chain_finish(s.op, M, d, s.ci, s.cf, oi, of, lev_mode(s.p) == LEV_ZERO ? ~0ull : Kw);
        return;
    }
    case INDEL:
    case RATIO: {
        const u64 M = l1 + l2;
        if (!pl.run) {
            *oi = 0;
            return;
        }
        const u64 K = pl.Kchain;
        u64 d = raw >= 0 ? M - 2 * (u64)raw : K + 1;
        d = d <= K ? d : K + 1;
        if (s.metric == RATIO) /* |c| <= 200 percent implies c / 100 <= 2: ratio_finish's shortcut, inline */
            *of = (M != 0 && d > K && abs_le_bits(s.cf, 200.0)) ? 0.0 : ratio_finish(M, d, s.cf, K);
        else dist_chain_finish(s.op, M, d, s.ci, s.cf, oi, of, K);
        return;
    }
    case OSA: {
        const u64 M = l1 > l2 ? l1 : l2;
        if (!pl.run) {
            *oi = 0;
            return;
        }
        const u64 K = pl.Kchain;
        const u64 d = (u64)raw <= K ? (u64)raw : K + 1;
        dist_chain_finish(s.op, M, d, s.ci, s.cf, oi, of, K);
        return;
    }
    case LCSSEQ: {
        const u64 M = l1 > l2 ? l1 : l2;
        const u64 cs = pl.lcs_min;
        u64 sim = 0;
        if (pl.run && raw >= 0 && (u64)raw >= cs) sim = (u64)raw;
        switch (s.op) {
        case SIMILARITY: *oi = (i64)sim; return;
        case DISTANCE: {
            const u64 d = M - sim;
            *oi = (i64)(d <= s.ci ? d : s.ci + 1);
            return;
        }
        case NORM_DISTANCE: {
            const u64 Kd = pl.Kchain;
            u64 d = M - sim;
            d = d <= Kd ? d : Kd + 1;
            if (d > Kd && M != 0 && s.cf <= 2.0 && s.cf >= -2.0) { /* see dist_chain_finish */
                *of = 1.0;
                return;
            }
            const double nd = M != 0 ? ddiv((double)d, (double)M) : 0.0;
            *of = nd <= s.cf ? nd : 1.0;
            return;
        }
        default: {
            const u64 Kd = pl.Kchain;
            const double c2 = norm_sim_to_norm_dist(s.cf);
            u64 d = M - sim;
            d = d <= Kd ? d : Kd + 1;
            if (d > Kd && M != 0 && s.cf <= 2.0 && s.cf >= -2.0) {
                *of = 0.0;
                return;
            }
            double nd = M != 0 ? ddiv((double)d, (double)M) : 0.0;
            nd = nd <= c2 ? nd : 1.0;
            const double ns = dsub(1.0, nd);
            *of = ns >= s.cf ? ns : 0.0;
            return;
        }
        }
    }
    }
}

/* Jaro families.  prefix: common prefix (<= 4) of the two strings. */
/* The band classes of the band kernel: 32-bit words of window */
#define BAND_CLASSES 8
RFG_HD int band_class_words(int i)
{
    const int w[BAND_CLASSES] = {1, 2, 3, 4, 6, 8, 12, 16};
    return w[i];
}

/* The metrics the band kernel takes: unit-weight Levenshtein, and the LCS families
 * (Indel, LCSseq, ratio), whose plans carry an Indel-distance bound K (plan_int) */
RFG_HD bool band_metric(int metric, const ScoreParams& sp)
{
    if (metric == LEVENSHTEIN) return sp.ins == 1 && sp.del == 1 && sp.rep == 1;
    return metric == INDEL || metric == LCSSEQ || metric == RATIO;
}

/* The choice lengths whose pairs with a pattern of m units pass the length filter
 * |m - n| <= K(n) (Levenshtein_impl.hpp:863, LCSseq_impl.hpp:389) for a band metric:
 * [*nlo, *nhi] within [1, max(m, maxlen)], holding every passing length (the rest of
 * the interval may hold lengths that fail), and an upper bound *Kmax of the bound K any
 * passing pair gets.
 *   - n <= m: K(n) <= K(m) (Levenshtein, LCSseq distance and similarity: one value or
 *     falling with m - n; Indel and ratio: K rises with n), so every passing n is at
 *     least m - K(m);
 *   - n > m: K(n) - (n - m) does not grow with n (the distance ops: K(n) = ci, n - ci,
 *     m + n - ci, min(m + n, 2 ci - (n - m)) or m + n - 2 ci; the normalized ops, cutoff c in [0, 1]:
 *     K(n) = ceil(fl(M c)) (LCSseq: twice that less n - m) rises by at most 1 per unit of
 *     the maximum M, fl being monotone and exact at integers), so the passing n > m form
 *     one run that a binary search ends.  K(n) there is largest at the run's end except
 *     for LCSseq (normalized: K moves by +1 or -1 per unit of n; distance: K = m + n
 *     while max(m, n) < ci, 2 ci - (n - m) after), whose run is scanned.
 * n = 0 never reaches the core.  Returns false when no pair passes (or the cutoff is
 * outside the range the argument covers). */
RFG_HD bool band_range(int metric, int op, int form, const ScoreParams& sp, u64 ci, double cf, i64 m, i64 maxlen,
                       i64* nlo, i64* nhi, i64* Kmax)
{
    if (m < 1 || !band_metric(metric, sp) || form == FORM_MULTI) return false;
    if (metric == RATIO ? !(cf >= 0.0 && cf <= 100.0)
                        : (op == NORM_DISTANCE || op == NORM_SIMILARITY) && !(cf >= 0.0 && cf <= 1.0))
        return false;
    PairSpec s;
    s.metric = metric;
    s.op = op;
    s.form = form;
    s.ci = ci;
    s.cf = cf;
    s.p = sp;
    s.l1 = (u64)m;
    s.kd_pre = ~0ull;
    auto bound = [&](i64 n, bool* pass) -> i64 {
        s.l2 = (u64)n;
        const Plan pl = plan_int(s);
        if (!pl.run) {
            *pass = false;
            return -1;
        }
        *pass = pl.K >= (n > m ? n - m : m - n);
        return pl.K;
    };
    bool pass = false;
    const i64 Km = bound(m, &pass);
    if (!pass) return false;
    i64 lo = m;
    if (maxlen > m) {
        i64 hi = maxlen; /* lo passes; find the last passing n */
        while (lo < hi) {
            const i64 mid = lo + (hi - lo + 1) / 2;
            bool p;
            bound(mid, &p);
            if (p) lo = mid;
            else hi = mid - 1;
        }
    }
    bool p;
    i64 Khi = bound(lo, &p);
    if (metric == LCSSEQ)
        for (i64 n = m + 1; n < lo; ++n) {
            const i64 k = bound(n, &p);
            Khi = k > Khi ? k : Khi;
            if (Khi > 1024) { /* no band class holds it: K <= m + n bounds the rest */
                Khi = m + lo;
                break;
            }
        }
    *nlo = m - Km > 1 ? m - Km : 1;
    *nhi = lo;
    *Kmax = Khi > Km ? Khi : Km;
    return true;
}

/* The band class of a pattern of m units against choices of at most maxlen units: the
 * index of the narrowest band_class_words width holding Ukkonen's band (about K + 2
 * diagonals) of every pair that passes the length filter, or -1 when the band is not
 * narrower than the pattern (or wider than 512 bits). */
RFG_HD int band_class(int metric, int op, int form, const ScoreParams& sp, u64 ci, double cf, i64 m, i64 maxlen)
{
    i64 nlo, nhi, Kmax;
    if (m < 2 || !band_range(metric, op, form, sp, ci, cf, m, maxlen, &nlo, &nhi, &Kmax)) return -1;
    const i64 bits = Kmax + 2;
    if (Kmax < 0 || bits >= m || bits > 512) return -1;
    const int words = (int)((bits + 31) / 32);
    for (int i = 0; i < BAND_CLASSES; ++i)
        if (band_class_words(i) >= words) return i;
    return -1;
}

/* The result of every pair of a band-class pattern that fails the length filter (the
 * chain's value for the pruned distance K + 1, which depends on neither length):
 * distance K + 1 with K the cutoff (fast: fast_k; LCSseq: the LCS is 0, the distance the
 * maximum, which exceeds the cutoff), similarity 0, normalized distance 1.0, normalized
 * similarity and ratio 0.0 -- the pruned-pair shortcuts of dist_chain_finish and
 * ratio_finish, which hold for cutoffs in [0, 1] (ratio: [0, 100]; band_range refuses
 * others). */
RFG_HD void band_reject_value(int metric, int op, u64 ci, int fast, i64 fast_k, i64* vi, double* vf)
{
    *vi = 0;
    *vf = 0.0;
    if (metric == RATIO) return;
    switch (op) {
    case DISTANCE: *vi = (fast ? fast_k : clamp_bound(ci)) + 1; break;
    case SIMILARITY: break;
    case NORM_DISTANCE: *vf = 1.0; break;
    default: break;
    }
}

RFG_HD double jaro_cutoff_for(const PairSpec& s, i64 prefix)
{
    if (s.form == FORM_MULTI) return 0.0; /* Multi: counts are always read */
    const double c = fsim_chain_cutoff(s.op, s.cf);
    return s.metric == JARO ? c : jw_jaro_cutoff(prefix, s.p.prefix_weight, c);
}

RFG_HD bool jaro_pair_needs_counts(const PairSpec& s, i64 prefix)
{
    if (s.form == FORM_MULTI) return s.l2 != 0;
    return jaro_needs_counts((i64)s.l1, (i64)s.l2, jaro_cutoff_for(s, prefix));
}

/* ---------------------------------------------------------- partial_ratio
 * fuzz::partial_ratio / CachedPartialRatio::similarity (fuzz_impl.hpp:49-293) for a
 * query q (pattern table pm, W words) and a choice c, both given as resolved rows.
 * Every LCS runs on the query's table: against windows of the choice directly, and
 * with the query in the haystack role through a shifted view of the table (the table
 * of q[a, a+L) is bits a..a+L-1 of q's table), so no per-pair table is built.
 * Scratch: st holds W + 1 state words; work holds 5 * |m - n| + 2 32-bit slots. */

/* pattern table of q[a, a + L) from q's table */
template <typename PMW>
struct PMShift {
    const PMW* pm;
    int W, a, L;
    RFG_HD u64 operator()(u64 c, int w) const
    {
        const int bit = a + 64 * w, w0 = bit >> 6, sh = bit & 63;
        u64 x = w0 < W ? (*pm)(c, w0) >> sh : 0;
        if (sh && w0 + 1 < W) x |= (*pm)(c, w0 + 1) << (64 - sh);
        const int rem = L - 64 * w;
        return rem >= 64 ? x : x & low_mask(rem < 0 ? 0 : rem);
    }
};

/* bits [a, a + 64) of row c of a W-word table (zero outside it) */
template <typename PMW>
RFG_HD u64 pm_bits(const PMW& pm, int W, u64 c, int a)
{
    if (a <= -64 || a >= 64 * W) return 0;
    if (a < 0) return pm(c, 0) << (-a);
    const int w0 = a >> 6, sh = a & 63;
    u64 x = pm(c, w0) >> sh;
    if (sh && w0 + 1 < W) x |= pm(c, w0 + 1) << (64 - sh);
    return x;
}

RFG_HD u64 bitrev64(u64 x)
{
#ifdef __CUDA_ARCH__
    return __brevll(x);
#else
    x = ((x >> 1) & 0x5555555555555555ull) | ((x & 0x5555555555555555ull) << 1);
    x = ((x >> 2) & 0x3333333333333333ull) | ((x & 0x3333333333333333ull) << 2);
    x = ((x >> 4) & 0x0F0F0F0F0F0F0F0Full) | ((x & 0x0F0F0F0F0F0F0F0Full) << 4);
    x = ((x >> 8) & 0x00FF00FF00FF00FFull) | ((x & 0x00FF00FF00FF00FFull) << 8);
    x = ((x >> 16) & 0x0000FFFF0000FFFFull) | ((x & 0x0000FFFF0000FFFFull) << 16);
    return (x >> 32) | (x << 32);
#endif
}

/* pattern table of the reversed pattern q[m-1], ..., q[0] from q's table */
template <typename PMW>
struct PMRev {
    const PMW* pm;
    int W, m;
    RFG_HD u64 operator()(u64 c, int w) const
    {
        /* reversed bits 64w .. 64w+63 are q's bits m-1-64w down to m-64-64w */
        const u64 r = bitrev64(pm_bits(*pm, W, c, m - 64 - 64 * w));
        const int rem = m - 64 * w;
        return rem >= 64 ? r : r & low_mask(rem < 0 ? 0 : rem);
    }
};

/* text rows read backwards: t[len-1], t[len-2], ... */
template <typename TXT>
struct RevText {
    const TXT* t;
    int len;
    RFG_HD u64 operator[](int j) const { return (*t)[len - 1 - j]; }
};

/* Hyyro's LCS bit vector over the first T units of t (S: W words); after(j) runs after
 * unit j.  LCS(pattern[0, i), text so far) = lcs_count(S, W, i). */
template <typename PMW, typename TXT, typename F>
RFG_HD void lcs_stream(const PMW& pm, int W, const TXT& t, int T, u64* S, F after)
{
    for (int w = 0; w < W; ++w) S[w] = ~0ull;
    for (int j = 0; j < T; ++j) {
        const u64 c = t[j];
        u32 carry = 0;
        for (int w = 0; w < W; ++w) {
            const u64 X = pm(c, w);
            const u64 sv = S[w];
            const u64 u = sv & X;
            const u64 x = add_carry(sv, u, carry, &carry);
            S[w] = x | (sv - u);
        }
        after(j);
    }
}

RFG_HD u64 lcs_count(const u64* S, int W, int i)
{
    u64 l = 0;
    for (int w = 0; w < W && 64 * w < i; ++w) l += popc64(~S[w] & low_mask(i - 64 * w));
    return l;
}

/* text rows t[a, a + L) */
template <typename TXT>
struct TextSlice {
    const TXT* t;
    int a;
    RFG_HD u64 operator[](int j) const { return (*t)[a + j]; }
};

/* a * b >= c * d over 128-bit products */
RFG_HD bool prod_ge(u64 a, u64 b, u64 c, u64 d)
{
#ifdef __CUDA_ARCH__
    const u64 h1 = __umul64hi(a, b), h2 = __umul64hi(c, d);
    return h1 != h2 ? h1 > h2 : a * b >= c * d;
#else
    return (unsigned __int128)a * b >= (unsigned __int128)c * d;
#endif
}

/* CachedRatio::similarity from an exact LCS (fuzz_impl.hpp:43-47 over the Indel chain) */
RFG_HD double ratio_from_lcs(u64 l1, u64 l2, u64 lcs, double cutoff)
{
    const u64 M = l1 + l2;
    const u64 K = norm_cut(NORM_SIMILARITY, M, cutoff, 1);
    u64 d = M - 2 * lcs;
    d = d <= K ? d : K + 1;
    return (M != 0 && d > K && abs_le_bits(cutoff, 200.0)) ? 0.0 : ratio_finish(M, d, cutoff, K);
}

/* partial_ratio_impl with needle = q (QN = true: q shorter or equal) or needle = c */
template <bool QN, typename PMW, typename TXT>
RFG_HD double partial_impl_dev(const PMW& pm, int W, int m, const TXT& c, int n, double cutoff, u64* st, u32* work)
{
    const int len1 = QN ? m : n, len2 = QN ? n : m;
    double res = 0.0;
    u64 bd = 1, bM = 1; /* res = 0 as the fraction 1 / 1 */
    /* LCS of the needle against haystack[a, a + L) */
    auto lcs_at = [&](int a, int L) -> u64 {
        if (QN) {
            const TextSlice<TXT> sub{&c, a};
            return m ? (u64)lcs_multi_rt(pm, W, m, sub, L, (i64)1 << 62, st) : 0;
        }
        const PMShift<PMW> pq{&pm, W, a, L};
        return L ? (u64)lcs_multi_rt(pq, (L + 63) / 64, L, c, n, (i64)1 << 62, st) : 0;
    };
    /* does the needle hold the haystack unit at position i */
    auto needle_has = [&](int i) -> bool {
        if (QN) {
            const u64 r = c[i];
            for (int w = 0; w < W; ++w)
                if (pm(r, w)) return true;
            return false;
        }
        /* the haystack is q: q[i] occurs in c when some c[j] has bit i in q's table */
        const int bit = i;
        for (int j = 0; j < n; ++j) {
            const u64 r = c[j];
            if ((pm(r, bit >> 6) >> (bit & 63)) & 1u) return true;
        }
        return false;
    };
    if (len2 > len1) {
        const u64 maximum = (u64)len1 * 2;
        u64 cutoff_dist = ceil_cut(maximum, norm_sim_to_norm_dist(ddiv(cutoff, 100.0)));
        u64 best = ~0ull;
        const int L = len2 - len1;
        const u32 NONE = 0xffffffffu;
        u32* scores = work;
        u32* wa = work + L;          /* windows of this level: pairs */
        u32* wb = work + 3 * L + 1;  /* windows of the next level */
        for (int i = 0; i < L; ++i) scores[i] = NONE;
        int na = 1, nb = 0;
        wa[0] = 0;
        wa[1] = (u32)(L - 1);
        while (na) {
            for (int k = 0; k < na; ++k) {
                const int first = (int)wa[2 * k], second = (int)wa[2 * k + 1];
                for (int e = 0; e < 2; ++e) {
                    const int pos = e ? second : first;
                    if (scores[pos] != NONE) continue;
                    const u64 lcs = lcs_at(pos, len1);
                    scores[pos] = (u32)(2 * (u64)len1 - 2 * lcs);
                    if ((u64)scores[pos] < cutoff_dist) {
                        cutoff_dist = best = scores[pos];
                        if (best == 0) return 100.0;
                    }
                }
                const u64 cell_diff = (u64)(second - first);
                if (cell_diff == 1) continue;
                const u64 sa = scores[first], sb = scores[second];
                const u64 known = sa > sb ? sa - sb : sb - sa;
                const u64 max_imp = (cell_diff - known / 2) / 2 * 2;
                const i64 min_score = (i64)(sa < sb ? sa : sb) - (i64)max_imp;
                if (min_score < (i64)cutoff_dist) {
                    const int center = (int)(cell_diff / 2);
                    wb[2 * nb] = (u32)first;
                    wb[2 * nb + 1] = (u32)(first + center);
                    wb[2 * nb + 2] = (u32)(first + center);
                    wb[2 * nb + 3] = (u32)second;
                    nb += 2;
                }
            }
            u32* tmp = wa;
            wa = wb;
            wb = tmp;
            na = nb;
            nb = 0;
        }
        double score = dsub(1.0, ddiv((double)best, (double)maximum));
        score = dmul(score, 100.0);
        if (score >= cutoff) {
            cutoff = res = score;
            bd = best;
            bM = maximum;
        }
    }
    /* res is f(bd, bM) with f(d, M) = (1 - d / M) * 100 in correctly rounded steps, which
     * never increases with d / M: a candidate with d * bM >= bd * M cannot beat res, so
     * only the others pay the double-precision chain (a negative res, possible only
     * under a negative cutoff, turns the test off) */
    const bool pf = res >= 0.0;
    /* the cutoff side: the chain prunes d > ceil(M * c_nd) to 0; with cfix >= c_nd * 2^32,
     * floor(M * cfix / 2^32) + 2 bounds that integer cutoff from above */
    u64 cfix = 0;
    auto set_cfix = [&]() {
        const double cnd = norm_sim_to_norm_dist(ddiv(cutoff, 100.0));
        cfix = cnd >= 2.0 ? ~0ull : (u64)dceil(dmul(cnd, 4294967296.0)) + 1;
    };
    set_cfix();
    auto may_beat = [&](u64 L2, u64 lcs) {
        if (!pf) return true;
        const u64 M = (u64)len1 + L2, d = M - 2 * lcs;
        if (cfix != ~0ull) {
#ifdef __CUDA_ARCH__
            const u64 hi = __umul64hi(M, cfix), lo = M * cfix;
            const u64 kup = ((hi << 32) | (lo >> 32)) + 2;
#else
            const u64 kup = (u64)(((unsigned __int128)M * cfix) >> 32) + 2;
#endif
            if (d > kup) return false;
        }
        return !prod_ge(d, bM, bd, M);
    };
    /* prefixes and suffixes of the haystack shorter than the needle: every LCS of one
     * family comes from a single bit-vector pass (text prefixes are the pass's steps,
     * pattern prefixes the final vector's low bits; suffixes are prefixes of the reversed
     * strings), kept in lbuf[length] -- the window search no longer needs work */
    u32* lbuf = work;
    const PMRev<PMW> pr{&pm, W, m};
    const RevText<TXT> rc{&c, n};
    if (QN) {
        if (len1 > 1) lcs_stream(pm, W, c, len1 - 1, st, [&](int j) { lbuf[j + 1] = (u32)lcs_count(st, W, m); });
    }
    else {
        lcs_stream(pm, W, c, n, st, [](int) {});
        for (int i = 1; i < len1; ++i) lbuf[i] = (u32)lcs_count(st, W, i);
    }
    for (int i = 1; i < len1; ++i) {
        if (!needle_has(i - 1) || !may_beat((u64)i, lbuf[i])) continue;
        const double r = ratio_from_lcs((u64)len1, (u64)i, lbuf[i], cutoff);
        if (r > res) {
            cutoff = res = r;
            bM = (u64)len1 + i;
            bd = bM - 2 * (u64)lbuf[i];
            if (res == 100.0) return res;
            set_cfix();
        }
    }
    if (QN) lcs_stream(pr, W, rc, len1, st, [&](int k) { lbuf[k + 1] = (u32)lcs_count(st, W, m); });
    else {
        lcs_stream(pr, W, rc, n, st, [](int) {});
        for (int L = 1; L <= len1; ++L) lbuf[L] = (u32)lcs_count(st, W, L);
    }
    for (int i = len2 - len1; i < len2; ++i) {
        if (!needle_has(i) || !may_beat((u64)(len2 - i), lbuf[len2 - i])) continue;
        const double r = ratio_from_lcs((u64)len1, (u64)(len2 - i), lbuf[len2 - i], cutoff);
        if (r > res) {
            cutoff = res = r;
            bM = (u64)len1 + (len2 - i);
            bd = bM - 2 * (u64)lbuf[len2 - i];
            if (res == 100.0) return res;
            set_cfix();
        }
    }
    return res;
}

/* partial_ratio_alignment(q, c, cutoff).score (fuzz_impl.hpp:194-227) */
template <typename PMW, typename TXT>
RFG_HD double partial_ratio_dev(const PMW& pm, int W, int m, const TXT& c, int n, double cutoff, u64* st, u32* work)
{
    if (cutoff > 100) return 0.0;
    if (!m || !n) return (double)(m == n) * 100.0;
    if (m > n) return partial_impl_dev<false>(pm, W, m, c, n, cutoff, st, work);
    const double score = partial_impl_dev<true>(pm, W, m, c, n, cutoff, st, work);
    if (score != 100 && m == n) {
        cutoff = dmax(cutoff, score);
        const double score2 = partial_impl_dev<false>(pm, W, m, c, n, cutoff, st, work);
        if (score2 > score) return score2;
    }
    return score;
}

/* ------------------------------------------------ token_set_ratio family
 * token_set_ratio, partial_token_set_ratio, token_ratio, partial_token_ratio and WRatio
 * (fuzz_impl.hpp:372-889).  A string of these metrics arrives as the concatenation of up
 * to three parts -- the string itself (WRatio), its sorted-split join S (tokens sorted,
 * repeats kept) and the join J of its deduplicated tokens -- with the part lengths beside
 * it; PMShift / TextSlice views give each part's pattern table and text, so the query's
 * table is built once.  set_decomposition (common_impl.hpp:11-35) is a merge of the two
 * sorted token streams of the S parts that skips repeats; the intersection and the
 * differences are never written out:
 *   - diff_ab.join() is a subsequence of q's S part (the kept tokens and one separator
 *     before each kept token but the first), so its LCS with any text is the LCS of S
 *     under a pattern table masked to those positions (a unit that matches nothing
 *     changes no LCS);
 *   - diff_ba.join() is the subsequence of c's S part walked with the kept-token bits,
 *     the other units are left out of the recurrence.
 * Tokens hold no U+0020 and the joins hold exactly one U+0020 between tokens. */

/* the tokens of a join part [pos, end) of a unit accessor */
template <typename R>
struct TokWalk {
    const R* r;
    int pos, end;
    int a, len, idx; /* current token [a, a + len), its index in the part */
    RFG_HD bool next()
    {
        if (pos >= end) return false;
        a = pos;
        while (pos < end && (*r)[pos] != 0x20) ++pos;
        len = pos - a;
        ++pos;
        ++idx;
        return true;
    }
};

/* lexicographic order of two tokens by code unit (unsigned) */
template <typename R1, typename R2>
RFG_HD int tok_cmp(const R1& x, int a, int la, const R2& y, int b, int lb)
{
    const int n = la < lb ? la : lb;
    for (int k = 0; k < n; ++k) {
        const u64 p = x[a + k], q = y[b + k];
        if (p != q) return p < q ? -1 : 1;
    }
    return la < lb ? -1 : (la > lb ? 1 : 0);
}

/* the distinct tokens of a sorted join, in order (SplittedSentenceView::dedupe,
 * SplittedSentenceView.hpp:48-54); total counts every token walked */
template <typename R>
struct UniqWalk {
    TokWalk<R> w;
    int pa, pl, total;
    RFG_HD bool next()
    {
        while (w.next()) {
            ++total;
            if (total > 1 && tok_cmp(*w.r, pa, pl, *w.r, w.a, w.len) == 0) continue;
            pa = w.a;
            pl = w.len;
            return true;
        }
        return false;
    }
};

struct TokSplit {
    int sect_len, ab_len, ba_len; /* joined lengths of the intersection and the differences */
    int sect_n, ab_n, ba_n;       /* their token counts */
    int na, nb;                   /* token counts before deduplication (word_count) */
};

RFG_HD void set_bits(u64* k, int lo, int hi)
{
    for (int i = lo; i < hi;) {
        const int w = i >> 6, b = i & 63, n = (hi - i) < (64 - b) ? (hi - i) : (64 - b);
        k[w] |= low_mask(n) << b;
        i += n;
    }
}

/* set_decomposition of q's part [qa, qa + qn) and c's part [ca, ca + cn) (S or J parts).
 * kq (kqw words, may be null): bits of q's part in diff_ab.join(); kc (kcw words, may be
 * null): one bit per token of c's part (repeats included) that is in diff_ba. */
template <typename RQ, typename RC>
RFG_HD TokSplit tok_split(const RQ& q, int qa, int qn, const RC& c, int ca, int cn, u64* kq, int kqw, u64* kc,
                          int kcw)
{
    TokSplit r{0, 0, 0, 0, 0, 0, 0, 0};
    for (int w = 0; kq && w < kqw; ++w) kq[w] = 0;
    for (int w = 0; kc && w < kcw; ++w) kc[w] = 0;
    UniqWalk<RQ> A{TokWalk<RQ>{&q, qa, qa + qn, 0, 0, -1}, 0, 0, 0};
    UniqWalk<RC> B{TokWalk<RC>{&c, ca, ca + cn, 0, 0, -1}, 0, 0, 0};
    bool ha = A.next(), hb = B.next();
    while (ha || hb) {
        const int cmp = !ha ? 1 : !hb ? -1 : tok_cmp(q, A.w.a, A.w.len, c, B.w.a, B.w.len);
        if (cmp == 0) {
            r.sect_len += A.w.len + (r.sect_n > 0);
            ++r.sect_n;
            ha = A.next();
            hb = B.next();
        }
        else if (cmp < 0) {
            if (kq) set_bits(kq, A.w.a - qa - (r.ab_n > 0), A.w.a - qa + A.w.len);
            r.ab_len += A.w.len + (r.ab_n > 0);
            ++r.ab_n;
            ha = A.next();
        }
        else {
            if (kc) kc[B.w.idx >> 6] |= 1ull << (B.w.idx & 63);
            r.ba_len += B.w.len + (r.ba_n > 0);
            ++r.ba_n;
            hb = B.next();
        }
    }
    r.na = A.total;
    r.nb = B.total;
    return r;
}

/* one step of Hyyro's LCS bit vector over W words */
template <typename PMW>
RFG_HD void lcs_step(const PMW& pm, int W, u64 c, u64* S)
{
    u32 carry = 0;
    for (int w = 0; w < W; ++w) {
        const u64 X = pm(c, w), sv = S[w], u = sv & X;
        const u64 x = add_carry(sv, u, carry, &carry);
        S[w] = x | (sv - u);
    }
}

/* a pattern table restricted to the positions of a mask */
template <typename PMW>
struct PMMask {
    const PMW* pm;
    const u64* k;
    RFG_HD u64 operator()(u64 c, int w) const { return (*pm)(c, w) & k[w]; }
};

/* One pass over c's S part (rows t[ca, ca + cn)): SA (may be null) runs the LCS of q's
 * whole S part (table pms, W words), SB the LCS of diff_ab.join() (table pms masked by
 * kq) with diff_ba.join() (the tokens whose kc bit is set, one separator between them). */
template <typename PMW, typename TXT>
RFG_HD void tok_lcs(const PMW& pms, int W, const u64* kq, const TXT& t, int ca, int cn, const u64* kc, u64* SA,
                    u64* SB)
{
    for (int w = 0; w < W; ++w) {
        if (SA) SA[w] = ~0ull;
        if (SB) SB[w] = ~0ull;
    }
    const PMMask<PMW> pmk{&pms, kq};
    int ti = 0;
    bool kept = SB && (kc[0] & 1), seen = false;
    for (int j = 0; j < cn; ++j) {
        const u64 ch = t[ca + j];
        if (SA) lcs_step(pms, W, ch, SA);
        if (!SB) continue;
        if (ch == 0x20) {
            ++ti;
            kept = (kc[ti >> 6] >> (ti & 63)) & 1;
            if (kept && seen) lcs_step(pmk, W, 0x20, SB);
            continue;
        }
        if (kept) {
            lcs_step(pmk, W, ch, SB);
            seen = true;
        }
    }
}

/* norm_distance, score_cutoff_to_distance (fuzz_impl.hpp:55-66) */
RFG_HD double norm_distance_pct(u64 dist, u64 lensum, double cutoff)
{
    const double score = lensum > 0 ? dsub(100.0, ddiv(dmul(100.0, (double)dist), (double)lensum)) : 100.0;
    return score >= cutoff ? score : 0.0;
}

RFG_HD u64 cutoff_to_distance(double cutoff, u64 lensum)
{
    return (u64)dceil(dmul((double)lensum, dsub(1.0, ddiv(cutoff, 100.0))));
}

/* one pair of the family: q's table over its whole concatenation (W words), q's units,
 * c's rows (table keys) and units, and the part lengths (original, S, J) of both */
template <typename PMW, typename RQ, typename TXT, typename RC>
struct TokPair {
    typedef PMW PMType;
    typedef TXT TxtType;
    const PMW* pm;
    int W;
    const RQ* q;
    const TXT* t;
    const RC* c;
    int q0, qs, qj, c0, cs, cj;
};

RFG_HD int words_of(int L) { return (L + 63) >> 6; }

/* per-thread scratch (words) of a pair whose concatenations are at most L units with a
 * W-word table: kq, SA, SB (W each), kc (one bit per token), then partial_ratio's state
 * words and window slots */
RFG_HD i64 tok_scratch_words(int W, i64 L) { return 3 * (i64)W + (L + 1) / 128 + 1 + W + 1 + (5 * L + 3) / 2; }

/* token_set_ratio (with_sorted = false; fuzz_impl.hpp:372-420, the empty-token exit in the
 * caller) and token_ratio (with_sorted = true; fuzz_impl.hpp:518-564) over the S parts */
template <typename P>
RFG_NOINL double token_set_dev(const P& p, double cutoff, bool with_sorted, u64* st)
{
    if (cutoff > 100) return 0.0;
    const int qa = p.q0, ca = p.c0, Ws = words_of(p.qs), kcw = (p.cs + 1) / 128 + 1;
    u64* kq = st;
    u64* kc = st + Ws;
    u64* SA = kc + kcw;
    u64* SB = SA + Ws;
    const TokSplit r = tok_split(*p.q, qa, p.qs, *p.c, ca, p.cs, kq, Ws, kc, kcw);
    if (r.sect_n > 0 && (r.ab_n == 0 || r.ba_n == 0)) return 100.0;
    const bool needB = r.ab_n > 0 && r.ba_n > 0;
    u64 lcsA = 0, lcsB = 0;
    if (Ws && (with_sorted || needB)) {
        const PMShift<typename P::PMType> pms{p.pm, p.W, qa, p.qs};
        tok_lcs(pms, Ws, kq, *p.t, ca, p.cs, kc, with_sorted ? SA : nullptr, needB ? SB : nullptr);
        if (with_sorted) lcsA = lcs_count(SA, Ws, p.qs);
        if (needB) lcsB = lcs_count(SB, Ws, p.qs);
    }
    double result = with_sorted ? ratio_from_lcs((u64)p.qs, (u64)p.cs, lcsA, cutoff) : 0.0;
    const u64 ab = (u64)r.ab_len, ba = (u64)r.ba_len, sect = (u64)r.sect_len;
    const u64 sab = sect + (sect != 0) + ab, sba = sect + (sect != 0) + ba;
    const u64 cd = cutoff_to_distance(cutoff, sab + sba);
    const u64 dist = ab + ba - 2 * lcsB;
    if (dist <= cd) {
        const double nd = norm_distance_pct(dist, sab + sba, cutoff);
        result = with_sorted ? dmax(result, nd) : nd;
    }
    if (!sect) return result;
    const double r_ab = norm_distance_pct((sect != 0) + ab, sect + sab, cutoff);
    const double r_ba = norm_distance_pct((sect != 0) + ba, sect + sba, cutoff);
    return dmax(dmax(result, r_ab), r_ba);
}

/* ratio of q's part [qa, qa + qm) with c's part [ca, ca + cn) (fuzz_impl.hpp:22-32) */
template <typename P>
RFG_HD double tok_ratio(const P& p, int qa, int qm, int ca, int cn, double cutoff, u64* st)
{
    u64 lcs = 0;
    if (qm && cn) {
        const PMShift<typename P::PMType> pv{p.pm, p.W, qa, qm};
        const TextSlice<typename P::TxtType> tv{p.t, ca};
        lcs_stream(pv, words_of(qm), tv, cn, st, [](int) {});
        lcs = lcs_count(st, words_of(qm), qm);
    }
    return ratio_from_lcs((u64)qm, (u64)cn, lcs, cutoff);
}

/* partial_ratio of q's part [qa, qa + qm) with c's part [ca, ca + cn) */
template <typename P>
RFG_NOINL double tok_partial(const P& p, int qa, int qm, int ca, int cn, double cutoff, u64* st)
{
    const PMShift<typename P::PMType> pv{p.pm, p.W, qa, qm};
    const TextSlice<typename P::TxtType> tv{p.t, ca};
    return partial_ratio_dev(pv, words_of(qm), qm, tv, cn, cutoff, st, (u32*)(st + p.W + 1));
}

/* partial_token_ratio (fuzz_impl.hpp:704-731): partial_ratio of the S parts, then of the
 * J parts (diff_ab / diff_ba are every distinct token when the intersection is empty)
 * unless neither side had repeats */
template <typename P>
RFG_HD double partial_token_ratio_dev(const P& p, double cutoff, u64* st)
{
    if (cutoff > 100) return 0.0;
    const TokSplit r = tok_split(*p.q, p.q0, p.qs, *p.c, p.c0, p.cs, (u64*)nullptr, 0, (u64*)nullptr, 0);
    if (r.sect_n) return 100.0;
    const double result = tok_partial(p, p.q0, p.qs, p.c0, p.cs, cutoff, st);
    if (r.na == r.ab_n && r.nb == r.ba_n) return result;
    return dmax(result, tok_partial(p, p.q0 + p.qs, p.qj, p.c0 + p.cs, p.cj, dmax(cutoff, result), st));
}

/* WRatio / CachedWRatio::similarity (fuzz_impl.hpp:789-822, 842-879) */
template <typename P>
RFG_HD double wratio_dev(const P& p, double cutoff, u64* st)
{
    const double UNBASE_SCALE = 0.95;
    if (cutoff > 100) return 0.0;
    const int len1 = p.q0, len2 = p.c0;
    if (!len1 || !len2) return 0.0;
    const double len_ratio = len1 > len2 ? ddiv((double)len1, (double)len2) : ddiv((double)len2, (double)len1);
    double end_ratio = tok_ratio(p, 0, len1, 0, len2, cutoff, st);
    if (len_ratio < 1.5) {
        cutoff = ddiv(dmax(cutoff, end_ratio), UNBASE_SCALE);
        return dmax(end_ratio, dmul(token_set_dev(p, cutoff, true, st), UNBASE_SCALE));
    }
    const double PARTIAL_SCALE = len_ratio <= 8.0 ? 0.9 : 0.6;
    cutoff = ddiv(dmax(cutoff, end_ratio), PARTIAL_SCALE);
    end_ratio = dmax(end_ratio, dmul(tok_partial(p, 0, len1, 0, len2, cutoff, st), PARTIAL_SCALE));
    cutoff = ddiv(dmax(cutoff, end_ratio), UNBASE_SCALE);
    return dmax(end_ratio, dmul(dmul(partial_token_ratio_dev(p, cutoff, st), UNBASE_SCALE), PARTIAL_SCALE));
}

/* one pair of the token scorers (free and Cached forms give the same values):
 * token_sort_ratio, partial_token_sort_ratio (fuzz_impl.hpp:297-349) and QRatio
 * (fuzz_impl.hpp:891-909) on their parts here serve extract over a corpus; rfg_cdist
 * scores them with the ratio kernels */
template <typename P>
RFG_HD double token_family_dev(int metric, const P& p, double cutoff, u64* st)
{
    if (cutoff > 100) return 0.0;
    switch (metric) {
    case TOKEN_SORT_RATIO: return tok_ratio(p, p.q0, p.qs, p.c0, p.cs, cutoff, st);
    case PARTIAL_TOKEN_SORT_RATIO: return tok_partial(p, p.q0, p.qs, p.c0, p.cs, cutoff, st);
    case QRATIO:
        if (!p.q0 || !p.c0) return 0.0;
        return tok_ratio(p, 0, p.q0, 0, p.c0, cutoff, st);
    case TOKEN_SET_RATIO:
        if (!p.qs || !p.cs) return 0.0; /* no tokens on a side (fuzz_impl.hpp:379) */
        return token_set_dev(p, cutoff, false, st);
    case PARTIAL_TOKEN_SET_RATIO: { /* fuzz_impl.hpp:460-477, on the J parts */
        if (!p.qj || !p.cj) return 0.0;
        const int qa = p.q0 + p.qs, ca = p.c0 + p.cs;
        const TokSplit r = tok_split(*p.q, qa, p.qj, *p.c, ca, p.cj, (u64*)nullptr, 0, (u64*)nullptr, 0);
        if (r.sect_n) return 100.0;
        return tok_partial(p, qa, p.qj, ca, p.cj, cutoff, st);
    }
    case TOKEN_RATIO: return token_set_dev(p, cutoff, true, st);
    case PARTIAL_TOKEN_RATIO: return partial_token_ratio_dev(p, cutoff, st);
    default: return wratio_dev(p, cutoff, st);
    }
}

/* Per-query tables of the Jaro chains (free / Cached forms): everything that depends
 * only on the common prefix (0..4) and the text length.  minc[p][tl] is 0 when the
 * reference never reads the counts (its early exits), else the smallest common-character
 * count passing jaro_common_filter (the filter is monotone in the count), 0xffff when
 * none does.  jc[p]: the cutoff the inner Jaro runs with; v0[p]: its value when the
 * counts are not read.  With them a pair needs doubles only when it can pass. */
#define RFG_JT_MAXT 256
struct JaroTab {
    double jc[5];
    double vfail[5]; /* the API result of a pair whose count stays below minc */
    unsigned short minc[5][RFG_JT_MAXT + 1];
};

RFG_HD double jaro_tab_cutoff(const PairSpec& s, int prefix)
{
    const double c = fsim_chain_cutoff(s.op, s.cf);
    return s.metric == JARO ? c : jw_jaro_cutoff(prefix, s.p.prefix_weight, c);
}

/* entry (prefix, tl) for a query of length pl; s carries metric, op, cutoff, weight */
RFG_HD unsigned short jaro_tab_minc(const PairSpec& s, i64 pl, int prefix, i64 tl)
{
    const double c = jaro_tab_cutoff(s, prefix);
    if (!jaro_needs_counts(pl, tl, c)) return 0;
    const i64 cmax = pl < tl ? pl : tl;
    i64 lo = 1, hi = cmax + 1; /* first passing count in [1, cmax], or cmax + 1 */
    while (lo < hi) {
        const i64 mid = (lo + hi) / 2;
        if (jaro_common_filter(pl, tl, mid, c)) hi = mid;
        else lo = mid + 1;
    }
    return lo > cmax ? (unsigned short)0xffff : (unsigned short)(lo > 0xfffe ? 0xfffe : lo);
}

/* jaro_from_counts with the table: identical values */
RFG_HD double jaro_from_counts_tab(i64 pl, i64 tl, i64 common, i64 transp, double c, unsigned short minc)
{
    if (minc == 0) return c > 1.0 ? 0.0 : ((pl == 0 && tl == 0) ? 1.0 : 0.0);
    if (pl == 1 && tl == 1) return (double)(common == 1);
    if (common < (i64)minc) return 0.0;
    const double sim = jaro_formula(pl, tl, common, transp);
    return sim >= c ? sim : 0;
}

RFG_HD double finish_jaro_tab(const PairSpec& s, const JaroTab& t, i64 prefix, i64 common, i64 transp)
{
    const i64 pl = (i64)s.l1, tl = (i64)s.l2;
    const double jc = t.jc[prefix];
    const double sim_j = jaro_from_counts_tab(pl, tl, common, transp, jc, t.minc[prefix][tl]);
    const double sim = s.metric == JARO ? sim_j : jw_finish(sim_j, prefix, s.p.prefix_weight, fsim_chain_cutoff(s.op, s.cf));
    if (s.op == SIMILARITY) return sim;
    return fsim_chain_finish(s.op, sim, s.cf);
}

RFG_HD void jaro_tab_head(JaroTab& t, const PairSpec& s)
{
    for (int p = 0; p < 5; ++p) {
        t.jc[p] = jaro_tab_cutoff(s, p);
        /* finish_jaro_tab with the inner Jaro at 0.0 (jaro_from_counts_tab's value below minc) */
        const double sim = s.metric == JARO ? 0.0 : jw_finish(0.0, p, s.p.prefix_weight, fsim_chain_cutoff(s.op, s.cf));
        t.vfail[p] = s.op == SIMILARITY ? sim : fsim_chain_finish(s.op, sim, s.cf);
    }
}

RFG_HD double finish_jaro(const PairSpec& s, i64 prefix, i64 common, i64 transp)
{
    const i64 pl = (i64)s.l1, tl = (i64)s.l2;
    const double pw = s.p.prefix_weight;
    if (s.form == FORM_MULTI) {
        if (s.metric == JARO) {
            const double a = multi_jaro_from_counts(pl, tl, common, transp, s.cf);
            const double b = multi_jaro_from_counts(pl, tl, common, transp, 0.0);
            return multi_fsim_finish(s.op, a, b, s.cf);
        }
        const double a = multi_jw(multi_jaro_from_counts(pl, tl, common, transp, dmin(0.7, s.cf)), prefix, pw, s.cf);
        const double b = multi_jw(multi_jaro_from_counts(pl, tl, common, transp, dmin(0.7, 0.0)), prefix, pw, 0.0);
        return multi_fsim_finish(s.op, a, b, s.cf);
    }
    const double c = fsim_chain_cutoff(s.op, s.cf);
    double sim;
    if (s.metric == JARO) {
        sim = jaro_from_counts(pl, tl, common, transp, c);
    }
    else {
        const double jc = jw_jaro_cutoff(prefix, pw, c);
        sim = jw_finish(jaro_from_counts(pl, tl, common, transp, jc), prefix, pw, c);
    }
    return fsim_chain_finish(s.op, sim, s.cf);
}

} // namespace rfg
