/* Editops of many (s1, s2) pairs, one thread per pair: levenshtein_editops
 * (Levenshtein_impl.hpp:956-1045, 1185-1257) and lcs_seq_editops / indel_editops
 * (LCSseq_impl.hpp:437-529).
 *
 * After the common prefix and suffix are removed (on the host, which also sizes every
 * pair's regions), the thread runs the bit-parallel recurrence over s2' with s1' as the
 * pattern (Hyyro's Levenshtein VP/VN with word carries, or Hyyro's LCS S vector) and
 * records every row's vectors in its scratch region; then it walks back from the end as
 * the reference's recover_alignment does and writes the operations, last first, into its
 * output region.  The recorded matrices are the full (unbanded) ones: every bit the walk
 * reads is an exact table delta. */
#include "rfg_device.cuh"
#include "rfg_kernels.h"

namespace rfg {

__device__ __forceinline__ u64 unit(const KStrings& s, int64_t base, int64_t i) { return load_unit(s.data, s.width, base + i); }

/* match word w of s1'[0, m) for the unit c (no table: the pattern is scanned) */
__device__ __forceinline__ u64 match_word(const KStrings& s, int64_t base, int64_t m, int w, u64 c)
{
    u64 x = 0;
    const int64_t i0 = (int64_t)w * 64, i1 = i0 + 64 < m ? i0 + 64 : m;
    for (int64_t i = i0; i < i1; ++i) x |= (u64)(unit(s, base, i) == c) << (i - i0);
    return x;
}

__global__ void __launch_bounds__(128) k_editops(const EditopsParams P)
{
    const int64_t p = P.p0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= P.p0 + P.np) return;
    const int64_t pre = P.pre[p], suf = P.suf[p];
    const int64_t ab = P.a.off[p] + pre, bb = P.b.off[p] + pre;
    const int64_t m = P.a.off[p + 1] - P.a.off[p] - pre - suf, n = P.b.off[p + 1] - P.b.off[p] - pre - suf;
    const int W = (int)((m + 63) / 64);
    u64* M = P.mat + P.moff[p];
    int64_t dist;
    if (m == 0 || n == 0) dist = m + n;
    else if (P.lev) {
        /* rows of 2W words, VP then VN; before the first row VP = 1^m, VN = 0 */
        for (int64_t r = 0; r < n; ++r) {
            const u64 c = unit(P.b, bb, r);
            u64 hp_c = 1, hn_c = 0;
            for (int w = 0; w < W; ++w) {
                const u64 VP = r ? M[(r - 1) * 2 * W + w] : ~0ull;
                const u64 VN = r ? M[(r - 1) * 2 * W + W + w] : 0ull;
                const u64 X = match_word(P.a, ab, m, w, c) | hn_c;
                const u64 D0 = (((X & VP) + VP) ^ VP) | X | VN;
                u64 HP = VN | ~(D0 | VP);
                u64 HN = D0 & VP;
                const u64 hp_o = HP >> 63, hn_o = HN >> 63;
                HP = (HP << 1) | hp_c;
                HN = (HN << 1) | hn_c;
                M[r * 2 * W + w] = HN | ~(D0 | HP);
                M[r * 2 * W + W + w] = HP & D0;
                hp_c = hp_o;
                hn_c = hn_o;
            }
        }
        /* D[m][n] = n + (sum of the last row's vertical deltas over the m pattern bits) */
        dist = n;
        for (int w = 0; w < W; ++w) {
            const u64 mk = low_mask((int)(m - 64 * (int64_t)w));
            dist += popc64(M[(n - 1) * 2 * W + w] & mk) - popc64(M[(n - 1) * 2 * W + W + w] & mk);
        }
    }
    else {
        for (int64_t r = 0; r < n; ++r) {
            const u64 c = unit(P.b, bb, r);
            u32 carry = 0;
            for (int w = 0; w < W; ++w) {
                const u64 S = r ? M[(r - 1) * W + w] : ~0ull;
                const u64 u = S & match_word(P.a, ab, m, w, c);
                const u64 x = add_carry(S, u, carry, &carry);
                M[r * W + w] = x | (S - u);
            }
        }
        int64_t sim = 0;
        for (int w = 0; w < W; ++w)
            sim += popc64(~M[(n - 1) * W + w] & low_mask((int)(m - 64 * (int64_t)w)));
        dist = m + n - 2 * sim;
    }
    P.count[p] = dist;
    EditopDev* out = P.ops + P.ooff[p];
    auto bit = [&](int64_t row, int64_t col, int which) -> bool {
        /* which: 0 VP / S, 1 VN */
        const int64_t stride = P.lev ? 2 * W : W;
        return (M[row * stride + (which ? W : 0) + (col >> 6)] >> (col & 63)) & 1;
    };
    auto put = [&](int type, int64_t col, int64_t row) {
        if (dist <= 0) { /* more operations than the distance: flag it, write nothing */
            atomicExch(P.err, 3);
            return;
        }
        --dist;
        out[dist] = EditopDev{type, 0, col + pre, row + pre};
    };
    int64_t col = m, row = n;
    if (dist == 0) return;
    while (row && col) {
        if (bit(row - 1, col - 1, 0)) { /* Delete (LCS: S bit set, the LCS does not grow) */
            --col;
            put(3, col, row);
        }
        else {
            --row;
            if (row && (P.lev ? bit(row - 1, col - 1, 1) : !bit(row - 1, col - 1, 0)))
                put(2, col, row); /* Insert */
            else {
                --col; /* Match, or Replace (Levenshtein) */
                if (P.lev && unit(P.a, ab, col) != unit(P.b, bb, row)) put(1, col, row);
            }
        }
    }
    while (col) {
        --col;
        put(3, col, row);
    }
    while (row) {
        --row;
        put(2, col, row);
    }
}

/* pair i's operations from its region at ooff[i] to dst[off[i], off[i + 1]) */
__global__ void __launch_bounds__(128) k_editops_pack(const EditopDev* src, const int64_t* ooff, const int64_t* off,
                                                      EditopDev* dst, int64_t np)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int64_t n = off[i + 1] - off[i];
    for (int64_t k = 0; k < n; ++k) dst[off[i] + k] = src[ooff[i] + k];
}

const void* editops_kernel() { return (const void*)&k_editops; }
const void* editops_pack_kernel() { return (const void*)&k_editops_pack; }

} // namespace rfg
