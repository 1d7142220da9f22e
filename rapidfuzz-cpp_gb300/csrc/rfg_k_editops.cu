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
    if (p >= P.p0 + P.np || (P.hb && P.hb[p])) return;
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

/* ------------------------------------------------ long Levenshtein pairs
 * levenshtein_editops's own flow (Levenshtein_impl.hpp:1184-1257) for pairs whose
 * matrices may pass 1 MB: the score hint decides the first band, then every segment drops
 * its common affix and is either aligned from a recorded matrix (the reference's
 * levenshtein_align; here a diagonal band of the full matrix, wide enough for every cell
 * the walk reads) or split at s2's middle row and at the first s1 position where the
 * distance of the left part plus that of the right part is smallest (find_hirschberg_pos;
 * here from exact DP rows), the halves aligned in turn.  One thread per pair, an explicit
 * stack of pending segments.  Scratch layout (words): pattern table (256 x W, one-byte
 * units only), row vectors (4 W), band row offsets (n + 1), band storage. */
struct Seg {
    int64_t a, m, b, n;      /* s1[a, a + m), s2[b, b + n) (offsets within the pair) */
    int64_t sp, dp, pos;     /* source / destination positions, first operation slot */
    uint64_t max;            /* distance bound of the segment */
};

struct HBView {
    const KStrings* s;
    int64_t base;
    __device__ __forceinline__ u64 operator()(int64_t i) const { return load_unit(s->data, s->width, base + i); }
};

/* match word w of pattern A[a0 + step * i] (i < m) for the unit c: the table for one-byte
 * units, a scan otherwise */
struct HBPattern {
    HBView A;
    int64_t a0, m;
    int step; /* 1 forward, -1 backward (a0 is then the last unit) */
    const u64* pm; /* 256 x W rows or null */
    int W;
    __device__ __forceinline__ u64 match(int w, u64 c) const
    {
        if (pm) return c < 256 ? pm[c * W + w] : 0;
        u64 x = 0;
        const int64_t i0 = (int64_t)w * 64, i1 = i0 + 64 < m ? i0 + 64 : m;
        for (int64_t i = i0; i < i1; ++i) x |= (u64)(A(a0 + step * i) == c) << (i - i0);
        return x;
    }
};

__device__ void hb_build_pm(HBPattern& P, u64* pm, int one_byte)
{
    P.pm = nullptr;
    if (!one_byte) return;
    for (int64_t k = 0; k < 256 * (int64_t)P.W; ++k) pm[k] = 0;
    for (int64_t i = 0; i < P.m; ++i) pm[P.A(P.a0 + P.step * i) * P.W + (i >> 6)] |= 1ull << (i & 63);
    P.pm = pm;
}

/* Hyyro's recurrence over B[b0 + bstep * j] (j < n); vp / vn: W words in and out */
__device__ void hb_rows(const HBPattern& P, HBView B, int64_t b0, int bstep, int64_t n, u64* vp, u64* vn)
{
    for (int w = 0; w < P.W; ++w) {
        vp[w] = ~0ull;
        vn[w] = 0;
    }
    for (int64_t j = 0; j < n; ++j) {
        const u64 c = B(b0 + bstep * j);
        u64 hp_c = 1, hn_c = 0;
        for (int w = 0; w < P.W; ++w) {
            const u64 VP = vp[w], VN = vn[w];
            const u64 X = P.match(w, c) | hn_c;
            const u64 D0 = (((X & VP) + VP) ^ VP) | X | VN;
            u64 HP = VN | ~(D0 | VP);
            u64 HN = D0 & VP;
            const u64 hp_o = HP >> 63, hn_o = HN >> 63;
            HP = (HP << 1) | hp_c;
            HN = (HN << 1) | hn_c;
            vp[w] = HN | ~(D0 | HP);
            vn[w] = HP & D0;
            hp_c = hp_o;
            hn_c = hn_o;
        }
    }
}

__device__ __forceinline__ int64_t bit_of(const u64* v, int64_t i) { return (int64_t)((v[i >> 6] >> (i & 63)) & 1); }

__global__ void __launch_bounds__(64) k_editops_hb(const EditopsParams P)
{
    const int64_t p = P.p0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= P.p0 + P.np || !P.hb || !P.hb[p]) return;
    const HBView A{&P.a, P.a.off[p]}, B{&P.b, P.b.off[p]};
    const int64_t la = P.a.off[p + 1] - P.a.off[p], lb = P.b.off[p + 1] - P.b.off[p];
    const int Wmax = (int)((la + 63) / 64) > 0 ? (int)((la + 63) / 64) : 1;
    const int one_byte = P.a.width == 1 && P.b.width == 1;
    u64* pm = P.mat + P.moff[p];
    u64* rows = pm + (one_byte ? 256 * (int64_t)Wmax : 0);
    int64_t* roff = (int64_t*)(rows + 4 * (int64_t)Wmax);
    u64* band = (u64*)(roff + lb + 1);
    const u64* band_end = P.mat + P.moff[p + 1];
    EditopDev* out = P.ops + P.ooff[p];
    const int64_t ub = P.ooff[p + 1] - P.ooff[p];
    int64_t total = 0;
    /* the first band: levenshtein_editops (Levenshtein_impl.hpp:1234-1257) */
    uint64_t hint = P.hint < 31 ? 31 : P.hint;
    uint64_t cutoff = (uint64_t)(la > lb ? la : lb);
    if (~0ull / 2 > hint && 2 * hint < cutoff) {
        HBPattern pat{A, 0, la, 1, nullptr, Wmax};
        hb_build_pm(pat, pm, one_byte);
        hb_rows(pat, B, 0, 1, lb, rows, rows + Wmax);
        int64_t d = lb;
        for (int64_t i = 0; i < la; ++i) d += bit_of(rows, i) - bit_of(rows + Wmax, i);
        cutoff = (uint64_t)d;
    }
    Seg stack[64];
    int top = 0;
    stack[top++] = Seg{0, la, 0, lb, 0, 0, 0, cutoff};
    while (top > 0) {
        Seg g = stack[--top];
        int64_t pre = 0;
        while (pre < g.m && pre < g.n && A(g.a + pre) == B(g.b + pre)) ++pre;
        int64_t suf = 0;
        while (suf < g.m - pre && suf < g.n - pre && A(g.a + g.m - 1 - suf) == B(g.b + g.n - 1 - suf)) ++suf;
        g.a += pre;
        g.b += pre;
        g.m -= pre + suf;
        g.n -= pre + suf;
        g.sp += pre;
        g.dp += pre;
        const uint64_t mx = g.max < (uint64_t)(g.m > g.n ? g.m : g.n) ? g.max : (uint64_t)(g.m > g.n ? g.m : g.n);
        const uint64_t full_band = (uint64_t)g.m < 2 * mx + 1 ? (uint64_t)g.m : 2 * mx + 1;
        const int W = (int)((g.m + 63) / 64);
        if (2 * full_band * (uint64_t)g.n / 8 >= (1u << 20) && g.m >= 65 && g.n >= 10) {
            /* find_hirschberg_pos (Levenshtein_impl.hpp:1096-1180) from exact rows */
            const int64_t s2_mid = g.n / 2;
            HBPattern fw{A, g.a, g.m, 1, nullptr, W};
            hb_build_pm(fw, pm, one_byte);
            hb_rows(fw, B, g.b, 1, s2_mid, rows, rows + W);
            HBPattern bw{A, g.a + g.m - 1, g.m, -1, nullptr, W};
            hb_build_pm(bw, pm, one_byte);
            hb_rows(bw, B, g.b + g.n - 1, -1, g.n - s2_mid, rows + 2 * W, rows + 3 * W);
            /* left[i] = s2_mid + deltas of bits < i; right[k] = (n - s2_mid) + deltas < k */
            int64_t right = g.n - s2_mid;
            for (int64_t k = 0; k < g.m; ++k) right += bit_of(rows + 2 * W, k) - bit_of(rows + 3 * W, k);
            int64_t left = s2_mid, best = INT64_MAX, s1_mid = 0, ls = 0, rs = 0;
            for (int64_t i = 0; i <= g.m; ++i) {
                if (left + right < best) {
                    best = left + right;
                    s1_mid = i;
                    ls = left;
                    rs = right;
                }
                if (i < g.m) {
                    left += bit_of(rows, i) - bit_of(rows + W, i);
                    const int64_t k = g.m - 1 - i; /* right[m - i - 1] from right[m - i] */
                    right -= bit_of(rows + 2 * W, k) - bit_of(rows + 3 * W, k);
                }
            }
            if (top + 2 > 64) {
                atomicExch(P.err, 4);
                return;
            }
            stack[top++] = Seg{g.a + s1_mid, g.m - s1_mid, g.b + s2_mid, g.n - s2_mid, g.sp + s1_mid, g.dp + s2_mid,
                               g.pos + ls, (uint64_t)rs};
            stack[top++] = Seg{g.a, s1_mid, g.b, s2_mid, g.sp, g.dp, g.pos, (uint64_t)ls};
            continue;
        }
        /* a leaf: levenshtein_align over a band of the full matrix */
        int64_t dist;
        if (g.m == 0 || g.n == 0) dist = g.m + g.n;
        else {
            const int64_t D = (int64_t)mx + 2;
            HBPattern fw{A, g.a, g.m, 1, nullptr, W};
            hb_build_pm(fw, pm, one_byte);
            u64* vp = rows;
            u64* vn = rows + W;
            for (int w = 0; w < W; ++w) {
                vp[w] = ~0ull;
                vn[w] = 0;
            }
            int64_t used = 0;
            for (int64_t r = 0; r < g.n; ++r) {
                const u64 c = B(g.b + r);
                u64 hp_c = 1, hn_c = 0;
                for (int w = 0; w < W; ++w) {
                    const u64 VP = vp[w], VN = vn[w];
                    const u64 X = fw.match(w, c) | hn_c;
                    const u64 D0 = (((X & VP) + VP) ^ VP) | X | VN;
                    u64 HP = VN | ~(D0 | VP);
                    u64 HN = D0 & VP;
                    const u64 hp_o = HP >> 63, hn_o = HN >> 63;
                    HP = (HP << 1) | hp_c;
                    HN = (HN << 1) | hn_c;
                    vp[w] = HN | ~(D0 | HP);
                    vn[w] = HP & D0;
                    hp_c = hp_o;
                    hn_c = hn_o;
                }
                /* words of columns [r - D, r + D] */
                const int64_t c0 = r - D > 0 ? r - D : 0, c1 = r + D < g.m - 1 ? r + D : g.m - 1;
                const int64_t w0 = c0 >> 6, w1 = c1 >> 6, cnt = w1 - w0 + 1;
                if (band + used + 2 * cnt > band_end) {
                    atomicExch(P.err, 5);
                    return;
                }
                roff[r] = used;
                for (int64_t w = 0; w < cnt; ++w) {
                    band[used + w] = vp[w0 + w];
                    band[used + cnt + w] = vn[w0 + w];
                }
                used += 2 * cnt;
            }
            dist = g.n;
            for (int64_t i = 0; i < g.m; ++i) dist += bit_of(vp, i) - bit_of(vn, i);
            /* bit (row, col) of VP (which 0) or VN (1); -1 outside the stored band */
            auto bitm = [&](int64_t row, int64_t col, int which) -> int {
                const int64_t c0 = row - D > 0 ? row - D : 0, c1 = row + D < g.m - 1 ? row + D : g.m - 1;
                const int64_t w0 = c0 >> 6, cnt = (c1 >> 6) - w0 + 1, w = col >> 6;
                if (col < c0 || col > c1) return -1;
                return (int)((band[roff[row] + (which ? cnt : 0) + (w - w0)] >> (col & 63)) & 1);
            };
            int64_t rem = dist, col = g.m, row = g.n;
            bool bad = false;
            auto put = [&](int type, int64_t cc, int64_t rr) {
                if (rem <= 0 || g.pos + rem - 1 >= ub) {
                    bad = true;
                    return;
                }
                --rem;
                out[g.pos + rem] = EditopDev{type, 0, cc + g.sp, rr + g.dp};
            };
            while (row && col && !bad) {
                const int b1 = bitm(row - 1, col - 1, 0);
                if (b1 < 0) {
                    bad = true;
                    break;
                }
                if (b1) {
                    --col;
                    put(3, col, row);
                }
                else {
                    --row;
                    int b2 = 0;
                    if (row) {
                        b2 = bitm(row - 1, col - 1, 1);
                        if (b2 < 0) {
                            bad = true;
                            break;
                        }
                    }
                    if (row && b2) put(2, col, row);
                    else {
                        --col;
                        if (A(g.a + col) != B(g.b + row)) put(1, col, row);
                    }
                }
            }
            while (col && !bad) {
                --col;
                put(3, col, row);
            }
            while (row && !bad) {
                --row;
                put(2, col, row);
            }
            if (bad || rem != 0) {
                atomicExch(P.err, 6);
                return;
            }
            total += dist;
            continue;
        }
        /* one side empty: deletions or insertions only */
        for (int64_t k = 0; k < dist; ++k) {
            if (g.pos + k >= ub) {
                atomicExch(P.err, 6);
                return;
            }
            out[g.pos + k] = g.m ? EditopDev{3, 0, g.sp + k, g.dp} : EditopDev{2, 0, g.sp, g.dp + k};
        }
        total += dist;
    }
    P.count[p] = total;
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
const void* editops_hb_kernel() { return (const void*)&k_editops_hb; }
const void* editops_pack_kernel() { return (const void*)&k_editops_pack; }

} // namespace rfg
