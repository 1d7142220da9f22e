/* The library's scorer cores (rfg_core.cuh: the same templates the kernels instantiate)
 * compiled for the host, behind C entry points for the CPU tests, which compare them with
 * the oracle's exact values.  The dispatch restates the kernels' callers: the length
 * filter and empty-string rules first, then the core the kernel would pick.  One-byte
 * strings; patterns of any length (the table holds 256 rows of W words, plus one zero row
 * per query for the several-queries cores). */
#include <stdint.h>

#include <vector>

#include "rfg_core.cuh"

using namespace rfg;

namespace {

struct PM1 { /* one-word table */
    const u64* rows;
    u64 operator()(u64 c) const { return rows[c]; }
};
struct PMW { /* W-word table */
    const u64* rows;
    int W;
    u64 operator()(u64 c, int w) const { return rows[c * (u64)W + w]; }
};
struct PMQ { /* several one-word patterns: 257 rows each (row 256 is zero) */
    const u64* rows;
    u64 operator()(int q, unsigned c) const { return rows[q * 257 + c]; }
};
struct Txt {
    const uint8_t* p;
    u64 operator[](int j) const { return p[j]; }
};

std::vector<u64> table(const uint8_t* a, int m, int W)
{
    std::vector<u64> rows((size_t)256 * W, 0);
    for (int k = 0; k < m; ++k) rows[(size_t)a[k] * W + k / 64] |= 1ull << (k % 64);
    return rows;
}

/* fam 0 Levenshtein, 1 Indel (via LCS), 2 OSA: the raw core value with the callers'
 * shortcuts (LCS: the length, or -1 when pruned; distances: d or any value > K) */
template <int W>
i64 reg_core(int fam, const PMW& pm, const PM1& pm1, int m, const Txt& t, int n, i64 K)
{
    const i64 diff = m > n ? m - n : n - m;
    if (fam == 1) {
        if (m == 0 || n == 0) return 0;
        if (K < diff) return -1;
        return W == 1 ? lcs_word(pm1, m, t, n, K) : lcs_multi<W>(pm, m, t, n, K);
    }
    if (m == 0) return n;
    if (K < diff) return K + 1;
    if (n == 0) return m;
    if (fam == 2) return W == 1 ? osa_word(pm1, m, t, n, K) : osa_multi<W>(pm, m, t, n, K);
    if (W == 1) return lev_word(pm1, m, t, n, K);
    if (K < m) {
        const i64 band = 2 * K + 1;
        if (W > 1 && band <= 64) return lev_band<1>(pm, W, m, t, n, (int)K);
        if (W > 2 && band <= 128) return lev_band<2>(pm, W, m, t, n, (int)K);
        if (W > 4 && band <= 256) return lev_band<4>(pm, W, m, t, n, (int)K);
    }
    return lev_multi<W>(pm, m, t, n, K);
}

i64 rt_core(int fam, const PMW& pm, int W, int m, const Txt& t, int n, i64 K)
{
    std::vector<u64> st((size_t)4 * W + 4);
    const i64 diff = m > n ? m - n : n - m;
    if (fam == 1) {
        if (m == 0 || n == 0) return 0;
        if (K < diff) return -1;
        return lcs_multi_rt(pm, W, m, t, n, K, st.data());
    }
    if (m == 0) return n;
    if (K < diff) return K + 1;
    if (n == 0) return m;
    if (fam == 2) return osa_multi_rt(pm, W, m, t, n, K, st.data(), st.data() + W, st.data() + 2 * W, st.data() + 3 * W);
    if (K < m && 2 * K + 1 <= 64) return lev_band<1>(pm, W, m, t, n, (int)K);
    if (K < m && 2 * K + 1 <= 128) return lev_band<2>(pm, W, m, t, n, (int)K);
    if (K < m && 2 * K + 1 <= 256) return lev_band<4>(pm, W, m, t, n, (int)K);
    if (K < m && 2 * K + 1 <= 512) return lev_band<8>(pm, W, m, t, n, (int)K);
    return lev_multi_rt(pm, W, m, t, n, K, st.data(), st.data() + W);
}

/* the distance chain d <= K ? d : K + 1 of a raw core value */
int64_t chain(int fam, int m, int n, i64 raw, i64 K)
{
    i64 d = raw;
    if (fam == 1) d = raw < 0 ? K + 1 : (i64)m + n - 2 * raw;
    return d <= K ? d : K + 1;
}

} // namespace

extern "C" {

/* variant 0: the register-resident cores of the tile kernel (W = 1, 2, 4, 8 by the
 * pattern length, at most 512 units); variant 1: the any-length kernel's cores (runtime
 * W, bands up to 8 words).  Returns the distance chain, or -2 for a shape the variant
 * does not take. */
int64_t hc_distance(int fam, int variant, const uint8_t* a, int m, const uint8_t* b, int n, int64_t K)
{
    const int W = m > 0 ? (m + 63) / 64 : 1;
    const Txt t{b};
    if (variant == 0) {
        const int Wr = W <= 1 ? 1 : W <= 2 ? 2 : W <= 4 ? 4 : W <= 8 ? 8 : 0;
        if (!Wr) return -2;
        const std::vector<u64> rows = table(a, m, Wr);
        const std::vector<u64> rows1 = table(a, m < 64 ? m : 64, 1);
        const PMW pm{rows.data(), Wr};
        const PM1 pm1{rows1.data()};
        i64 raw = 0;
        switch (Wr) {
        case 1: raw = reg_core<1>(fam, pm, pm1, m, t, n, K); break;
        case 2: raw = reg_core<2>(fam, pm, pm1, m, t, n, K); break;
        case 4: raw = reg_core<4>(fam, pm, pm1, m, t, n, K); break;
        default: raw = reg_core<8>(fam, pm, pm1, m, t, n, K); break;
        }
        return chain(fam, m, n, raw, K);
    }
    const std::vector<u64> rows = table(a, m, W);
    return chain(fam, m, n, rt_core(fam, PMW{rows.data(), W}, W, m, t, n, K), K);
}

/* the several-queries core (group_word_dist) on two patterns of at most 64 units (32
 * with word32) against one text; out[q] = the distance chain of pattern q */
int hc_group(int fam, int word32, const uint8_t* a1, int m1, const uint8_t* a2, int m2, const uint8_t* b, int n,
             int64_t K1, int64_t K2, int64_t* out)
{
    if (m1 > 64 || m2 > 64 || (word32 && (m1 > 32 || m2 > 32))) return -2;
    std::vector<u64> rows(2 * 257, 0);
    for (int k = 0; k < m1; ++k) rows[a1[k]] |= 1ull << k;
    for (int k = 0; k < m2; ++k) rows[257 + a2[k]] |= 1ull << k;
    const int m[2] = {m1, m2};
    const i64 Kq[2] = {K1, K2};
    i64 d[2] = {0, 0};
    const PMQ pm{rows.data()};
    const int F = fam == 0 ? FAM_LEV : fam == 1 ? FAM_LCS : FAM_OSA;
    const Txt t{b};
    if (F == FAM_LEV) {
        if (word32) group_word_dist<FAM_LEV, 2, PMQ, Txt, u32>(pm, m, 2, t, n, Kq, d);
        else group_word_dist<FAM_LEV, 2, PMQ, Txt, u64>(pm, m, 2, t, n, Kq, d);
    }
    else if (F == FAM_LCS) {
        if (word32) group_word_dist<FAM_LCS, 2, PMQ, Txt, u32>(pm, m, 2, t, n, Kq, d);
        else group_word_dist<FAM_LCS, 2, PMQ, Txt, u64>(pm, m, 2, t, n, Kq, d);
    }
    else {
        if (word32) group_word_dist<FAM_OSA, 2, PMQ, Txt, u32>(pm, m, 2, t, n, Kq, d);
        else group_word_dist<FAM_OSA, 2, PMQ, Txt, u64>(pm, m, 2, t, n, Kq, d);
    }
    out[0] = d[0];
    out[1] = d[1];
    return 0;
}

/* the 32-bit banded cores (lev_band32<B>, or with lcs lcs_band32<B>: the Indel distance)
 * with the compact padded table of the band kernel; B = 32-bit words of the window.
 * Returns -2 where the shape does not apply (band_bits > 32B, K >= m, |m-n| > K, or an
 * empty string). */
struct PM32 {
    const uint32_t* base;
    const int32_t* rmap;
    const uint32_t* operator()(uint64_t c) const { return base + rmap[c & 255]; }
};

int64_t hc_band32(int lcs, int B, const uint8_t* a, int m, const uint8_t* b, int n, int64_t K)
{
    if (m == 0 || n == 0 || K >= m || (m > n ? m - n : n - m) > K || band_bits((int)K, m - n) > 32 * B) return -2;
    const int W32 = (m + 31) / 32, pad = B + 1, S = W32 + 3 * pad;
    std::vector<int32_t> rmap(256, 0);
    int R = 1; /* row 0: the zero row */
    for (int k = 0; k < m; ++k)
        if (!rmap[a[k]]) rmap[a[k]] = R++;
    std::vector<uint32_t> rows((size_t)R * S, 0);
    for (int k = 0; k < m; ++k) rows[(size_t)rmap[a[k]] * S + pad + k / 32] |= 1u << (k % 32);
    for (int c = 0; c < 256; ++c) rmap[c] = rmap[c] * S + pad;
    const PM32 pm{rows.data(), rmap.data()};
    const Txt t{b};
    if (lcs) switch (B) {
        case 1: return lcs_band32<1>(pm, m, t, n, (int)K);
        case 2: return lcs_band32<2>(pm, m, t, n, (int)K);
        case 3: return lcs_band32<3>(pm, m, t, n, (int)K);
        case 4: return lcs_band32<4>(pm, m, t, n, (int)K);
        case 8: return lcs_band32<8>(pm, m, t, n, (int)K);
        case 16: return lcs_band32<16>(pm, m, t, n, (int)K);
        }
    switch (B) {
    case 1: return lev_band32<1>(pm, m, t, n, (int)K);
    case 2: return lev_band32<2>(pm, m, t, n, (int)K);
    case 4: return lev_band32<4>(pm, m, t, n, (int)K);
    case 8: return lev_band32<8>(pm, m, t, n, (int)K);
    case 16: return lev_band32<16>(pm, m, t, n, (int)K);
    }
    return -2;
}

/* the count bound of the warp tiles' filter (hist_lower_bound) for a pair of one-byte
 * strings of at most RFG_HIST_MAXLEN units; fam 0 Levenshtein / OSA, 1 Indel */
int hc_hist_bound(int fam, const uint8_t* a, int m, const uint8_t* b, int n)
{
    unsigned char ca[32] = {0}, cb[32] = {0};
    for (int i = 0; i < m; ++i) ++ca[a[i] & 31];
    for (int i = 0; i < n; ++i) ++cb[b[i] & 31];
    u32 ha[8], hb[8];
    for (int w = 0; w < 8; ++w) {
        ha[w] = (u32)ca[4 * w] | (u32)ca[4 * w + 1] << 8 | (u32)ca[4 * w + 2] << 16 | (u32)ca[4 * w + 3] << 24;
        hb[w] = (u32)cb[4 * w] | (u32)cb[4 * w + 1] << 8 | (u32)cb[4 * w + 2] << 16 | (u32)cb[4 * w + 3] << 24;
    }
    return hist_lower_bound(fam == 1 ? FAM_LCS : FAM_LEV, ha, hb, m, n);
}

/* band launches' host logic: band_range (the passing choice lengths of a pattern of m
 * units, unit-weight Levenshtein, op / ci / cf the chain) and band_reject_value; and one
 * pair's plan as the band kernel makes it: *pass = the pair reaches the core, else
 * (vi, vf) = the chain's value of the pruned pair */
int hc_band_range(int metric, int op, uint64_t ci, double cf, int64_t m, int64_t maxlen, int64_t* nlo, int64_t* nhi,
                  int64_t* kmax)
{
    ScoreParams sp;
    sp.ins = sp.del = sp.rep = 1;
    sp.prefix_weight = 0.1;
    return band_range(metric, op, FORM_CACHED, sp, ci, cf, m, maxlen, nlo, nhi, kmax) ? 1 : 0;
}

/* the kernels' fast chain (d <= K ? d : K + 1) serves the unit-weight distances:
 * Levenshtein and Indel */
void hc_band_reject(int metric, int op, uint64_t ci, int64_t* vi, double* vf)
{
    const int fast = op == DISTANCE && (metric == LEVENSHTEIN || metric == INDEL);
    band_reject_value(metric, op, ci, fast, clamp_bound(ci), vi, vf);
}

/* one pair as the band kernel stores it when the pair never reaches the core (raw: the
 * pruned distance K + 1; the LCS families: the LCS -1) and whether it passes the length
 * filter; K the plan's bound */
void hc_band_pair(int metric, int op, uint64_t ci, double cf, int64_t m, int64_t n, int* pass, int64_t* vi, double* vf,
                  int64_t* kout)
{
    PairSpec s;
    s.metric = metric;
    s.op = op;
    s.form = FORM_CACHED;
    s.ci = ci;
    s.cf = cf;
    s.p.ins = s.p.del = s.p.rep = 1;
    s.p.prefix_weight = 0.1;
    s.l1 = (u64)m;
    s.l2 = (u64)n;
    const Plan pl = plan_int(s);
    const i64 K = pl.run ? pl.K : -1;
    const i64 diff = m > n ? m - n : n - m;
    *pass = K >= 0 && m > 0 && n > 0 && K >= diff;
    *kout = K;
    i64 raw = 0;
    if (K >= 0) raw = m == 0 ? n : n == 0 ? m : K + 1;
    *vi = 0;
    *vf = 0.0;
    const bool lcs = metric != LEVENSHTEIN;
    if (op == DISTANCE && (metric == LEVENSHTEIN || metric == INDEL))
        *vi = raw <= (i64)clamp_bound(ci) ? raw : clamp_bound(ci) + 1;
    else if (lcs) finish_int(s, pl, raw <= K ? (m + n - raw) >> 1 : -1, vi, vf);
    else finish_int(s, pl, raw, vi, vf);
}

/* the warp tiles' core (fast_group, int bookkeeping, one cutoff K for every pattern) on
 * four patterns (packed, offsets off[0..4]) of at most 64 units (32 with word32) against
 * one text; qn of the four slots are used; out[q] = the distance chain of pattern q */
int hc_fast(int fam, int word32, const uint8_t* pats, const int64_t* off, int qn, const uint8_t* b, int n, int K,
            int* out)
{
    std::vector<u64> rows(4 * 257, 0);
    int m[4] = {0, 0, 0, 0};
    for (int q = 0; q < qn; ++q) {
        m[q] = (int)(off[q + 1] - off[q]);
        if (m[q] > (word32 ? 32 : 64)) return -2;
        for (int k = 0; k < m[q]; ++k) rows[q * 257 + pats[off[q] + k]] |= 1ull << k;
    }
    const PMQ pm{rows.data()};
    const Txt t{b};
    int d[4] = {0, 0, 0, 0};
    if (fam == 0) {
        if (word32) fast_group<FAM_LEV, 4, PMQ, Txt, u32>(pm, m, qn, t, n, K, d);
        else fast_group<FAM_LEV, 4, PMQ, Txt, u64>(pm, m, qn, t, n, K, d);
    }
    else if (fam == 1) {
        if (word32) fast_group<FAM_LCS, 4, PMQ, Txt, u32>(pm, m, qn, t, n, K, d);
        else fast_group<FAM_LCS, 4, PMQ, Txt, u64>(pm, m, qn, t, n, K, d);
    }
    else {
        if (word32) fast_group<FAM_OSA, 4, PMQ, Txt, u32>(pm, m, qn, t, n, K, d);
        else fast_group<FAM_OSA, 4, PMQ, Txt, u64>(pm, m, qn, t, n, K, d);
    }
    for (int q = 0; q < qn; ++q) out[q] = d[q];
    return 0;
}

/* Jaro common characters and (unhalved) transpositions, m, n > 0.  variant 0: jaro_word
 * (pattern <= 64 units, effective text end <= 64); 1: jaro_multi<W> (W = 1, 2, 4, 8);
 * 2: jaro_multi_rt; 3: group_jaro_word with the pattern in both slots (as variant 0).
 * Returns -2 for a shape the variant does not take. */
int hc_jaro(int variant, const uint8_t* a, int m, const uint8_t* b, int n, int64_t* common, int64_t* transp)
{
    int bound = (m > n ? m : n) / 2;
    if (bound > 0) --bound;
    const int te = n < m + bound ? n : m + bound;
    const Txt t{b};
    int c = 0, tr = 0;
    const int W = (m + 63) / 64;
    if (variant == 0 || variant == 3) {
        if (m > 64 || te > 64) return -2;
        if (variant == 0) {
            const std::vector<u64> rows = table(a, m, 1);
            jaro_word(PM1{rows.data()}, m, t, n, &c, &tr);
        }
        else {
            std::vector<u64> rows(2 * 257, 0);
            for (int k = 0; k < m; ++k) {
                rows[a[k]] |= 1ull << k;
                rows[257 + a[k]] |= 1ull << k;
            }
            const int pl[2] = {m, m}, need[2] = {0, 0};
            int C[2] = {0, 0}, T[2] = {0, 0};
            group_jaro_word<2>(PMQ{rows.data()}, pl, 3u, t, n, need, C, T);
            if (C[0] != C[1] || T[0] != T[1]) return -3;
            c = C[0];
            tr = T[0];
        }
    }
    else if (variant == 1) {
        const int Wr = W <= 1 ? 1 : W <= 2 ? 2 : W <= 4 ? 4 : W <= 8 ? 8 : 0;
        if (!Wr) return -2;
        const std::vector<u64> rows = table(a, m, Wr);
        const PMW pm{rows.data(), Wr};
        switch (Wr) {
        case 1: jaro_multi<1>(pm, m, t, n, &c, &tr); break;
        case 2: jaro_multi<2>(pm, m, t, n, &c, &tr); break;
        case 4: jaro_multi<4>(pm, m, t, n, &c, &tr); break;
        default: jaro_multi<8>(pm, m, t, n, &c, &tr); break;
        }
    }
    else {
        const std::vector<u64> rows = table(a, m, W);
        std::vector<u64> f1((size_t)W), f2((size_t)W);
        jaro_multi_rt(PMW{rows.data(), W}, W, m, t, n, &c, &tr, f1.data(), f2.data());
    }
    *common = c;
    *transp = tr;
    return 0;
}

} /* extern "C" */
