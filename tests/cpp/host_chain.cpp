/* One scorer call the way the kernels make it: the pair's plan and formula chains
 * (plan_int / finish_int / finish_jaro in rfg_core.cuh) around the runtime-W cores, as the
 * any-length kernel runs them (score_pair_generic), or with the tile kernels' per-query
 * length tables; compiled for the host behind the oracle's rfo_score signature, so the
 * CPU tests can run the reference-made fixtures through the device code's chains.
 * Code units of any width: units below 256 index the table directly, wider ones get a row
 * each (a text unit the pattern lacks reads a zero row), as the kernels' hashed rows do. */
#include <stdint.h>
#include <string.h>

#include <map>
#include <vector>

#include "rfg_core.cuh"

using namespace rfg;

namespace {

struct Params {
    int64_t ins, del, rep;
    double prefix_weight;
};
struct PMRows {
    const u64* rows;
    int W;
    u64 operator()(u64 r, int w) const { return rows[r * (u64)W + w]; }
};
struct Seq {
    const u64* p;
    u64 operator[](int j) const { return p[j]; }
};

std::vector<u64> widen(const void* s, int64_t n, int w)
{
    std::vector<u64> v((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        switch (w) {
        case 1: v[i] = ((const uint8_t*)s)[i]; break;
        case 2: v[i] = ((const uint16_t*)s)[i]; break;
        case 4: v[i] = ((const uint32_t*)s)[i]; break;
        default: v[i] = ((const uint64_t*)s)[i]; break;
        }
    }
    return v;
}

/* tables: the per-query length tables of the tile kernels (text lengths up to
 * RFG_JT_MAXT): the Jaro table (jaro_tab_head / jaro_tab_minc, finish_jaro_tab or the
 * failing value) and the normalized chains' integer cutoff (chain_kd as kd_pre) */
int score(int metric, int op, int form, const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb,
          const Params* p, uint64_t ci, double cf, int64_t* oi, double* of, bool tables)
{
    if (metric < 0 || metric > RATIO) return -1;
    const std::vector<u64> A = widen(a, la, ca), B = widen(b, lb, cb);
    std::map<u64, u64> wide;
    for (u64 x : A)
        if (x >= 256 && !wide.count(x)) wide.emplace(x, 256 + wide.size());
    const u64 zero_row = 256 + wide.size();
    std::vector<u64> rb((size_t)lb);
    for (int64_t j = 0; j < lb; ++j) {
        const u64 x = B[j];
        rb[j] = x < 256 ? x : (wide.count(x) ? wide[x] : zero_row);
    }
    const int m = (int)la, n = (int)lb, W = m > 0 ? (m + 63) / 64 : 1;
    std::vector<u64> table((size_t)(zero_row + 1) * W, 0);
    for (int k = 0; k < m; ++k) table[(A[k] < 256 ? A[k] : wide[A[k]]) * W + k / 64] |= 1ull << (k % 64);
    const PMRows pm{table.data(), W};
    const Seq txt{rb.data()}, q{A.data()}, t2{B.data()};
    std::vector<u64> st((size_t)(4 * W + m + 8));

    PairSpec s;
    s.metric = metric;
    s.op = op;
    s.form = form;
    s.l1 = (u64)m;
    s.l2 = (u64)n;
    s.ci = ci;
    s.cf = cf;
    s.p = ScoreParams{p->ins, p->del, p->rep, p->prefix_weight};
    const int fam = metric_family(metric, form, s.p);
    *oi = 0;
    *of = 0.0;
    const bool tab = tables && n <= RFG_JT_MAXT && form != FORM_MULTI; /* the kernels: no tables for Multi */
    if (fam == FAM_JARO) {
        i64 prefix = 0;
        const int mx = (m < n ? m : n) < 4 ? (m < n ? m : n) : 4;
        for (; prefix < mx; ++prefix)
            if (B[prefix] != A[prefix]) break;
        int common = 0, transp = 0;
        if (tab) {
            JaroTab jt;
            jaro_tab_head(jt, s);
            const unsigned short mc = jaro_tab_minc(s, m, (int)prefix, n);
            jt.minc[prefix][n] = mc;
            const int cmax = m < n ? m : n;
            const bool one = m == 1 && n == 1;
            bool fail = mc != 0 && !one && (mc == 0xffff || cmax < (int)mc);
            if (mc != 0 && !fail) {
                jaro_multi_rt(pm, W, m, txt, n, &common, &transp, st.data(), st.data() + W);
                fail = common < (one ? 0 : (int)mc);
            }
            if (mc == 0 && !(m == 0 && n == 0)) fail = true;
            *of = fail ? jt.vfail[prefix] : finish_jaro_tab(s, jt, prefix, common, transp);
            return 0;
        }
        if (m > 0 && n > 0 && jaro_pair_needs_counts(s, prefix))
            jaro_multi_rt(pm, W, m, txt, n, &common, &transp, st.data(), st.data() + W);
        *of = finish_jaro(s, prefix, common, transp);
        return 0;
    }
    if (tab && (metric == RATIO || op >= NORM_DISTANCE)) s.kd_pre = chain_kd(s);
    const Plan pl = plan_int(s);
    i64 raw = 0;
    if (pl.run) {
        const i64 K = pl.K;
        const i64 diff = m > n ? m - n : n - m;
        if (fam == FAM_WF) raw = (i64)wf_distance(q, m, t2, n, s.p, (u64)K, st.data());
        else if (fam == FAM_LCS) {
            if (m == 0 || n == 0) raw = 0;
            else if (K < diff) raw = -1;
            else raw = lcs_multi_rt(pm, W, m, txt, n, K, st.data());
        }
        else if (m == 0) raw = n;
        else if (K < diff) raw = K + 1;
        else if (n == 0) raw = m;
        else if (fam == FAM_OSA)
            raw = osa_multi_rt(pm, W, m, txt, n, K, st.data(), st.data() + W, st.data() + 2 * W, st.data() + 3 * W);
        else if (K < m && 2 * K + 1 <= 64) raw = lev_band<1>(pm, W, m, txt, n, (int)K);
        else if (K < m && 2 * K + 1 <= 128) raw = lev_band<2>(pm, W, m, txt, n, (int)K);
        else if (K < m && 2 * K + 1 <= 256) raw = lev_band<4>(pm, W, m, txt, n, (int)K);
        else if (K < m && 2 * K + 1 <= 512) raw = lev_band<8>(pm, W, m, txt, n, (int)K);
        else raw = lev_multi_rt(pm, W, m, txt, n, K, st.data(), st.data() + W);
    }
    finish_int(s, pl, raw, oi, of);
    return 0;
}

} // namespace

extern "C" {

/* rfo_score's arguments; free, Cached and Multi forms of Levenshtein .. ratio (metrics 0..6):
 * the any-length kernel's path (hc_score) and the tile kernels' table path
 * (hc_score_tab).  Return 0, or -1 for a metric outside that set. */
int hc_score(int metric, int op, int form, const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb,
             const Params* p, uint64_t ci, double cf, int64_t* oi, double* of)
{
    return score(metric, op, form, a, la, ca, b, lb, cb, p, ci, cf, oi, of, false);
}

int hc_score_tab(int metric, int op, int form, const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb,
                 const Params* p, uint64_t ci, double cf, int64_t* oi, double* of)
{
    return score(metric, op, form, a, la, ca, b, lb, cb, p, ci, cf, oi, of, true);
}

} /* extern "C" */
