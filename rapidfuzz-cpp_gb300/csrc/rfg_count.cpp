/* Work accounting for the roofline of the single-word scoring kernels (host only).
 *
 * The device kernels stop a pair early once its diagonal lower bound exceeds the
 * cutoff (checked every 8 text characters) and skip pairs outside the length filter,
 * so the word steps they execute are fewer than the full n per pair that the
 * reference's single-word Hyyro loop runs (Levenshtein_impl.hpp:283-309,
 * LCSseq_impl.hpp:219-252, OSA_impl.hpp:49-71).  This file runs the core the warp tiles
 * run (fast_group in rfg_core.cuh) on the host with a text accessor that counts the
 * characters fetched; for one-word patterns that count is the number of word steps the
 * kernels execute for the same (queries, choices, cutoff), split by the word width of
 * the query's launch.  It computes no result a caller sees.
 */
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "rfg_core.cuh"

namespace {
using namespace rfg;

struct HostPM {
    u64 row[256];
    u64 operator()(u64 c) const { return row[c & 255]; }
};

struct Txt8 {
    const uint8_t* p;
    u64 operator[](int j) const { return p[j]; }
};

struct CountingText {
    const uint8_t* p;
    uint64_t* fetched;
    u64 operator[](int j) const
    {
        ++*fetched;
        return p[j];
    }
};

struct HostPMQ {
    const u64* row;
    u64 operator()(int, unsigned c) const { return row[c]; }
};

/* a string's count histogram (hist_lower_bound), for strings of at most
 * RFG_HIST_MAXLEN units */
void host_hist(const uint8_t* s, int n, u32* h)
{
    unsigned char b[32] = {0};
    if (n <= RFG_HIST_MAXLEN)
        for (int i = 0; i < n; ++i) ++b[s[i] & 31];
    for (int w = 0; w < 8; ++w) h[w] = (u32)b[4 * w] | (u32)b[4 * w + 1] << 8 | (u32)b[4 * w + 2] << 16 | (u32)b[4 * w + 3] << 24;
}

/* the unit-weight distance fast path of the warp tiles (fast_group, one query, the word
 * width of the query's launch: 32 bits for patterns of at most 32 units), with the count
 * filter the tiles apply below cutoffs of 2 * RFG_HIST_MAXLEN */
uint64_t pair_steps(int metric, const HostPM& pm, int m, const uint8_t* t, int n, int K, const u32* hq)
{
    uint64_t f = 0;
    const CountingText txt{t, &f};
    const HostPMQ pq{pm.row};
    const int mm[1] = {m};
    int d[1];
    if (K < 2 * RFG_HIST_MAXLEN && n <= RFG_HIST_MAXLEN) {
        u32 hc[8];
        host_hist(t, n, hc);
        const int diff = m > n ? m - n : n - m;
        if (m > 0 && n > 0 && K >= diff && hist_lower_bound(metric == 1 ? FAM_LCS : FAM_LEV, hq, hc, m, n) > K) return 0;
    }
    if (m <= 32) {
        if (metric == 1) fast_group<FAM_LCS, 1, HostPMQ, CountingText, u32>(pq, mm, 1, txt, n, K, d);
        else if (metric == 3) fast_group<FAM_OSA, 1, HostPMQ, CountingText, u32>(pq, mm, 1, txt, n, K, d);
        else fast_group<FAM_LEV, 1, HostPMQ, CountingText, u32>(pq, mm, 1, txt, n, K, d);
    }
    else {
        if (metric == 1) fast_group<FAM_LCS, 1, HostPMQ, CountingText, u64>(pq, mm, 1, txt, n, K, d);
        else if (metric == 3) fast_group<FAM_OSA, 1, HostPMQ, CountingText, u64>(pq, mm, 1, txt, n, K, d);
        else fast_group<FAM_LEV, 1, HostPMQ, CountingText, u64>(pq, mm, 1, txt, n, K, d);
    }
    return f;
}
} // namespace

extern "C" {

/* the warp tiles' count filter on the same inputs as rfg_count_word_steps2: *checks =
 * (query, choice) pairs it examines (both lengths at most RFG_HIST_MAXLEN, the length
 * filter passed, a cutoff below 2 * RFG_HIST_MAXLEN), *survivors = those whose bound
 * does not exceed the cutoff (they run the recurrence) */
int rfg_count_filter(int metric, const uint8_t* qd, const int64_t* qo, int64_t nq, const uint8_t* cd,
                     const int64_t* co, int64_t nc, uint64_t cutoff, uint64_t* checks, uint64_t* survivors)
{
    if (!checks || !survivors || (metric != 0 && metric != 1 && metric != 3)) return -1;
    *checks = *survivors = 0;
    const int K = (int)std::min<uint64_t>(cutoff, 0x7fffffffull);
    if (K >= 2 * RFG_HIST_MAXLEN) return 0;
    std::vector<u32> hc((size_t)nc * 8);
    for (int64_t c = 0; c < nc; ++c) host_hist(cd + co[c], (int)(co[c + 1] - co[c]), &hc[(size_t)c * 8]);
    for (int64_t i = 0; i < nq; ++i) {
        const int m = (int)(qo[i + 1] - qo[i]);
        if (m == 0 || m > RFG_HIST_MAXLEN) continue;
        u32 hq[8];
        host_hist(qd + qo[i], m, hq);
        for (int64_t c = 0; c < nc; ++c) {
            const int n = (int)(co[c + 1] - co[c]);
            if (n == 0 || n > RFG_HIST_MAXLEN || (m > n ? m - n : n - m) > K) continue;
            ++*checks;
            if (hist_lower_bound(metric == 1 ? FAM_LCS : FAM_LEV, hq, &hc[(size_t)c * 8], m, n) <= K) ++*survivors;
        }
    }
    return 0;
}

/* metric: 0 Levenshtein (1/1/1), 1 Indel, 3 OSA; uint8 strings, every query <= 64
 * code units; distance cutoff.  Returns 0 and the executed word steps of queries of
 * 33..64 units (64-bit words) in *steps64 and of queries of at most 32 units (32-bit
 * words) in *steps32, or -1 for an input outside that shape. */
int rfg_count_word_steps2(int metric, const uint8_t* qd, const int64_t* qo, int64_t nq, const uint8_t* cd,
                          const int64_t* co, int64_t nc, uint64_t cutoff, int nthreads, uint64_t* steps64,
                          uint64_t* steps32)
{
    if (!steps64 || !steps32 || (metric != 0 && metric != 1 && metric != 3)) return -1;
    for (int64_t i = 0; i < nq; ++i)
        if (qo[i + 1] - qo[i] > 64) return -1;
    const int K = (int)std::min<uint64_t>(cutoff, 0x7fffffffull);
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int64_t> next(0);
    std::vector<uint64_t> p64(nthreads, 0), p32(nthreads, 0);
    std::vector<std::thread> th;
    for (int w = 0; w < nthreads; ++w)
        th.emplace_back([&, w]() {
            HostPM pm;
            uint64_t a64 = 0, a32 = 0;
            for (;;) {
                const int64_t qi = next.fetch_add(1);
                if (qi >= nq) break;
                const int m = (int)(qo[qi + 1] - qo[qi]);
                std::fill(pm.row, pm.row + 256, 0ull);
                for (int k = 0; k < m; ++k) pm.row[qd[qo[qi] + k]] |= 1ull << k;
                u32 hq[8];
                host_hist(qd + qo[qi], m, hq);
                uint64_t acc = 0;
                for (int64_t c = 0; c < nc; ++c)
                    acc += pair_steps(metric, pm, m, cd + co[c], (int)(co[c + 1] - co[c]), K, hq);
                (m <= 32 ? a32 : a64) += acc;
            }
            p64[w] = a64;
            p32[w] = a32;
        });
    for (auto& t : th) t.join();
    *steps64 = *steps32 = 0;
    for (int w = 0; w < nthreads; ++w) {
        *steps64 += p64[w];
        *steps32 += p32[w];
    }
    return 0;
}

/* Band classes of unit-weight Levenshtein or of an LCS family (metric in rfg_metric
 * numbering; the band kernel, lev_band32 / lcs_band32) on one-byte strings under the
 * chain of `op` (rfg_op numbering) with the cutoff ci / cf: for every
 * pair of a band-class query that passes the length filter, the text units the core
 * fetches (steps) times the class's window words (*exec_words, what the kernel runs) and
 * times the words Ukkonen's band of the pair needs (*alg_words); *pairs counts those
 * pairs.  Queries outside the band classes are not counted. */
int rfg_count_band_steps(int metric, int op, uint64_t ci, double cf, const uint8_t* qd, const int64_t* qo, int64_t nq,
                         const uint8_t* cd, const int64_t* co, int64_t nc, int nthreads, uint64_t* exec_words,
                         uint64_t* alg_words, uint64_t* pairs)
{
    if (!exec_words || !alg_words || !pairs) return -1;
    int64_t maxlen = 0;
    for (int64_t c = 0; c < nc; ++c) maxlen = std::max<int64_t>(maxlen, co[c + 1] - co[c]);
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    ScoreParams sp;
    sp.ins = sp.del = sp.rep = 1;
    sp.prefix_weight = 0.1;
    std::atomic<int64_t> next(0);
    std::vector<uint64_t> pe(nthreads, 0), pa(nthreads, 0), pp(nthreads, 0);
    std::vector<std::thread> th;
    for (int w = 0; w < nthreads; ++w)
        th.emplace_back([&, w]() {
            for (;;) {
                const int64_t qi = next.fetch_add(1);
                if (qi >= nq) break;
                const int m = (int)(qo[qi + 1] - qo[qi]);
                const int bc = band_class(metric, op, FORM_CACHED, sp, ci, cf, m, maxlen);
                if (bc < 0) continue;
                const int B = band_class_words(bc);
                const uint8_t* a = qd + qo[qi];
                const int W32 = (m + 31) / 32, pad = B + 1, S = W32 + 3 * pad;
                std::vector<int32_t> rmap(256, 0);
                int R = 1;
                for (int k = 0; k < m; ++k)
                    if (!rmap[a[k]]) rmap[a[k]] = R++;
                std::vector<uint32_t> rows((size_t)R * S, 0);
                for (int k = 0; k < m; ++k) rows[(size_t)rmap[a[k]] * S + pad + k / 32] |= 1u << (k % 32);
                for (int c = 0; c < 256; ++c) rmap[c] = rmap[c] * S + pad;
                struct PM {
                    const uint32_t* base;
                    const int32_t* rmap;
                    const uint32_t* operator()(u64 c) const { return base + rmap[c & 255]; }
                } pm{rows.data(), rmap.data()};
                PairSpec s;
                s.metric = metric;
                s.op = op;
                s.form = FORM_CACHED;
                s.ci = ci;
                s.cf = cf;
                s.p = sp;
                s.l1 = (u64)m;
                for (int64_t c = 0; c < nc; ++c) {
                    const int n = (int)(co[c + 1] - co[c]);
                    s.l2 = (u64)n;
                    s.kd_pre = ~0ull;
                    const Plan pl = plan_int(s);
                    if (!pl.run || n == 0) continue;
                    const i64 K = pl.K, diff = m > n ? m - n : n - m;
                    if (K < diff || K >= m) continue;
                    int st = 0;
                    const Txt8 txt{cd + co[c]};
                    if (metric != LEVENSHTEIN) switch (B) {
                        case 1: lcs_band32<1>(pm, m, txt, n, (int)K, &st); break;
                        case 2: lcs_band32<2>(pm, m, txt, n, (int)K, &st); break;
                        case 3: lcs_band32<3>(pm, m, txt, n, (int)K, &st); break;
                        case 4: lcs_band32<4>(pm, m, txt, n, (int)K, &st); break;
                        case 6: lcs_band32<6>(pm, m, txt, n, (int)K, &st); break;
                        case 8: lcs_band32<8>(pm, m, txt, n, (int)K, &st); break;
                        case 12: lcs_band32<12>(pm, m, txt, n, (int)K, &st); break;
                        default: lcs_band32<16>(pm, m, txt, n, (int)K, &st); break;
                        }
                    else switch (B) {
                    case 1: lev_band32<1>(pm, m, txt, n, (int)K, &st); break;
                    case 2: lev_band32<2>(pm, m, txt, n, (int)K, &st); break;
                    case 3: lev_band32<3>(pm, m, txt, n, (int)K, &st); break;
                    case 4: lev_band32<4>(pm, m, txt, n, (int)K, &st); break;
                    case 6: lev_band32<6>(pm, m, txt, n, (int)K, &st); break;
                    case 8: lev_band32<8>(pm, m, txt, n, (int)K, &st); break;
                    case 12: lev_band32<12>(pm, m, txt, n, (int)K, &st); break;
                    default: lev_band32<16>(pm, m, txt, n, (int)K, &st); break;
                    }
                    /* the steps the kernel runs: every unit up to the end of the 8-unit
                     * block at which the pair ends */
                    pe[w] += (uint64_t)st * (uint64_t)B;
                    pa[w] += (uint64_t)st * (uint64_t)((band_bits((int)K, m - n) + 31) / 32);
                    ++pp[w];
                }
            }
        });
    for (auto& t : th) t.join();
    *exec_words = *alg_words = *pairs = 0;
    for (int w = 0; w < nthreads; ++w) {
        *exec_words += pe[w];
        *alg_words += pa[w];
        *pairs += pp[w];
    }
    return 0;
}

} // extern "C"
