/* Work accounting for the roofline of the single-word scoring kernels (host only).
 *
 * The device kernels stop a pair early once its diagonal lower bound exceeds the
 * cutoff (checked every 8 text characters) and skip pairs outside the length filter,
 * so the word steps they execute are fewer than the full n per pair that the
 * reference's single-word Hyyro loop runs (Levenshtein_impl.hpp:283-309,
 * LCSseq_impl.hpp:219-252, OSA_impl.hpp:49-71).  This file runs the same templated
 * cores as the kernels (rfg_core.cuh) on the host with a text accessor that counts
 * the characters fetched; for one-word patterns that count is the number of word
 * steps the kernel executes for the same (queries, choices, cutoff).  It computes no
 * result a caller sees.
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

struct CountingText {
    const uint8_t* p;
    uint64_t* fetched;
    u64 operator[](int j) const
    {
        ++*fetched;
        return p[j];
    }
};

/* the unit-weight distance fast path of the tile kernel (W = 1) */
uint64_t pair_steps(int metric, const HostPM& pm, int m, const uint8_t* t, int n, i64 K)
{
    uint64_t f = 0;
    const CountingText txt{t, &f};
    const i64 diff = m > n ? m - n : n - m;
    if (metric == 1) { /* Indel: LCS core */
        if (m == 0 || n == 0 || K < diff) return 0;
        (void)lcs_word(pm, m, txt, n, K);
        return f;
    }
    if (m == 0 || K < diff || n == 0) return 0;
    if (metric == 3) (void)osa_word(pm, m, txt, n, K);
    else (void)lev_word(pm, m, txt, n, K);
    return f;
}
} // namespace

extern "C" {

/* metric: 0 Levenshtein (1/1/1), 1 Indel, 3 OSA; uint8 strings, every query <= 64
 * code units; distance cutoff.  Returns 0 and the executed word steps in *steps, or -1
 * for an input outside that shape. */
int rfg_count_word_steps(int metric, const uint8_t* qd, const int64_t* qo, int64_t nq, const uint8_t* cd,
                         const int64_t* co, int64_t nc, uint64_t cutoff, int nthreads, uint64_t* steps)
{
    if (!steps || (metric != 0 && metric != 1 && metric != 3)) return -1;
    for (int64_t i = 0; i < nq; ++i)
        if (qo[i + 1] - qo[i] > 64) return -1;
    const i64 K = clamp_bound(cutoff);
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int64_t> next(0);
    std::vector<uint64_t> part(nthreads, 0);
    std::vector<std::thread> th;
    for (int w = 0; w < nthreads; ++w)
        th.emplace_back([&, w]() {
            HostPM pm;
            uint64_t acc = 0;
            for (;;) {
                const int64_t qi = next.fetch_add(1);
                if (qi >= nq) break;
                const int m = (int)(qo[qi + 1] - qo[qi]);
                std::fill(pm.row, pm.row + 256, 0ull);
                for (int k = 0; k < m; ++k) pm.row[qd[qo[qi] + k]] |= 1ull << k;
                for (int64_t c = 0; c < nc; ++c)
                    acc += pair_steps(metric, pm, m, cd + co[c], (int)(co[c + 1] - co[c]), K);
            }
            part[w] = acc;
        });
    for (auto& t : th) t.join();
    uint64_t s = 0;
    for (uint64_t v : part) s += v;
    *steps = s;
    return 0;
}

} // extern "C"
