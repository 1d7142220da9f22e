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

/* the unit-weight distance fast path of the warp tiles (fast_group, one query, the word
 * width of the query's launch: 32 bits for patterns of at most 32 units) */
uint64_t pair_steps(int metric, const HostPM& pm, int m, const uint8_t* t, int n, int K)
{
    uint64_t f = 0;
    const CountingText txt{t, &f};
    const HostPMQ pq{pm.row};
    const int mm[1] = {m};
    int d[1];
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
                uint64_t acc = 0;
                for (int64_t c = 0; c < nc; ++c)
                    acc += pair_steps(metric, pm, m, cd + co[c], (int)(co[c + 1] - co[c]), K);
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

} // extern "C"
