/* The fuzz scorers of the device path (partial_ratio_dev, token_family_dev in
 * rfg_core.cuh, the templates the kernels instantiate) compiled for the host behind a C
 * entry point for the CPU tests, with the host token front end (rfg_token.cpp) making the
 * [string][S][J] part concatenations the kernels read.  One-byte strings. */
#include <stdint.h>

#include <vector>

#include "rfg_core.cuh"
#include "rfg_token.h"

using namespace rfg;

namespace {

struct PMRows { /* W-word table over the table rows (one-byte units: the unit) */
    const u64* rows;
    int W;
    u64 operator()(u64 c, int w) const { return rows[c * (u64)W + w]; }
};
struct Units {
    const uint8_t* p;
    u64 operator[](int j) const { return p[j]; }
};

std::vector<u64> table(const uint8_t* a, int m, int W)
{
    std::vector<u64> rows((size_t)256 * W, 0);
    for (int k = 0; k < m; ++k) rows[(size_t)a[k] * W + k / 64] |= 1ull << (k % 64);
    return rows;
}

} // namespace

extern "C" {

/* metric: 7 partial_ratio (the pair itself), 8..15 the token scorers over the part
 * concatenations (token_sort_ratio .. WRatio, numbered as in the C ABI); *out = the
 * similarity with the cutoff.  Returns 0, or -1 for another metric. */
int hf_score(int metric, const uint8_t* a, int64_t la, const uint8_t* b, int64_t lb, double cutoff, double* out)
{
    if (metric == 7) {
        const int W = la > 0 ? (int)((la + 63) / 64) : 1;
        const std::vector<u64> rows = table(a, (int)la, W);
        std::vector<u64> st((size_t)(W + 1 + (5 * (la > lb ? la : lb) + 3) / 2 + 64));
        const PMRows pm{rows.data(), W};
        *out = partial_ratio_dev(pm, W, (int)la, Units{b}, (int)lb, cutoff, st.data(), (u32*)(st.data() + W + 1));
        return 0;
    }
    if (metric < 8 || metric > 15) return -1;
    const int64_t oa[2] = {0, la}, ob[2] = {0, lb};
    std::vector<unsigned char> da, db;
    std::vector<int64_t> fa, fb;
    std::vector<int32_t> pa, pb;
    token_parts_set(a, oa, 1, 1, true, true, true, &da, &fa, &pa);
    token_parts_set(b, ob, 1, 1, true, true, true, &db, &fb, &pb);
    const int La = (int)fa[1], Lb = (int)fb[1];
    const int W = La > 0 ? (La + 63) / 64 : 1;
    const std::vector<u64> rows = table(da.data(), La, W);
    const PMRows pm{rows.data(), W};
    const Units q{da.data()}, t{db.data()};
    std::vector<u64> st((size_t)tok_scratch_words(W, La > Lb ? La : Lb) + 64);
    typedef TokPair<PMRows, Units, Units, Units> Pair;
    const Pair p{&pm, W, &q, &t, &t, pa[0], pa[1], pa[2], pb[0], pb[1], pb[2]};
    *out = token_family_dev(metric, p, cutoff, st.data());
    return 0;
}

} /* extern "C" */
