/* k_generic instantiations (any-length cores and weighted Wagner-Fischer) */
#include "rfg_device.cuh"
#include "rfg_kernels.h"

namespace rfg {

template <typename CT, bool TOPK>
static const void* pick_generic(int fam)
{
    switch (fam) {
    case FAM_LEV: return (const void*)&k_generic<FAM_LEV, CT, TOPK>;
    case FAM_LCS: return (const void*)&k_generic<FAM_LCS, CT, TOPK>;
    case FAM_OSA: return (const void*)&k_generic<FAM_OSA, CT, TOPK>;
    case FAM_JARO: return (const void*)&k_generic<FAM_JARO, CT, TOPK>;
    case FAM_WF: return (const void*)&k_generic<FAM_WF, CT, TOPK>;
    case FAM_PARTIAL: return (const void*)&k_generic<FAM_PARTIAL, CT, TOPK>;
    }
    return nullptr;
}

const void* generic_kernel(int fam, int width, bool topk)
{
    if (fam == FAM_TOKEN) return token_kernel(width, topk);
    switch (width) {
    case 1: return topk ? pick_generic<uint8_t, true>(fam) : pick_generic<uint8_t, false>(fam);
    case 2: return topk ? pick_generic<uint16_t, true>(fam) : pick_generic<uint16_t, false>(fam);
    case 4: return topk ? pick_generic<uint32_t, true>(fam) : pick_generic<uint32_t, false>(fam);
    case 8: return topk ? pick_generic<unsigned long long, true>(fam) : pick_generic<unsigned long long, false>(fam);
    }
    return nullptr;
}

const void* topk_merge_kernel() { return (const void*)&k_topk_merge; }

const void* jaro_tables_kernel() { return (const void*)&k_jaro_tables; }

/* QRatio's empty-string rule (fuzz_impl.hpp:887-931) on a device result matrix: the
 * entries (rows[i], cols[j]) are set to 0 (ratio gives 100 where both strings are
 * empty).  Grid-stride over nr * ncol entries. */
__global__ void k_zero_pairs(double* out, int64_t ld, const int64_t* rows, int64_t nr, const int64_t* cols,
                             int64_t ncol)
{
    const int64_t total = nr * ncol;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
        out[rows[t / ncol] * ld + cols[t % ncol]] = 0.0;
}

const void* zero_pairs_kernel() { return (const void*)&k_zero_pairs; }

} // namespace rfg
