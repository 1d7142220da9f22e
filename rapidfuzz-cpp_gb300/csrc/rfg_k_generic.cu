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

} // namespace rfg
