/* k_generic instantiations (any-length cores and weighted Wagner-Fischer) */
#include "rfg_device.cuh"
#include "rfg_kernels.h"

namespace rfg {

template <typename CT>
static const void* pick_generic(int fam)
{
    switch (fam) {
    case FAM_LEV: return (const void*)&k_generic<FAM_LEV, CT>;
    case FAM_LCS: return (const void*)&k_generic<FAM_LCS, CT>;
    case FAM_OSA: return (const void*)&k_generic<FAM_OSA, CT>;
    case FAM_JARO: return (const void*)&k_generic<FAM_JARO, CT>;
    case FAM_WF: return (const void*)&k_generic<FAM_WF, CT>;
    }
    return nullptr;
}

const void* generic_kernel(int fam, int width)
{
    switch (width) {
    case 1: return pick_generic<uint8_t>(fam);
    case 2: return pick_generic<uint16_t>(fam);
    case 4: return pick_generic<uint32_t>(fam);
    case 8: return pick_generic<unsigned long long>(fam);
    }
    return nullptr;
}

} // namespace rfg
