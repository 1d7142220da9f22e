/* k_generic instantiations of the token scorer family (dense results and extract lists) */
#include "rfg_device.cuh"
#include "rfg_kernels.h"

namespace rfg {

template <bool TOPK>
static const void* pick_token(int width)
{
    switch (width) {
    case 1: return (const void*)&k_generic<FAM_TOKEN, uint8_t, TOPK>;
    case 2: return (const void*)&k_generic<FAM_TOKEN, uint16_t, TOPK>;
    case 4: return (const void*)&k_generic<FAM_TOKEN, uint32_t, TOPK>;
    case 8: return (const void*)&k_generic<FAM_TOKEN, unsigned long long, TOPK>;
    }
    return nullptr;
}

const void* token_kernel(int width, bool topk) { return topk ? pick_token<true>(width) : pick_token<false>(width); }

} // namespace rfg
