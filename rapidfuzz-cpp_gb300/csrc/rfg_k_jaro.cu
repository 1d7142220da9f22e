/* k_tiles instantiations of the JARO core family */
#include "rfg_device.cuh"
#include "rfg_kernels.h"

namespace rfg {

template <typename CT>
static const void* pick_jaro(int W, bool topk)
{
    switch (W) {
    case 1: return topk ? (const void*)&k_tiles<FAM_JARO, CT, 1, true> : (const void*)&k_tiles<FAM_JARO, CT, 1>;
    case 2: return topk ? (const void*)&k_tiles<FAM_JARO, CT, 2, true> : (const void*)&k_tiles<FAM_JARO, CT, 2>;
    case 4: return topk ? (const void*)&k_tiles<FAM_JARO, CT, 4, true> : (const void*)&k_tiles<FAM_JARO, CT, 4>;
    case 8: return topk ? (const void*)&k_tiles<FAM_JARO, CT, 8, true> : (const void*)&k_tiles<FAM_JARO, CT, 8>;
    }
    return nullptr;
}

const void* tiles_kernel_jaro(int width, int W, bool topk)
{
    switch (width) {
    case 1: return pick_jaro<uint8_t>(W, topk);
    case 2: return pick_jaro<uint16_t>(W, topk);
    case 4: return pick_jaro<uint32_t>(W, topk);
    case 8: return pick_jaro<unsigned long long>(W, topk);
    }
    return nullptr;
}

const void* tiles_mq_kernel_jaro(int width)
{
    switch (width) {
    case 1: return (const void*)&k_tiles_mq_jaro<uint8_t, 2>;
    case 2: return (const void*)&k_tiles_mq_jaro<uint16_t, 2>;
    case 4: return (const void*)&k_tiles_mq_jaro<uint32_t, 2>;
    case 8: return (const void*)&k_tiles_mq_jaro<unsigned long long, 2>;
    }
    return nullptr;
}

} // namespace rfg
