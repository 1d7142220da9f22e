/* k_tiles instantiations of the OSA core family */
#include "rfg_device.cuh"
#include "rfg_fast.cuh"
#include "rfg_kernels.h"

namespace rfg {

template <typename CT>
static const void* pick_osa(int W, bool topk)
{
    switch (W) {
    case 1: return topk ? (const void*)&k_tiles<FAM_OSA, CT, 1, true> : (const void*)&k_tiles<FAM_OSA, CT, 1>;
    case 2: return topk ? (const void*)&k_tiles<FAM_OSA, CT, 2, true> : (const void*)&k_tiles<FAM_OSA, CT, 2>;
    case 4: return topk ? (const void*)&k_tiles<FAM_OSA, CT, 4, true> : (const void*)&k_tiles<FAM_OSA, CT, 4>;
    case 8: return topk ? (const void*)&k_tiles<FAM_OSA, CT, 8, true> : (const void*)&k_tiles<FAM_OSA, CT, 8>;
    }
    return nullptr;
}

const void* tiles_kernel_osa(int width, int W, bool topk)
{
    switch (width) {
    case 1: return pick_osa<uint8_t>(W, topk);
    case 2: return pick_osa<uint16_t>(W, topk);
    case 4: return pick_osa<uint32_t>(W, topk);
    case 8: return pick_osa<unsigned long long>(W, topk);
    }
    return nullptr;
}

template <typename CT>
static const void* pick_mq_osa(bool norm, bool half)
{
    if (half)
        return norm ? (const void*)&k_tiles_mq<FAM_OSA, CT, true, 2, true>
                    : (const void*)&k_tiles_mq<FAM_OSA, CT, false, 2, true>;
    return norm ? (const void*)&k_tiles_mq<FAM_OSA, CT, true, 2> : (const void*)&k_tiles_mq<FAM_OSA, CT, false, 2>;
}

const void* tiles_mq_kernel_osa(int width, bool norm, bool half)
{
    switch (width) {
    case 1: return pick_mq_osa<uint8_t>(norm, half);
    case 2: return pick_mq_osa<uint16_t>(norm, half);
    case 4: return pick_mq_osa<uint32_t>(norm, half);
    case 8: return pick_mq_osa<unsigned long long>(norm, half);
    }
    return nullptr;
}

template <typename CT>
static const void* pick_fast_osa(bool half)
{
    return half ? (const void*)&k_fast<FAM_OSA, CT, 2, true> : (const void*)&k_fast<FAM_OSA, CT, 2, false>;
}

const void* fast_kernel_osa(int width, bool half)
{
    switch (width) {
    case 1: return pick_fast_osa<uint8_t>(half);
    case 2: return pick_fast_osa<uint16_t>(half);
    case 4: return pick_fast_osa<uint32_t>(half);
    case 8: return pick_fast_osa<unsigned long long>(half);
    }
    return nullptr;
}

} // namespace rfg
