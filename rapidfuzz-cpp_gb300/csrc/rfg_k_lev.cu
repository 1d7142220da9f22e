/* k_tiles instantiations of the LEV core family */
#include "rfg_device.cuh"
#include "rfg_fast.cuh"
#include "rfg_kernels.h"

namespace rfg {

template <typename CT>
static const void* pick_lev(int W, bool topk)
{
    switch (W) {
    case 1: return topk ? (const void*)&k_tiles<FAM_LEV, CT, 1, true> : (const void*)&k_tiles<FAM_LEV, CT, 1>;
    case 2: return topk ? (const void*)&k_tiles<FAM_LEV, CT, 2, true> : (const void*)&k_tiles<FAM_LEV, CT, 2>;
    case 4: return topk ? (const void*)&k_tiles<FAM_LEV, CT, 4, true> : (const void*)&k_tiles<FAM_LEV, CT, 4>;
    case 8: return topk ? (const void*)&k_tiles<FAM_LEV, CT, 8, true> : (const void*)&k_tiles<FAM_LEV, CT, 8>;
    }
    return nullptr;
}

const void* tiles_kernel_lev(int width, int W, bool topk)
{
    switch (width) {
    case 1: return pick_lev<uint8_t>(W, topk);
    case 2: return pick_lev<uint16_t>(W, topk);
    case 4: return pick_lev<uint32_t>(W, topk);
    case 8: return pick_lev<unsigned long long>(W, topk);
    }
    return nullptr;
}

template <typename CT>
static const void* pick_mq_lev(bool norm, bool half)
{
    if (half)
        return norm ? (const void*)&k_tiles_mq<FAM_LEV, CT, true, 2, true>
                    : (const void*)&k_tiles_mq<FAM_LEV, CT, false, 2, true>;
    return norm ? (const void*)&k_tiles_mq<FAM_LEV, CT, true, 2> : (const void*)&k_tiles_mq<FAM_LEV, CT, false, 2>;
}

const void* tiles_mq_kernel_lev(int width, bool norm, bool half)
{
    switch (width) {
    case 1: return pick_mq_lev<uint8_t>(norm, half);
    case 2: return pick_mq_lev<uint16_t>(norm, half);
    case 4: return pick_mq_lev<uint32_t>(norm, half);
    case 8: return pick_mq_lev<unsigned long long>(norm, half);
    }
    return nullptr;
}

template <typename CT>
static const void* pick_fast_lev(bool half)
{
    return half ? (const void*)&k_fast<FAM_LEV, CT, 2, true> : (const void*)&k_fast<FAM_LEV, CT, 2, false>;
}

const void* fast_hist_kernel() { return (const void*)&k_fast_hist; }

const void* fast_kernel_lev(int width, bool half)
{
    switch (width) {
    case 1: return pick_fast_lev<uint8_t>(half);
    case 2: return pick_fast_lev<uint16_t>(half);
    case 4: return pick_fast_lev<uint32_t>(half);
    case 8: return pick_fast_lev<unsigned long long>(half);
    }
    return nullptr;
}

} // namespace rfg
