/* k_tiles instantiations of the LCS core family */
#include "rfg_device.cuh"
#include "rfg_fast.cuh"
#include "rfg_kernels.h"

namespace rfg {

template <typename CT>
static const void* pick_lcs(int W, bool topk)
{
    switch (W) {
    case 1: return topk ? (const void*)&k_tiles<FAM_LCS, CT, 1, true> : (const void*)&k_tiles<FAM_LCS, CT, 1>;
    case 2: return topk ? (const void*)&k_tiles<FAM_LCS, CT, 2, true> : (const void*)&k_tiles<FAM_LCS, CT, 2>;
    case 4: return topk ? (const void*)&k_tiles<FAM_LCS, CT, 4, true> : (const void*)&k_tiles<FAM_LCS, CT, 4>;
    case 8: return topk ? (const void*)&k_tiles<FAM_LCS, CT, 8, true> : (const void*)&k_tiles<FAM_LCS, CT, 8>;
    }
    return nullptr;
}

const void* tiles_kernel_lcs(int width, int W, bool topk)
{
    switch (width) {
    case 1: return pick_lcs<uint8_t>(W, topk);
    case 2: return pick_lcs<uint16_t>(W, topk);
    case 4: return pick_lcs<uint32_t>(W, topk);
    case 8: return pick_lcs<unsigned long long>(W, topk);
    }
    return nullptr;
}

template <typename CT>
static const void* pick_mq_lcs(bool norm, bool half)
{
    if (half)
        return norm ? (const void*)&k_tiles_mq<FAM_LCS, CT, true, 4, true>
                    : (const void*)&k_tiles_mq<FAM_LCS, CT, false, 4, true>;
    return norm ? (const void*)&k_tiles_mq<FAM_LCS, CT, true, 4> : (const void*)&k_tiles_mq<FAM_LCS, CT, false, 4>;
}

const void* tiles_mq_kernel_lcs(int width, bool norm, bool half)
{
    switch (width) {
    case 1: return pick_mq_lcs<uint8_t>(norm, half);
    case 2: return pick_mq_lcs<uint16_t>(norm, half);
    case 4: return pick_mq_lcs<uint32_t>(norm, half);
    case 8: return pick_mq_lcs<unsigned long long>(norm, half);
    }
    return nullptr;
}

template <typename CT>
static const void* pick_fast_lcs(bool half)
{
    return half ? (const void*)&k_fast<FAM_LCS, CT, RFG_FAST_LCS_Q, true> : (const void*)&k_fast<FAM_LCS, CT, RFG_FAST_LCS_Q, false>;
}

const void* fast_kernel_lcs(int width, bool half)
{
    switch (width) {
    case 1: return pick_fast_lcs<uint8_t>(half);
    case 2: return pick_fast_lcs<uint16_t>(half);
    case 4: return pick_fast_lcs<uint32_t>(half);
    case 8: return pick_fast_lcs<unsigned long long>(half);
    }
    return nullptr;
}

} // namespace rfg
