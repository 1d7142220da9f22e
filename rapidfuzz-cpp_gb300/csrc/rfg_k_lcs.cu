/* k_tiles instantiations of the LCS core family */
#include "rfg_device.cuh"
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

const void* tiles_mq_kernel_lcs(int width, bool norm)
{
    switch (width) {
    case 1:
        return norm ? (const void*)&k_tiles_mq<FAM_LCS, uint8_t, true, 4>
                    : (const void*)&k_tiles_mq<FAM_LCS, uint8_t, false, 4>;
    case 2:
        return norm ? (const void*)&k_tiles_mq<FAM_LCS, uint16_t, true, 4>
                    : (const void*)&k_tiles_mq<FAM_LCS, uint16_t, false, 4>;
    case 4:
        return norm ? (const void*)&k_tiles_mq<FAM_LCS, uint32_t, true, 4>
                    : (const void*)&k_tiles_mq<FAM_LCS, uint32_t, false, 4>;
    case 8:
        return norm ? (const void*)&k_tiles_mq<FAM_LCS, unsigned long long, true, 4>
                    : (const void*)&k_tiles_mq<FAM_LCS, unsigned long long, false, 4>;
    }
    return nullptr;
}

} // namespace rfg
