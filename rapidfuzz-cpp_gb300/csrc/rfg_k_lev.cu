/* k_tiles instantiations of the LEV core family */
#include "rfg_device.cuh"
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

const void* tiles_mq_kernel_lev(int width, bool norm)
{
    switch (width) {
    case 1:
        return norm ? (const void*)&k_tiles_mq<FAM_LEV, uint8_t, true, 2>
                    : (const void*)&k_tiles_mq<FAM_LEV, uint8_t, false, 2>;
    case 2:
        return norm ? (const void*)&k_tiles_mq<FAM_LEV, uint16_t, true, 2>
                    : (const void*)&k_tiles_mq<FAM_LEV, uint16_t, false, 2>;
    case 4:
        return norm ? (const void*)&k_tiles_mq<FAM_LEV, uint32_t, true, 2>
                    : (const void*)&k_tiles_mq<FAM_LEV, uint32_t, false, 2>;
    case 8:
        return norm ? (const void*)&k_tiles_mq<FAM_LEV, unsigned long long, true, 2>
                    : (const void*)&k_tiles_mq<FAM_LEV, unsigned long long, false, 2>;
    }
    return nullptr;
}

} // namespace rfg
