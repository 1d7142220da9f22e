/* k_tiles instantiations of the LEV core family */
#include "rfg_device.cuh"
#include "rfg_kernels.h"

namespace rfg {

template <typename CT>
static const void* pick_lev(int W)
{
    switch (W) {
    case 1: return (const void*)&k_tiles<FAM_LEV, CT, 1>;
    case 2: return (const void*)&k_tiles<FAM_LEV, CT, 2>;
    case 4: return (const void*)&k_tiles<FAM_LEV, CT, 4>;
    case 8: return (const void*)&k_tiles<FAM_LEV, CT, 8>;
    }
    return nullptr;
}

const void* tiles_kernel_lev(int width, int W)
{
    switch (width) {
    case 1: return pick_lev<uint8_t>(W);
    case 2: return pick_lev<uint16_t>(W);
    case 4: return pick_lev<uint32_t>(W);
    case 8: return pick_lev<unsigned long long>(W);
    }
    return nullptr;
}

} // namespace rfg
