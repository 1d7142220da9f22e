/* k_tiles instantiations of the OSA core family */
#include "rfg_device.cuh"
#include "rfg_kernels.h"

namespace rfg {

template <typename CT>
static const void* pick_osa(int W)
{
    switch (W) {
    case 1: return (const void*)&k_tiles<FAM_OSA, CT, 1>;
    case 2: return (const void*)&k_tiles<FAM_OSA, CT, 2>;
    case 4: return (const void*)&k_tiles<FAM_OSA, CT, 4>;
    case 8: return (const void*)&k_tiles<FAM_OSA, CT, 8>;
    }
    return nullptr;
}

const void* tiles_kernel_osa(int width, int W)
{
    switch (width) {
    case 1: return pick_osa<uint8_t>(W);
    case 2: return pick_osa<uint16_t>(W);
    case 4: return pick_osa<uint32_t>(W);
    case 8: return pick_osa<unsigned long long>(W);
    }
    return nullptr;
}

} // namespace rfg
