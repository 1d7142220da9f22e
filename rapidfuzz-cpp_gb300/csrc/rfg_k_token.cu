/* k_generic instantiations of the token_set_ratio family (dense results only) */
#include "rfg_device.cuh"
#include "rfg_kernels.h"

namespace rfg {

const void* token_kernel(int width)
{
    switch (width) {
    case 1: return (const void*)&k_generic<FAM_TOKEN, uint8_t, false>;
    case 2: return (const void*)&k_generic<FAM_TOKEN, uint16_t, false>;
    case 4: return (const void*)&k_generic<FAM_TOKEN, uint32_t, false>;
    case 8: return (const void*)&k_generic<FAM_TOKEN, unsigned long long, false>;
    }
    return nullptr;
}

} // namespace rfg
