/* k_band instantiations: banded unit-weight Levenshtein for one-byte choices, one kernel
 * per band width in 32-bit words */
#include "rfg_band.cuh"
#include "rfg_kernels.h"

namespace rfg {

const void* band_kernel(int width, int B)
{
    if (width != 1) return nullptr;
    switch (B) {
    case 1: return (const void*)&k_band<uint8_t, 1>;
    case 2: return (const void*)&k_band<uint8_t, 2>;
    case 3: return (const void*)&k_band<uint8_t, 3>;
    case 4: return (const void*)&k_band<uint8_t, 4>;
    case 6: return (const void*)&k_band<uint8_t, 6>;
    case 8: return (const void*)&k_band<uint8_t, 8>;
    case 12: return (const void*)&k_band<uint8_t, 12>;
    case 16: return (const void*)&k_band<uint8_t, 16>;
    }
    return nullptr;
}

} // namespace rfg
