/* k_band instantiations: banded unit-weight Levenshtein for one-byte choices, one kernel
 * per band width in 32-bit words (the banded LCS families: rfg_k_band_lcs.cu) */
#include "rfg_band.cuh"
#include "rfg_kernels.h"

namespace rfg {

const void* band_kernel(int width, int B, bool lcs)
{
    if (width != 1) return nullptr;
    if (lcs) return band_lcs_kernel(B);
    switch (B) {
    case 1: return (const void*)&k_band<uint8_t, 1, false>;
    case 2: return (const void*)&k_band<uint8_t, 2, false>;
    case 3: return (const void*)&k_band<uint8_t, 3, false>;
    case 4: return (const void*)&k_band<uint8_t, 4, false>;
    case 6: return (const void*)&k_band<uint8_t, 6, false>;
    case 8: return (const void*)&k_band<uint8_t, 8, false>;
    case 12: return (const void*)&k_band<uint8_t, 12, false>;
    case 16: return (const void*)&k_band<uint8_t, 16, false>;
    }
    return nullptr;
}

} // namespace rfg
