/* k_band instantiations of the banded LCS families (Indel, LCSseq, ratio) for one-byte
 * choices, one kernel per band width in 32-bit words */
#include "rfg_band.cuh"
#include "rfg_kernels.h"

namespace rfg {

const void* band_lcs_kernel(int B)
{
    switch (B) {
    case 1: return (const void*)&k_band<uint8_t, 1, true>;
    case 2: return (const void*)&k_band<uint8_t, 2, true>;
    case 3: return (const void*)&k_band<uint8_t, 3, true>;
    case 4: return (const void*)&k_band<uint8_t, 4, true>;
    case 6: return (const void*)&k_band<uint8_t, 6, true>;
    case 8: return (const void*)&k_band<uint8_t, 8, true>;
    case 12: return (const void*)&k_band<uint8_t, 12, true>;
    case 16: return (const void*)&k_band<uint8_t, 16, true>;
    }
    return nullptr;
}

} // namespace rfg
