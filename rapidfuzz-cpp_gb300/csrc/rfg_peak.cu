/*
 * rfg_peak.cu -- INT32 issue-rate microbenchmark used as the roofline denominator of
 * the scorer kernels (measurement helper, built as its own library, not part of the
 * scorer ABI).  Each thread runs independent chains of 32-bit LOP3 (three-input
 * logic), IADD3 and funnel shifts -- the instruction mix of a bit-parallel cell
 * update -- so the measured rate is what the integer pipes sustain on this GPU.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#define CHAINS 8

__global__ void __launch_bounds__(256) k_int_peak(uint32_t* out, int iters, uint32_t seed)
{
    uint32_t a[CHAINS], b[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) {
        a[c] = seed * (threadIdx.x + 1) + c * 0x9E3779B9u;
        b[c] = a[c] ^ 0x7F4A7C15u;
    }
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) {
            uint32_t x = a[c], y = b[c];
            x = (x & y) ^ (~x | (y >> 3));             /* lop3-style logic */
            y = y + x + 0x1234567u;                    /* iadd3 */
            x = __funnelshift_l(x, y, 1);              /* shf */
            y = (y ^ x) | (x & 0x0F0F0F0Fu);           /* lop3 */
            x = x + y + c;                             /* iadd3 */
            y = __funnelshift_r(y, x, 1);              /* shf */
            a[c] = (x | y) ^ (x >> 5);                 /* lop3 + shift */
            b[c] = y;
        }
    }
    uint32_t r = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) r ^= a[c] + b[c];
    if (r == 0x12345678u) out[blockIdx.x] = r; /* keeps the chains live */
}

extern "C" int rfg_peak_int_ops(int iters, double* ops_per_s, double* ms)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint32_t* out = nullptr;
    if (cudaMalloc(&out, 4096 * sizeof(uint32_t)) != cudaSuccess) return 2;
    const int blocks = sms * 8, threads = 256;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_int_peak<<<blocks, threads>>>(out, iters / 10 + 1, 1u); /* warm-up */
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0);
        k_int_peak<<<blocks, threads>>>(out, iters, 3u + r);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        if (t < best) best = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return 3;
    /* per chain and iteration at least 9 integer instructions: 3 three-input logic
     * (LOP3), 2 three-input adds (IADD3), 2 funnel shifts and 2 plain shifts */
    const double ops = (double)blocks * threads * (double)iters * CHAINS * 9.0;
    *ops_per_s = ops / (best * 1e-3);
    *ms = best;
    return 0;
}
