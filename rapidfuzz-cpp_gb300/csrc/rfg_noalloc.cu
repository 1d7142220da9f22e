/*
 * rfg_noalloc.cu -- all-pairs scoring for callers that cannot allocate device memory.
 *
 * Some callers of this library run where they may not call cudaMalloc or any other
 * allocator: code inside another framework's memory manager that forbids foreign
 * allocations, a process whose device memory is fully reserved by its host application,
 * or a service that must not grow its footprint after start-up.  They already hold
 * their strings and their result buffer in device memory and only need the scoring.
 * rfg_cdist_noalloc serves them: it runs the any-length scratch kernel with its scratch
 * in the statically sized array below, so a call allocates nothing -- no cudaMalloc,
 * no cudaFree, no pool or library allocation.
 *
 *  - The array is RFG_NOALLOC_SCRATCH_BYTES (32 MiB) of device memory in this library's
 *    image; every GPU that loads the library holds it until the process exits.
 *  - Host code cannot use the array's name as a device address (it is a host-side
 *    stand-in), so the device address is looked up with cudaGetSymbolAddress once per
 *    device, with that device current, on the first call made on that device.  Make
 *    that first call before any stream capture.
 *  - Every call on a device shares the array and finds the previous call's contents
 *    there; the work counter and the check flag are cleared at the start of each call.
 *    Calls that overlap on the GPU (different streams, or host threads at once) race on
 *    the array: serialise them.
 *  - Limits: query lengths up to RFG_NOALLOC_MAX_QUERY_LEN (4096) code units; larger
 *    arguments are rejected with RFG_ERR_INVALID_ARGUMENT before anything is launched.
 *    A query longer than the caller's max_query_len is found on the device: its row of
 *    `out` is left as it was, every other row is written, and the call returns
 *    RFG_ERR_INVALID_ARGUMENT -- so after that error `out` is partly written.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "rapidfuzz_gb300.h"
#include "rfg_device.cuh"

namespace rfg {
rfg_status set_last_error(rfg_status s, const char* msg);
}

using namespace rfg;

#define RFG_NOALLOC_SCRATCH_BYTES (32ull << 20)
#define RFG_NOALLOC_MAX_QUERY_LEN 4096
#define RFG_NOALLOC_HEADER_WORDS 32 /* 256 bytes: tile counter and check flag */
#define RFG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned long long rfg_noalloc_scratch[RFG_NOALLOC_SCRATCH_BYTES / 8];

namespace {

std::mutex g_setup_mu;
u64* g_scratch_addr[RFG_NOALLOC_MAX_DEVICES];

/* the any-length kernel over all queries in their own order, scratch from the array */
template <int FAM, typename CT>
__global__ void __launch_bounds__(128) k_generic_noalloc(const KParams a, int64_t max_len)
{
    const int W = a.wmax;
    u64* region = a.scratch + (int64_t)blockIdx.x * a.scratch_per_cta;
    u64* rows = region;
    u64* keys = rows + (int64_t)(256 + a.hcap + 1) * W;
    u64* st = region + (int64_t)(256 + a.hcap + 1) * W + a.hcap + (int64_t)threadIdx.x * a.scratch_per_thread;
    __shared__ int64_t s_tile;
    int64_t cur_q = -1;
    int m = 0;
    bool skip = false;
    const unsigned char* qb = nullptr;
    const int64_t ntiles = (int64_t)a.nq * a.nchunks;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(a.counter, 1);
        __syncthreads();
        const int64_t t = s_tile;
        if (t >= ntiles) break;
        const int64_t qi = t / a.nchunks;
        const int64_t ch = t % a.nchunks;
        if (qi != cur_q) {
            const int64_t q0 = a.q.off[qi];
            const int64_t len = a.q.off[qi + 1] - q0;
            qb = a.q.data + q0 * a.q.width;
            skip = len < 0 || len > max_len;
            m = skip ? 0 : (int)len;
            if (skip && threadIdx.x == 0) atomicExch(a.err, 3); /* longer than the caller's bound */
            if (FAM != FAM_WF && !skip) build_pm_rt(rows, keys, a.hcap, W, qb, m, a.q.width, a.err);
            cur_q = qi;
        }
        if (!skip) {
            const int64_t c0 = ch * a.chunk;
            const int64_t c1 = c0 + a.chunk < a.c.n ? c0 + a.chunk : a.c.n;
            for (int64_t ci = c0 + threadIdx.x; ci < c1; ci += blockDim.x)
                score_pair_generic<FAM, CT>(a, rows, keys, W, qi, m, qb, ci, st);
        }
        __syncthreads();
    }
}

template <typename CT>
const void* pick(int fam)
{
    switch (fam) {
    case FAM_LEV: return (const void*)&k_generic_noalloc<FAM_LEV, CT>;
    case FAM_LCS: return (const void*)&k_generic_noalloc<FAM_LCS, CT>;
    case FAM_OSA: return (const void*)&k_generic_noalloc<FAM_OSA, CT>;
    case FAM_JARO: return (const void*)&k_generic_noalloc<FAM_JARO, CT>;
    default: return (const void*)&k_generic_noalloc<FAM_WF, CT>;
    }
}

const void* pick_width(int fam, int width)
{
    switch (width) {
    case 1: return pick<uint8_t>(fam);
    case 2: return pick<uint16_t>(fam);
    case 4: return pick<uint32_t>(fam);
    default: return pick<unsigned long long>(fam);
    }
}

rfg_status bad(const char* msg) { return set_last_error(RFG_ERR_INVALID_ARGUMENT, msg); }

rfg_status cuda_fail(const char* what, cudaError_t e)
{
    (void)e;
    return set_last_error(RFG_ERR_CUDA, what);
}

} // namespace

extern "C" rfg_status rfg_cdist_noalloc(rfg_metric metric, rfg_op op, rfg_form form, const rfg_strings* queries,
                                        const rfg_strings* choices, int64_t max_query_len, const rfg_params* params,
                                        rfg_cutoff cutoff, rfg_dtype out_dtype, void* out, int64_t ld,
                                        void* cuda_stream)
{
    if (metric < RFG_LEVENSHTEIN || metric > RFG_RATIO) return bad("unknown metric");
    if (op < RFG_DISTANCE || op > RFG_NORMALIZED_SIMILARITY) return bad("unknown op");
    if (form < RFG_FORM_FREE || form > RFG_FORM_MULTI) return bad("unknown form");
    if (metric == RFG_RATIO && op != RFG_SIMILARITY) return bad("fuzz::ratio only has a similarity");
    if (!queries || !choices || !out) return bad("NULL argument");
    const bool int_result = !(metric == RFG_JARO || metric == RFG_JARO_WINKLER || metric == RFG_RATIO) &&
                            (op == RFG_DISTANCE || op == RFG_SIMILARITY);
    if (out_dtype < RFG_I32 || out_dtype > RFG_F64 || (!int_result && out_dtype != RFG_F64))
        return bad("output dtype does not fit the result type (doubles need RFG_F64)");
    for (const rfg_strings* s : {queries, choices}) {
        if (s->count < 0 || !s->offsets || (s->count && !s->data)) return bad("invalid string batch");
        if (s->char_width != 1 && s->char_width != 2 && s->char_width != 4 && s->char_width != 8)
            return bad("char_width must be 1, 2, 4 or 8");
    }
    if (max_query_len < 0 || max_query_len > RFG_NOALLOC_MAX_QUERY_LEN)
        return bad("max_query_len exceeds the no-allocation limit of 4096 code units");
    const int64_t nq = queries->count, nc = choices->count;
    if (ld == 0) ld = nc;
    if (ld < nc) return bad("ld must be >= the number of choices");
    ScoreParams sp;
    sp.ins = params ? params->insert_cost : 1;
    sp.del = params ? params->delete_cost : 1;
    sp.rep = params ? params->replace_cost : 1;
    sp.prefix_weight = params ? params->prefix_weight : 0.1;
    if (metric == RFG_LEVENSHTEIN && (sp.ins < 0 || sp.del < 0 || sp.rep < 0)) return bad("negative weights");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_last_error(RFG_ERR_NO_DEVICE, "no CUDA device available");
    if (dev < 0 || dev >= RFG_NOALLOC_MAX_DEVICES) return bad("device index beyond the supported range");
    u64* scratch;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, rfg_noalloc_scratch);
            if (e != cudaSuccess || !p) return cuda_fail("cudaGetSymbolAddress of the scratch array failed", e);
            g_scratch_addr[dev] = (u64*)p;
        }
        scratch = g_scratch_addr[dev];
    }
    if (nq == 0 || nc == 0) return RFG_OK;

    int fam = metric_family(metric, form, sp);
    if (fam == FAM_NONE) fam = FAM_WF;
    /* at least one word: a bound of 0 (only empty queries) still gets a table of its own
     * per block */
    const int wmax = fam == FAM_WF ? 0 : (int)std::max<int64_t>(1, (max_query_len + 63) / 64);
    int hcap = 0;
    if (fam != FAM_WF && choices->char_width > 1 && queries->char_width > 1) {
        hcap = 8;
        while (hcap < 2 * max_query_len) hcap <<= 1;
    }
    int64_t per_thread;
    switch (fam) {
    case FAM_LEV: per_thread = 2 * (int64_t)wmax; break;
    case FAM_LCS: per_thread = wmax; break;
    case FAM_OSA: per_thread = 4 * (int64_t)wmax; break;
    case FAM_JARO: per_thread = 2 * (int64_t)wmax; break;
    default: per_thread = max_query_len + 1;
    }
    const int block = 128;
    const int64_t per_cta = (wmax ? (int64_t)(256 + hcap + 1) * wmax + hcap : 0) + (int64_t)block * per_thread;
    const int64_t avail = (int64_t)(RFG_NOALLOC_SCRATCH_BYTES / 8) - RFG_NOALLOC_HEADER_WORDS;
    const int64_t fit = per_cta > 0 ? avail / per_cta : 1;
    if (fit < 1) return bad("the call needs more scratch than the 32 MiB no-allocation array holds");

    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail("cudaDeviceGetAttribute failed", e);
    const int64_t slots = (int64_t)sms * 2;
    int64_t chunk = (nc * nq + slots * 4 - 1) / (slots * 4);
    chunk = chunk < block ? block : chunk;
    chunk = chunk > nc ? nc : chunk;
    chunk = (chunk + block - 1) / block * block;
    const int64_t nchunks = (nc + chunk - 1) / chunk;
    const int64_t ntiles = nq * nchunks;
    if (ntiles > 0x7fffffffll) return bad("batch too large for one launch");
    int64_t grid = ntiles < slots ? ntiles : slots;
    if (grid > fit) grid = fit;

    KParams a;
    memset(&a, 0, sizeof a);
    a.q = KStrings{(const unsigned char*)queries->data, queries->offsets, nq, queries->char_width};
    a.c = KStrings{(const unsigned char*)choices->data, choices->offsets, nc, choices->char_width};
    a.qlist = nullptr;
    a.nq = (int32_t)nq;
    a.chunk = chunk;
    a.nchunks = nchunks;
    a.counter = (int*)scratch;
    a.err = (int*)scratch + 1;
    a.metric = metric;
    a.op = op;
    a.form = form;
    a.sp = sp;
    a.ci = cutoff.cutoff_i;
    a.cf = cutoff.cutoff_f;
    a.out = out;
    a.out_dtype = out_dtype;
    a.ld = ld;
    a.hcap = hcap;
    a.scratch = scratch + RFG_NOALLOC_HEADER_WORDS;
    a.scratch_per_cta = per_cta;
    a.scratch_per_thread = per_thread;
    a.wmax = wmax;

    cudaStream_t st = (cudaStream_t)cuda_stream;
    e = cudaMemsetAsync(scratch, 0, RFG_NOALLOC_HEADER_WORDS * 8, st);
    if (e != cudaSuccess) return cuda_fail("clearing the scratch header failed", e);
    int64_t ml = max_query_len;
    void* args[] = {&a, &ml};
    e = cudaLaunchKernel(pick_width(fam, choices->char_width), dim3((unsigned)grid), dim3(block), args, 0, st);
    if (e != cudaSuccess) return cuda_fail("kernel launch failed", e);
    int hdr[2] = {0, 0}; /* tile counter, check flag */
    e = cudaMemcpyAsync(hdr, scratch, sizeof hdr, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail("waiting for the kernel failed", e);
    if (hdr[1] == 3) return bad("a query is longer than max_query_len");
    if (hdr[1]) return set_last_error(RFG_ERR_DEVICE_CHECK, "device-side check failed");
    return RFG_OK;
}
