// scan_noalloc.cu -- exclusive scan that allocates nothing.
//
// Same result as bcmc_scan_exclusive_u32_async (the single-pass look-back scan
// of scan.cu), for callers that must not allocate device memory on the call:
// a host runtime that owns every device byte through its own pool and forbids
// cudaMalloc/cudaFree outside it, code running between a stream's enqueue and
// its synchronisation where an allocation's implicit device synchronisation
// would stall other streams, and callers that hold no bcmc_ctx (creating one
// allocates).  Its only device scratch is the file-scope array below, a fixed
// 137,480 bytes (about 134 KiB) per device, so the input size is capped at
// BCMC_SCAN_NOALLOC_MAX_N (2^26 elements = 16,384 tiles).
//
// Scratch layout (one array per device, in this module's static memory):
//   words [0, kQueryWords)          QueryState: look-back epoch, tile counter,
//                                   wait-timeout error word
//   words [kQueryWords, +kStatus)   one look-back status word per 4096-element
//                                   tile, plus one
// Every call first runs k_noalloc_begin, which zeroes the tile counter, the
// error word and the status words the call will use, and sets epoch 1; so no
// state carries from one call to the next and nothing relies on the array's
// zero initialisation at module load.
//
// The array's device address is looked up with cudaGetSymbolAddress, in the
// CUDA context current on the calling thread, the first time a call runs in
// that context, and cached under the context's unique id (cuCtxGetId): a
// device reset, or a host runtime that makes its own context current, gets a
// fresh look-up instead of an address from another context.
//
// Calls on one device share that scratch: two calls whose kernels can overlap
// (different streams without an ordering between them, or different host
// threads) race on it and both results are undefined.  Order them on one
// stream, or with events.
//
// A look-back wait that runs out of spins (it cannot hang the GPU) marks the
// error word in the shared scratch, which no caller can read, and the prefixes
// after it are wrong: this entry point does not report wait timeouts.  The
// context-based scans report them as BCMC_E_TIMEOUT.
#include <cuda.h>

#include <mutex>

#include "bcmc_impl.h"

namespace bcmc {
namespace {

constexpr uint32_t kMaxN = BCMC_SCAN_NOALLOC_MAX_N;
constexpr uint32_t kMaxTiles = (kMaxN + kScanTile - 1) / kScanTile;
constexpr uint32_t kStatusWords = kMaxTiles + 1;
constexpr uint32_t kQueryWords = (uint32_t)((sizeof(QueryState) + 255) / 256 * 256 / 8);
constexpr uint32_t kScratchWords = kQueryWords + kStatusWords;
static_assert(kQueryWords * 8 >= sizeof(QueryState), "QueryState does not fit its scratch words");
// The scratch: 16,385 status words after the QueryState block (6,400 bytes),
// 137,480 bytes on each device the library runs on.
static_assert(kScratchWords * 8 == 137480u, "the scratch size stated in this file and in bcmc.h changed");
static __device__ __align__(256) uint64_t g_scan_scratch[kScratchWords];

// Set-up cache: one entry per CUDA context seen (by its process-unique id).
constexpr int kMaxContexts = 64;
struct ContextScratch {
    unsigned long long ctx_id;  // 0: unused
    int num_sms;
    uint64_t* words;  // device address of g_scan_scratch in that context
};
ContextScratch g_contexts[kMaxContexts];
int g_next_evict = 0;
std::mutex g_setup_mutex;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

__global__ void k_noalloc_begin(QueryState* q, uint64_t* status, uint32_t status_words)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        q->epoch = 1;
        q->tiles_active = 0;
        q->error = 0;
        q->debug_drop_tile = 0;
    }
    if (i < status_words) status[i] = 0;
}

// The unique id of the CUDA context current on this thread.  When no context
// is current, the device's primary context is made current first (what any
// runtime call would do); a context the caller made current is kept.
bcmc_status current_context_id(int dev, unsigned long long* id)
{
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q2 != cudaDriverEntryPointSuccess)
            return BCMC_E_CUDA;
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext c = nullptr;
    if (g_ctx_get_current(&c) != CUDA_SUCCESS) return BCMC_E_CUDA;
    if (!c) {
        if (cudaSetDevice(dev) != cudaSuccess || g_ctx_get_current(&c) != CUDA_SUCCESS || !c) return BCMC_E_CUDA;
    }
    return g_ctx_get_id(c, id) == CUDA_SUCCESS && *id ? BCMC_OK : BCMC_E_CUDA;
}

// Set-up for the current context, once per context: the device address of the
// scratch array (this also loads the module into that context, when the driver
// loads modules lazily) and the SM count that sizes the grid.
bcmc_status setup_current_context(ContextScratch* out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return BCMC_E_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return BCMC_E_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = 0;
    const bcmc_status st = current_context_id(dev, &id);
    if (st != BCMC_OK) return st;
    for (const ContextScratch& c : g_contexts) {
        if (c.ctx_id == id) {
            *out = c;
            return BCMC_OK;
        }
    }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scan_scratch) != cudaSuccess || !p) return BCMC_E_CUDA;
    ContextScratch& c = g_contexts[g_next_evict];
    g_next_evict = (g_next_evict + 1) % kMaxContexts;
    c.ctx_id = id;
    c.num_sms = sms;
    c.words = static_cast<uint64_t*>(p);
    *out = c;
    return BCMC_OK;
}

}  // namespace
}  // namespace bcmc

using namespace bcmc;

extern "C" bcmc_status bcmc_scan_exclusive_u32_noalloc(const uint32_t* d_in, uint32_t* d_out, uint32_t n,
                                                       uint32_t* d_total, void* stream)
{
    if (n > kMaxN) return BCMC_E_LIMIT;  // checked before anything touches the device
    if (n && (!d_in || !d_out)) return BCMC_E_ARG;
    ContextScratch d;
    const bcmc_status st = setup_current_context(&d);
    if (st != BCMC_OK) return st;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        if (d_total && cudaMemsetAsync(d_total, 0, 4, s) != cudaSuccess) return BCMC_E_CUDA;
        return BCMC_OK;
    }
    QueryState* q = reinterpret_cast<QueryState*>(d.words);
    uint64_t* status = d.words + kQueryWords;
    const uint32_t words = div_up(n, (uint32_t)kScanTile) + 1;
    k_noalloc_begin<<<div_up(words, 256u), 256, 0, s>>>(q, status, words);
    count_launches(1);
    if (cudaGetLastError() != cudaSuccess) return BCMC_E_CUDA;
    if (scan_launch_sms(d.num_sms, q, d_in, d_out, n, d_total, status, s) != cudaSuccess) return BCMC_E_CUDA;
    return BCMC_OK;
}
