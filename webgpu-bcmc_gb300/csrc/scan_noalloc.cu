// scan_noalloc.cu -- exclusive scan that allocates nothing.
//
// Same result as bcmc_scan_exclusive_u32_async (the single-pass look-back scan
// of scan.cu), for callers that must not allocate device memory on the call:
// a host runtime that owns every device byte through its own pool and forbids
// cudaMalloc/cudaFree outside it, code running between a stream's enqueue and
// its synchronisation where an allocation's implicit device synchronisation
// would stall other streams, and callers that hold no bcmc_ctx (creating one
// allocates).  Its only device scratch is the file-scope array below, a fixed
// ~132 KB per device, so the input size is capped at BCMC_SCAN_NOALLOC_MAX_N
// (2^26 elements = 16,384 tiles).
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
// Calls on one device share that scratch: two calls whose kernels can overlap
// (different streams without an ordering between them, or different host
// threads) race on it and both results are undefined.  Order them on one
// stream, or with events.
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
static_assert(kScratchWords * 8 <= 160u * 1024u, "scratch above its stated size");

// The scratch: 16,385 status words after the QueryState block (4,352 bytes),
// 135,432 bytes on each device the library runs on.
static __device__ __align__(256) uint64_t g_scan_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
struct DeviceScratch {
    bool ready;
    int num_sms;
    uint64_t* words;  // device address of g_scan_scratch on this device
};
DeviceScratch g_devices[kMaxDevices];
std::mutex g_setup_mutex;

__global__ void k_noalloc_begin(QueryState* q, uint64_t* status, uint32_t status_words)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        q->epoch = 1;
        q->tiles_active = 0;
        q->error = 0;
    }
    if (i < status_words) status[i] = 0;
}

// Set-up for the current device, once: the device address of the scratch
// array (this also loads the module on that device, when the driver loads
// modules lazily) and the SM count that sizes the grid.
bcmc_status setup_current_device(DeviceScratch** out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BCMC_E_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceScratch& d = g_devices[dev];
    if (!d.ready) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scan_scratch) != cudaSuccess || !p) return BCMC_E_CUDA;
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            return BCMC_E_CUDA;
        d.words = static_cast<uint64_t*>(p);
        d.num_sms = sms;
        d.ready = true;
    }
    *out = &d;
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
    DeviceScratch* d = nullptr;
    const bcmc_status st = setup_current_device(&d);
    if (st != BCMC_OK) return st;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        if (d_total && cudaMemsetAsync(d_total, 0, 4, s) != cudaSuccess) return BCMC_E_CUDA;
        return BCMC_OK;
    }
    QueryState* q = reinterpret_cast<QueryState*>(d->words);
    uint64_t* status = d->words + kQueryWords;
    const uint32_t words = div_up(n, (uint32_t)kScanTile) + 1;
    k_noalloc_begin<<<div_up(words, 256u), 256, 0, s>>>(q, status, words);
    count_launches(1);
    if (cudaGetLastError() != cudaSuccess) return BCMC_E_CUDA;
    if (scan_launch_sms(d->num_sms, q, d_in, d_out, n, d_total, status, s) != cudaSuccess) return BCMC_E_CUDA;
    return BCMC_OK;
}
