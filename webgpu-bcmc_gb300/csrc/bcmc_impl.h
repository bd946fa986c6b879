// bcmc_impl.h -- host-side declarations shared by the translation units of
// libbcmc_gb300 (launchers and object layouts).  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "bcmc_internal.cuh"

struct bcmc_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    bcmc_opts opts{};
    std::string last_error;
    // state of standalone primitive calls (epoch, tile counters, error word)
    bcmc::QueryState* d_prim = nullptr;
    uint64_t* d_status = nullptr;  // look-back status words for primitives
    size_t status_words = 0;
    uint32_t* d_scratch = nullptr;  // sort ping-pong buffers for primitives
    size_t scratch_words = 0;
    uint32_t* h_pinned = nullptr;   // small pinned host staging
    void* d_render = nullptr;       // render pass working buffers (grow-only)
    size_t render_bytes = 0;
    uint64_t device_bytes = 0;
    // volumes and caches made from this context; bcmc_ctx_destroy defers the
    // release until the last of them is destroyed
    uint32_t children = 0;
    bool destroy_pending = false;
    // test hook (bcmc_debug_drop_tile): 0, or the dropped tile + 1
    uint32_t debug_drop_tile = 0;
};

namespace bcmc {

// Kernels this library has launched (all contexts); reported by
// bcmc_kernel_launches() so callers can account for their GPU work.
extern std::atomic<uint64_t> g_kernel_launches;
inline void count_launches(uint64_t n) { g_kernel_launches.fetch_add(n, std::memory_order_relaxed); }

// Dynamic shared memory above the 48 KB a launch gets without opting in.
template <typename K>
inline void allow_smem(K kernel, size_t bytes)
{
    if (bytes > 48u * 1024u) BCMC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

// Objects made from a context (volumes, caches, engines) keep it alive:
// bcmc_ctx_destroy defers the release until the last of them is gone.
void ctx_child_added(bcmc_ctx* ctx);
void ctx_child_removed(bcmc_ctx* ctx);
// Growable device allocation helpers (cudaMalloc; throw CudaError).
void* dev_alloc(bcmc_ctx* ctx, size_t bytes);
void dev_free(bcmc_ctx* ctx, void* p, size_t bytes);
void ensure_status(bcmc_ctx* ctx, size_t words);
void ensure_scratch(bcmc_ctx* ctx, size_t words);

// ---- unpack.cu ----------------------------------------------------------------
void unpack_launch(bcmc_ctx* ctx, const uint2* verts, uint64_t n, const uint32_t dims[3], const float scale[3],
                   const float* proj_view, float* world, float* clip, cudaStream_t s);
void render_launch(bcmc_ctx* ctx, const uint2* verts, uint64_t n, const uint32_t dims[3], const float scale[3],
                   const bcmc_render_params& p, float* rgba, float* depth, uint32_t* triangle, cudaStream_t s);

// ---- engine.cu (for server.cu) ------------------------------------------------
int engine_device(bcmc_engine* e);
// Pipelined batches, for the server: two lanes of batch buffers, so that one
// batch's phase 1 (active test, claims, decode) runs while the other's phase 2
// (marching cubes) does.  engine_submit launches queries[0..n) on lane k and
// returns at once (on_done(arg) runs on a CUDA host thread when the batch's
// results are on the host); engine_complete takes the results (blocking until
// they are there), in submission order; engine_copy_lane_vertices copies from
// that lane's vertex buffer, valid until the lane's next submit.
bcmc_status engine_submit(bcmc_engine* e, int k, const bcmc_query* queries, uint32_t n, void (*on_done)(void*),
                          void* arg);
bcmc_status engine_complete(bcmc_engine* e, int k, bcmc_query_result* out, uint32_t* admitted);
bcmc_status engine_copy_lane_vertices(bcmc_engine* e, int k, uint64_t first, uint64_t count, void* host);
// Waits for everything the engine queued, host callbacks included.
void engine_drain(bcmc_engine* e);
uint32_t engine_max_batch(bcmc_engine* e);
uint32_t engine_num_volumes(bcmc_engine* e);
uint64_t engine_vertex_budget(bcmc_engine* e);
bcmc_ctx* engine_ctx(bcmc_engine* e);

// ---- sort.cu ----------------------------------------------------------------
constexpr int kSortThreads = 512;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys per tile
// Plan + onesweep passes over n (device-resident) pairs.  Input arrays are in
// natural order; the first pass applies the reference's tie-order permutation
// and the key transform (~key when descending).  Result lands in buffer
// q->sort_final (1 = b, 2 = c) as transformed keys + values.
struct SortBuffers {
    const uint32_t* in_keys;
    const uint32_t* in_vals;
    uint32_t* b_keys;
    uint32_t* b_vals;
    uint32_t* c_keys;
    uint32_t* c_vals;
    uint64_t* status;  // kSortTileStatus words per tile (256 per tile)
    // the LRU's age sort: dense rank of each age bin (age_bin; sort_key16 == 2)
    const uint8_t* age_rank = nullptr;
};
// plan_ready: the keys' producer already made the pass plan and bucket
// offsets in q (sort_plan), so the histogram kernel is not launched.
void sort_launch(bcmc_ctx* ctx, QueryState* q, const uint32_t* d_n, uint32_t n_max,
                 const SortBuffers& bufs, int reverse, cudaStream_t s, int plan_ready = 0);
// Copies the sorted pairs back to (keys, values) with the inverse key transform.
void sort_writeback(bcmc_ctx* ctx, QueryState* q, const uint32_t* d_n, uint32_t n_max,
                    const SortBuffers& bufs, uint32_t* keys, uint32_t* vals, int reverse,
                    cudaStream_t s);
size_t sort_status_words(uint32_t n_max);
int sort_grid(bcmc_ctx* ctx, uint32_t n_max);

// ---- scan.cu ----------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
void scan_launch(bcmc_ctx* ctx, QueryState* q, const uint32_t* in, uint32_t* out, uint32_t n,
                 uint32_t* d_total, uint64_t* status, cudaStream_t s);
// Same kernel as scan_launch, sized from an SM count instead of a context;
// reports a launch error by return value (throws nothing).
cudaError_t scan_launch_sms(int num_sms, QueryState* q, const uint32_t* in, uint32_t* out, uint32_t n,
                            uint32_t* d_total, uint64_t* status, cudaStream_t s);
void select_launch(bcmc_ctx* ctx, QueryState* q, const uint32_t* flags, uint32_t* out, uint32_t n,
                   uint32_t* d_count, uint64_t* status, cudaStream_t s);
void compact_launch(bcmc_ctx* ctx, uint32_t n, const uint32_t* flags, const uint32_t* offsets,
                    uint32_t* out, cudaStream_t s);
// Bumps q->epoch, clears tile counters and counts: begins a device-driven call.
void prim_begin(QueryState* q, cudaStream_t s);

// ---- zfp.cu -----------------------------------------------------------------
void zfp_ranges_launch(bcmc_ctx* ctx, const uint64_t* words, const uint32_t dims[3],
                       uint32_t max_bits, float* ranges, cudaStream_t s);
void zfp_decode_blocks_launch(bcmc_ctx* ctx, const uint64_t* words, uint32_t max_bits,
                              const uint32_t* ids, uint32_t n, const int32_t* item_slots,
                              float* cache, cudaStream_t s);
void zfp_decode_volume_launch(bcmc_ctx* ctx, const uint64_t* words, uint64_t nblocks,
                              uint32_t max_bits, float* out, cudaStream_t s);
void zfp_encode_launch(bcmc_ctx* ctx, const float* field, const uint32_t dims[3],
                       uint32_t max_bits, uint64_t* words, cudaStream_t s);

}  // namespace bcmc
