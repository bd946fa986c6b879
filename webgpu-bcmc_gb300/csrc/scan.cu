// scan.cu -- single-pass exclusive scan and stream compaction.
//
// Replaces ExclusiveScanner.scan (js/exclusive_scan.js:178-295), which runs a
// three-kernel Blelloch scan (prefix_sum.comp, block_prefix_sum.comp,
// add_block_sums.comp) per 512^2-element chunk with a host-side carry and a
// mapAsync readback of the total, and StreamCompact.compactActiveIDs
// (js/stream_compact.js:56-165, stream_compact.comp:26-32), one thread per
// workgroup.  Here a scan is one launch: 4096-element tiles scanned with warp
// shuffles, tiles chained by decoupled look-back.  uint32 sums wrap mod 2^32 as
// in the reference.
#include "bcmc_impl.h"

namespace bcmc {

__global__ void k_prim_begin(QueryState* q)
{
    // new epoch for the look-back status words; clear counters and the sort plan
    const int t = threadIdx.x;
    if (t == 0) {
        q->epoch += 1;
        q->tiles_active = q->tiles_slots = q->tiles_mc = q->tiles_sort_hist = 0;
        for (int i = 0; i < 4; ++i) q->tiles_sort[i] = 0;
        q->sort_arrived = 0;
        q->error = 0;
        q->num_with_verts = q->num_verts = 0;
        q->grow_needed = 0;
        q->vert_overflow = 0;
        for (int i = 0; i < 4; ++i) q->sort_run[i] = q->sort_src[i] = 0;  // the plan of zero keys
        q->sort_first = 4;
        q->sort_final = 1;
        q->sort_key16 = q->sort_wide = 0;
    }
    for (int i = t; i < 1536; i += blockDim.x) (&q->sort_hist[0][0])[i] = 0;  // and sort_hist16
}

void prim_begin(QueryState* q, cudaStream_t s)
{
    k_prim_begin<<<1, 256, 0, s>>>(q);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

// Shared-memory index with one pad word per 32, so that both the striped
// (coalesced) and the per-thread-consecutive views are free of bank conflicts.
__device__ __forceinline__ uint32_t spad(uint32_t i) { return i + (i >> 5); }
constexpr int kScanSmem = kScanTile + kScanTile / 32;

// Loads a tile striped (coalesced) into shared memory, then each thread owns
// kScanItems consecutive elements.
template <typename Op>
__device__ __forceinline__ void tile_scan(const uint32_t* __restrict__ in, uint32_t n, uint32_t tile,
                                          uint32_t* s_buf, uint32_t* s_warp, Op per_item_value,
                                          uint32_t vals[kScanItems], uint32_t* thread_excl,
                                          uint32_t* tile_total)
{
    const uint32_t base = tile * kScanTile;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        const uint32_t i = base + j * kScanThreads + threadIdx.x;
        s_buf[spad(j * kScanThreads + threadIdx.x)] = i < n ? in[i] : 0u;
    }
    __syncthreads();
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        const uint32_t v = per_item_value(s_buf[spad(threadIdx.x * kScanItems + j)]);
        vals[j] = v;
        sum += v;
    }
    __syncthreads();
    *thread_excl = cta_exclusive_scan<kScanThreads>(sum, s_warp, tile_total);
}

__global__ void __launch_bounds__(kScanThreads) k_scan(QueryState* q, const uint32_t* __restrict__ in,
                                                       uint32_t* out, uint32_t n, uint32_t* d_total,
                                                       uint64_t* status)
{
    __shared__ uint32_t s_buf[kScanSmem];
    __shared__ uint32_t s_warp[kScanThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_prefix;
    const uint32_t ntiles = div_up(n, kScanTile);
    const uint32_t epoch = q->epoch;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&q->tiles_active, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        uint32_t vals[kScanItems], excl, total;
        tile_scan(in, n, tile, s_buf, s_warp, [](uint32_t v) { return v; }, vals, &excl, &total);
        if (threadIdx.x < 32) {
            const uint32_t p = lb_dropped(q, tile) ? 0u : warp_lookback(status, tile, total, epoch, &q->error, 1u);
            if (threadIdx.x == 0) {
                s_prefix = p;
                if (tile == ntiles - 1 && d_total) *d_total = p + total;
            }
        }
        __syncthreads();
        uint32_t run = s_prefix + excl;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            s_buf[spad(threadIdx.x * kScanItems + j)] = run;
            run += vals[j];
        }
        __syncthreads();
        const uint32_t base = tile * kScanTile;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            const uint32_t i = base + j * kScanThreads + threadIdx.x;
            if (i < n) out[i] = s_buf[spad(j * kScanThreads + threadIdx.x)];
        }
        __syncthreads();
    }
}

// Fused scan + compaction: out[k] = index of the k-th nonzero flag.
__global__ void __launch_bounds__(kScanThreads) k_select(QueryState* q, const uint32_t* __restrict__ flags,
                                                         uint32_t* out, uint32_t n, uint32_t* d_count,
                                                         uint64_t* status)
{
    __shared__ uint32_t s_buf[kScanSmem];
    __shared__ uint32_t s_warp[kScanThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_prefix;
    const uint32_t ntiles = div_up(n, kScanTile);
    const uint32_t epoch = q->epoch;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&q->tiles_active, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        uint32_t vals[kScanItems], excl, total;
        tile_scan(flags, n, tile, s_buf, s_warp, [](uint32_t v) { return v != 0u ? 1u : 0u; }, vals, &excl,
                  &total);
        if (threadIdx.x < 32) {
            const uint32_t p = lb_dropped(q, tile) ? 0u : warp_lookback(status, tile, total, epoch, &q->error, 2u);
            if (threadIdx.x == 0) {
                s_prefix = p;
                if (tile == ntiles - 1 && d_count) *d_count = p + total;
            }
        }
        __syncthreads();
        uint32_t pos = s_prefix + excl;
        const uint32_t first = tile * kScanTile + threadIdx.x * kScanItems;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j)
            if (vals[j]) {
                if (pos < n) out[pos] = first + j;  // pos < n unless a look-back wait timed out
                ++pos;
            }
        __syncthreads();
    }
}

__global__ void k_compact(uint32_t n, const uint32_t* __restrict__ flags, const uint32_t* __restrict__ offsets,
                          uint32_t* out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flags[i] != 0u) out[offsets[i]] = i;
}

static int persistent_grid(bcmc_ctx* ctx, uint32_t tiles, uint32_t per_sm)
{
    const uint32_t r = (uint32_t)ctx->num_sms * per_sm;
    return (int)(tiles < r ? (tiles ? tiles : 1) : r);
}

void scan_launch(bcmc_ctx* ctx, QueryState* q, const uint32_t* in, uint32_t* out, uint32_t n,
                 uint32_t* d_total, uint64_t* status, cudaStream_t s)
{
    k_scan<<<persistent_grid(ctx, div_up(n, kScanTile), 4), kScanThreads, 0, s>>>(q, in, out, n, d_total, status);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

cudaError_t scan_launch_sms(int num_sms, QueryState* q, const uint32_t* in, uint32_t* out, uint32_t n,
                            uint32_t* d_total, uint64_t* status, cudaStream_t s)
{
    const uint32_t tiles = div_up(n, kScanTile), r = (uint32_t)num_sms * 4u;
    const int grid = (int)(tiles < r ? (tiles ? tiles : 1) : r);
    k_scan<<<grid, kScanThreads, 0, s>>>(q, in, out, n, d_total, status);
    count_launches(1);
    return cudaGetLastError();
}

void select_launch(bcmc_ctx* ctx, QueryState* q, const uint32_t* flags, uint32_t* out, uint32_t n,
                   uint32_t* d_count, uint64_t* status, cudaStream_t s)
{
    k_select<<<persistent_grid(ctx, div_up(n, kScanTile), 4), kScanThreads, 0, s>>>(q, flags, out, n, d_count,
                                                                                     status);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void compact_launch(bcmc_ctx* ctx, uint32_t n, const uint32_t* flags, const uint32_t* offsets, uint32_t* out,
                    cudaStream_t s)
{
    if (n == 0) return;
    const int grid = (int)min(div_up(n, 256u), (uint32_t)ctx->num_sms * 16u);
    k_compact<<<grid, 256, 0, s>>>(n, flags, offsets, out);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

}  // namespace bcmc
