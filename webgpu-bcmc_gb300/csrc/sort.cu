// sort.cu -- onesweep LSD radix sort of (uint32 key, uint32 value) pairs.
//
// Replaces RadixSorter.sort (js/radix_sort_by_key.js:161-400): the reference
// sorts 64-element chunks with 32 one-bit splits (radix_sort_chunk.comp), merges
// them pairwise log2(chunks) times (merge_sorted_chunks.comp, where elements of
// the right half come first among equal keys, :82-86) and, for a descending
// sort, reverses the result (reverse_buffer.comp).  That fixes the order among
// equal keys:
//   ascending : key asc,  then chunk (index/64) desc, then index asc
//   descending: key desc, then chunk asc,             then index desc
// Here one stable LSD radix sort reproduces it: the first pass reads the input
// through a permutation that lists the elements in that tie order, and sorts
// ~key for a descending sort.
//
// Kernels: a histogram/plan kernel (all four 8-bit digit histograms in one
// read, exclusive bucket offsets, and which digit passes can be skipped because
// every key shares the digit), then one cooperative kernel that runs the onesweep
// pass of each digit the plan keeps, grid barriers between them: tiles of 4096
// keys are ranked with warp match/popc, each tile publishes its 256 digit
// counts through decoupled look-back, and keys are scattered via shared memory
// so that global writes come out in runs.
//
// The LRU's age sort skips the histogram kernel: k_slots, which compacts the
// ages, accumulates the histograms and makes the plan (sort_plan).  When every
// age has a 16-bit key (age_key16) the plan sorts on that key (sort_key16 1),
// so the first pass maps each age through it and two digit passes suffice;
// when every age lies in an age bin (age_bin) and at most 256 bins are used,
// on the bins' dense ranks (sort_key16 2, older ages ranked first, from a
// table k_slots builds): one pass.
#include "bcmc_impl.h"

namespace bcmc {

// Sequence position q -> input index p giving the reference's tie order.
__device__ __forceinline__ uint32_t tie_perm(uint32_t q, uint32_t n, int reverse)
{
    const uint32_t chunks = (n + 63u) >> 6;
    const uint32_t last_len = n - 64u * (chunks - 1u);
    if (reverse) {
        const uint32_t c = q >> 6, r = q & 63u;
        const uint32_t len = (c == chunks - 1u) ? last_len : 64u;
        return 64u * c + (len - 1u - r);
    }
    if (q < last_len) return 64u * (chunks - 1u) + q;
    const uint32_t qq = q - last_len;
    return 64u * (chunks - 2u - (qq >> 6)) + (qq & 63u);
}

__global__ void __launch_bounds__(256) k_sort_hist(QueryState* q, const uint32_t* d_n, uint32_t n_host,
                                                   const uint32_t* __restrict__ keys, int reverse)
{
    __shared__ uint32_t h[4 * 256];
    __shared__ uint32_t warp_sums[9];
    __shared__ bool is_last;
    const uint32_t n = d_n ? *d_n : n_host;
    for (int i = threadIdx.x; i < 1024; i += 256) h[i] = 0;
    __syncthreads();
    // one shared atomic per distinct digit and warp: keys such as cache-slot
    // ages take few distinct values, and per-key atomics on them serialise
    for (uint32_t i0 = blockIdx.x * 256u; i0 < n; i0 += gridDim.x * 256u) {
        const uint32_t i = i0 + threadIdx.x;
        const bool valid = i < n;
        uint32_t k = valid ? keys[i] : 0u;
        if (reverse) k = ~k;
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            const uint32_t digit = valid ? (k >> (8 * d)) & 255u : 256u;
            const uint32_t peers = __match_any_sync(0xffffffffu, digit);
            if (valid && (threadIdx.x & 31u) == (uint32_t)__ffs(peers) - 1u)
                atomicAdd(&h[256 * d + digit], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    uint32_t* gh = &q->sort_hist[0][0];
    for (int i = threadIdx.x; i < 1024; i += 256)
        if (h[i]) atomicAdd(gh + i, h[i]);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(&q->tiles_sort_hist, 1u) == gridDim.x - 1u;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    sort_plan(q, n, warp_sums, &q->sort_hist[0][0], 4);
}

// All the digit passes of the plan in one cooperative launch: the passes
// that run are separated by grid barriers (each reads what the one before it
// scattered, so its key and value loads bypass L1), the others cost nothing.
__global__ void __launch_bounds__(kSortThreads, 2) k_sort(QueryState* q, const uint32_t* d_n, uint32_t n_host,
                                                       SortBuffers b, int reverse)
{
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];
    __shared__ uint16_t s_whist[kSortThreads / 32][256];  // per warp and digit: < 2^16
    __shared__ uint32_t s_start[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_warp_sums[kSortThreads / 32 + 1];
    __shared__ uint32_t s_tile;

    const uint32_t n = d_n ? *d_n : n_host;
    uint32_t barriers = 0;  // thread 0's count of grid barriers passed
    bool ran = false;
    for (int pass = 0; pass < 4; ++pass) {
        if (!q->sort_run[pass]) continue;
        if (ran) {
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                ++barriers;
                atomicAdd(&q->sort_arrived, 1u);
                uint32_t spins = 0;
                while (*reinterpret_cast<volatile uint32_t*>(&q->sort_arrived) < barriers * gridDim.x) {
                    if (++spins > kSpinLimit) {
                        atomicCAS(&q->error, 0u, 28u);
                        break;
                    }
                    if (spins > 8) __nanosleep(100);
                }
                __threadfence();
            }
            __syncthreads();
        }
        ran = true;
        const uint32_t src = q->sort_src[pass];
        const uint32_t* __restrict__ ks = src == 0 ? b.in_keys : (src == 1 ? b.b_keys : b.c_keys);
        const uint32_t* __restrict__ vs = src == 0 ? b.in_vals : (src == 1 ? b.b_vals : b.c_vals);
        uint32_t* __restrict__ kd = src == 1 ? b.c_keys : b.b_keys;
        uint32_t* __restrict__ vd = src == 1 ? b.c_vals : b.b_vals;
        const bool gather = src == 0;
        const uint32_t kmode = q->sort_key16;  // 0: the keys, 1: 16-bit age keys, 2: their dense ranks
        const uint32_t shift = 8u * (uint32_t)pass;
        const uint32_t epoch = q->epoch * 4u + (uint32_t)pass;
        const uint32_t ntiles = div_up(n, kSortTile);
        const uint32_t* bucket = q->sort_hist[pass];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const uint32_t lt_mask = (1u << lane) - 1u;

        for (;;) {
            if (threadIdx.x == 0) s_tile = atomicAdd(&q->tiles_sort[pass], 1u);
            for (int i = threadIdx.x; i < (kSortThreads / 32) * 256; i += kSortThreads) (&s_whist[0][0])[i] = 0;
            __syncthreads();
            const uint32_t tile = s_tile;
            if (tile >= ntiles) break;

            uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
            const uint32_t base = tile * kSortTile + (uint32_t)warp * (32u * kSortItems);
#pragma unroll
            for (int j = 0; j < kSortItems; ++j) {
                const uint32_t qi = base + 32u * j + lane;
                key[j] = 0;
                val[j] = 0;
                if (qi < n) {
                    const uint32_t p = gather ? tie_perm(qi, n, reverse) : qi;
                    uint32_t k = __ldcg(ks + p);
                    if (gather && kmode == 1u) k = age_key16(k);
                    if (gather && kmode == 2u) {
                        k = b.age_rank[age_bin(k)];  // ascending rank = descending age: no complement
                    } else if (gather && reverse) {
                        k = ~k;
                    }
                    key[j] = k;
                    val[j] = __ldcg(vs + p);
                }
            }
#pragma unroll
            for (int j = 0; j < kSortItems; ++j) {
                const uint32_t qi = base + 32u * j + lane;
                const uint32_t digit = qi < n ? (key[j] >> shift) & 255u : 256u;
                const uint32_t peers = __match_any_sync(0xffffffffu, digit);
                const uint32_t cnt = digit < 256u ? s_whist[warp][digit] : 0u;
                __syncwarp();
                if (digit < 256u && lane == __ffs(peers) - 1) s_whist[warp][digit] = (uint16_t)(cnt + __popc(peers));
                __syncwarp();
                rank[j] = cnt + __popc(peers & lt_mask);
            }
            __syncthreads();
            // thread t owns digit t: warp-exclusive offsets and the tile count
            const uint32_t t = threadIdx.x;
            uint32_t run = 0;
            if (t < 256) {
#pragma unroll
                for (int w = 0; w < kSortThreads / 32; ++w) {
                    const uint32_t c = s_whist[w][t];
                    s_whist[w][t] = (uint16_t)run;
                    run += c;
                }
            }
            uint32_t tile_total;
            const uint32_t start = cta_exclusive_scan<kSortThreads>(run, s_warp_sums, &tile_total);
            if (t < 256) {
                s_start[t] = start;
                const uint32_t excl = lookback_exclusive_w8(b.status + t, tile, run, epoch, &q->error, 20u + pass, 256u);
                s_gbase[t] = bucket[t] + excl - start;
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kSortItems; ++j) {
                const uint32_t qi = base + 32u * j + lane;
                if (qi < n) {
                    const uint32_t d = (key[j] >> shift) & 255u;
                    const uint32_t pos = s_start[d] + s_whist[warp][d] + rank[j];
                    s_keys[pos] = key[j];
                    s_vals[pos] = val[j];
                }
            }
            __syncthreads();
            const uint32_t count = min((uint32_t)kSortTile, n - tile * kSortTile);
            for (uint32_t i = threadIdx.x; i < count; i += kSortThreads) {
                const uint32_t k = s_keys[i];
                const uint32_t pos = s_gbase[(k >> shift) & 255u] + i;
                if (pos < n) {  // always true unless a look-back wait timed out
                    kd[pos] = k;
                    vd[pos] = s_vals[i];
                }
            }
            __syncthreads();
        }
    }
}

__global__ void k_sort_writeback(QueryState* q, const uint32_t* d_n, uint32_t n_host, SortBuffers b,
                                 uint32_t* keys, uint32_t* vals, int reverse)
{
    const uint32_t n = d_n ? *d_n : n_host;
    const uint32_t f = q->sort_final;
    const uint32_t* ks = f == 1 ? b.b_keys : b.c_keys;
    const uint32_t* vs = f == 1 ? b.b_vals : b.c_vals;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = ks[i];
        keys[i] = reverse ? ~k : k;
        vals[i] = vs[i];
    }
}

size_t sort_status_words(uint32_t n_max) { return (size_t)div_up(n_max ? n_max : 1, kSortTile) * 256u; }

// CTAs of k_sort resident per SM: the bound of its cooperative grid
static uint32_t sort_per_sm()
{
    static const uint32_t n = [] {
        int r = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_sort, kSortThreads, 0) != cudaSuccess || r < 1) r = 1;
        return (uint32_t)r;
    }();
    return n;
}

int sort_grid(bcmc_ctx* ctx, uint32_t n_max)
{
    const uint32_t tiles = div_up(n_max ? n_max : 1, kSortTile);
    const uint32_t resident = (uint32_t)ctx->num_sms * sort_per_sm();
    return (int)(tiles < resident ? tiles : resident);
}

void sort_launch(bcmc_ctx* ctx, QueryState* q, const uint32_t* d_n, uint32_t n_max,
                 const SortBuffers& bufs, int reverse, cudaStream_t s, int plan_ready)
{
    if (!plan_ready) {
        const int hist_grid = (int)min(div_up(n_max ? n_max : 1, 256u * 8u), (uint32_t)ctx->num_sms * 4u);
        k_sort_hist<<<hist_grid, 256, 0, s>>>(q, d_n, n_max, bufs.in_keys, reverse);
        count_launches(1);
    }
    // cooperative: the grid barriers between digit passes need every CTA resident
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(sort_grid(ctx, n_max));
    cfg.blockDim = dim3(kSortThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeCooperative;
    attr.val.cooperative = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    BCMC_CUDA(cudaLaunchKernelEx(&cfg, k_sort, q, d_n, n_max, bufs, reverse));
    count_launches(1);
}

void sort_writeback(bcmc_ctx* ctx, QueryState* q, const uint32_t* d_n, uint32_t n_max,
                    const SortBuffers& bufs, uint32_t* keys, uint32_t* vals, int reverse,
                    cudaStream_t s)
{
    const int grid = (int)min(div_up(n_max ? n_max : 1, 256u), (uint32_t)ctx->num_sms * 8u);
    k_sort_writeback<<<grid, 256, 0, s>>>(q, d_n, n_max, bufs, keys, vals, reverse);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

}  // namespace bcmc
