// bcmc_internal.cuh -- shared device/host helpers of libbcmc_gb300 (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "bcmc.h"  // include/ (on the include path)

namespace bcmc {

constexpr int kWarp = 32;
constexpr uint32_t kSpinLimit = 1u << 22;  // bounded device-side waits

// ---------------------------------------------------------------------------
// Per-query device state.  Every count the pipeline needs lives here so that a
// query is a fixed sequence of launches with no host round trip in between;
// the host reads this struct once at the end of the query.
// ---------------------------------------------------------------------------
// Inputs of one query as the host writes them (pinned memory, read directly by
// the first kernel of a query's CUDA graph).
struct QueryInputs {
    float isovalue;
    uint32_t capacity;
    uint32_t vert_capacity;
    uint32_t mc_only;
    uint32_t debug_drop_tile;  // test hook (bcmc_debug_drop_tile): 0, or tile + 1
};

struct QueryState {
    // inputs written by the host (or the query-init kernel)
    float isovalue;
    uint32_t epoch;          // tags the decoupled-lookback status words
    uint32_t capacity;       // physical slots of the cache buffers
    uint32_t cache_size;     // logical LRU size (js/lru_cache.js cacheSize)
    uint32_t vert_capacity;  // entries of the vertex buffer
    // active-block pass
    uint32_t num_active;
    uint32_t num_new;
    uint32_t old_cache_size;
    uint32_t new_cache_size;
    // LRU slot pass
    uint32_t num_avail;
    uint32_t display_slots_available;
    // marching cubes
    uint32_t num_with_verts;
    uint32_t num_verts;
    // flags
    uint32_t grow_needed;    // cache capacity exceeded: host grows and re-runs
    uint32_t vert_overflow;  // vertex buffer too small: host grows, re-runs MC
    uint32_t error;          // nonzero: a bounded wait timed out (code = site)
    // dynamic tile counters (zeroed by the init kernel)
    uint32_t tiles_active;
    uint32_t tiles_slots;
    uint32_t tiles_mc;
    uint32_t tiles_sort[4];
    uint32_t tiles_sort_hist;
    // radix sort plan (sort_plan, run by the last CTA of k_sort_hist or of
    // k_slots, whichever accumulated the digit histograms)
    uint32_t sort_src[4];     // source buffer (0/1) of each digit pass
    uint32_t sort_run[4];     // 1 if the digit pass runs
    uint32_t sort_first;      // index of the first pass that runs (4 = none)
    uint32_t sort_final;      // buffer holding the sorted values
    uint32_t sort_key16;      // 1: the passes sort the 16-bit age keys (age_key16); 2: their dense ranks (one pass)
    uint32_t sort_wide;       // k_slots: bit 0 an available slot's age has no 16-bit key, bit 1 none in an age bin
    uint32_t sort_hist[4][256];
    uint32_t sort_hist16[2][256];  // k_slots: digit histograms of the 16-bit age keys
    // test hook (bcmc_debug_drop_tile): 0, or t + 1 when tile t of the active
    // test and of the primitive scans must publish no look-back status
    uint32_t debug_drop_tile;
    // k_mc's grid barrier (CTAs arrived) and its emit tiles' counter
    uint32_t mc_arrived;
    uint32_t tiles_emit;
    uint32_t sort_arrived;  // k_sort's grid barriers between digit passes
    // the last age sort's plan was the one-pass one (k_slots then accumulates the
    // age bins alone); kept across queries, zero when the state is created
    uint32_t sort_prev_dense;
    uint32_t pad[3];
};

// The test hook's check: this tile publishes nothing, so the tiles after it
// wait on a status word that nobody sets until their bounded spin runs out.
__device__ __forceinline__ bool lb_dropped(const QueryState* q, uint32_t tile)
{
    return q->debug_drop_tile == tile + 1u;
}

// The LRU's slot ages (lru_cache.comp, lru_cache_init.comp) are small counts
// for slots used since the cache was (re)initialised and 100000 plus a count
// for the others.  While every age is below 2^15 or in [100000, 100000 + 2^15)
// this map is strictly increasing on them and fits 16 bits, so the sort by age
// can run two 8-bit digit passes instead of three with the same order and ties.
__device__ __forceinline__ bool age_has_key16(uint32_t age) { return age < 32768u || age - 100000u < 32768u; }
__device__ __forceinline__ uint32_t age_key16(uint32_t age) { return age < 32768u ? age : 32768u + (age - 100000u); }
// Ages below 256 within their class (a count of updates, or 100000 + a count):
// bin (class, low byte), in the order of age_key16.  kAgeBins marks any other age.
constexpr uint32_t kAgeBins = 512;
__device__ __forceinline__ uint32_t age_bin(uint32_t age)
{
    if (age < 256u) return age;
    if (age - 100000u < 256u) return 256u + (age - 100000u);
    return kAgeBins;
}

// ---------------------------------------------------------------------------
// Decoupled look-back status words: [epoch:30 | flag:2][value:32].
// flag 1 = tile aggregate, 2 = inclusive prefix.  Words from an older epoch read
// as "not ready", so the arrays need no clearing between launches.
// ---------------------------------------------------------------------------
constexpr uint64_t kFlagAggregate = 1;
constexpr uint64_t kFlagPrefix = 2;

__device__ __forceinline__ uint64_t lb_pack(uint32_t epoch, uint64_t flag, uint32_t value)
{
    return ((((uint64_t)epoch << 2) | flag) << 32) | value;
}

// Status words are published with relaxed stores: a reader uses only the
// flag and value carried in the word itself (never other data the writer
// wrote before it), so no release fence is needed, and a fence per publish
// would wait for every earlier store of the thread to reach L2.
__device__ __forceinline__ void lb_store(uint64_t* p, uint64_t v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Read side of the same: a relaxed load.  (An acquire load would also order
// every later load after it: the loads of a look-back window would complete
// one after another instead of together.)
__device__ __forceinline__ uint64_t lb_load(const uint64_t* p)
{
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Warp-cooperative look-back, called by all 32 lanes of one warp: each round
// reads the status words of 32 * kPer predecessors at once (a round trip to
// L2 costs microseconds when hundreds of tiles poll, so callers with many
// tiles widen the window), finds the nearest one
// holding an inclusive prefix with a ballot and sums the window with a warp
// reduction, so a walk past k unfinished predecessors costs k/32 round trips.
// Lane 0 publishes the aggregate first and the inclusive prefix at the end.
// Returns the exclusive prefix in every lane.  A timed-out wait records
// `site` in *err and stops the walk.
template <int kPer = 4>
__device__ __forceinline__ uint32_t warp_lookback(uint64_t* status, uint32_t tile, uint32_t aggregate,
                                                  uint32_t epoch, uint32_t* err, uint32_t site,
                                                  uint32_t stride = 1)
{
    const uint32_t lane = threadIdx.x & 31u;
    if (tile == 0) {
        if (lane == 0) lb_store(status, lb_pack(epoch, kFlagPrefix, aggregate));
        return 0;
    }
    if (lane == 0) lb_store(status + (uint64_t)tile * stride, lb_pack(epoch, kFlagAggregate, aggregate));
    // each lane owns kPer consecutive predecessors per round (nearest first):
    // 32 * kPer status words per round trip
    uint32_t exclusive = 0;
    int64_t tail = (int64_t)tile - 1;
    uint32_t spins = 0;
    bool timed_out = false;
    for (;;) {
        uint32_t flag[kPer], value[kPer];
        for (;;) {
            bool ready = true;
#pragma unroll
            for (int i = 0; i < kPer; ++i) {
                const int64_t pred = tail - (int64_t)(kPer * lane + i);
                flag[i] = (uint32_t)kFlagPrefix;  // before tile 0: prefix 0
                value[i] = 0;
                if (pred >= 0) {
                    const uint64_t s = lb_load(status + (uint64_t)pred * stride);
                    const uint32_t hi = (uint32_t)(s >> 32);
                    ready = ready && (hi >> 2) == epoch && (hi & 3u) != 0;
                    flag[i] = hi & 3u;
                    value[i] = (uint32_t)s;
                }
            }
            if (__all_sync(0xffffffffu, ready)) break;
            if (++spins > kSpinLimit) {
                timed_out = true;
                break;
            }
            if (spins > 8) __nanosleep(100);
        }
        if (timed_out) {
            if (lane == 0) atomicCAS(err, 0u, site);
            break;
        }
        // this lane's sum up to and including its nearest prefix (all 4 if none)
        uint32_t local = 0;
        bool has_prefix = false;
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            if (!has_prefix) local += value[i];
            has_prefix = has_prefix || flag[i] == (uint32_t)kFlagPrefix;
        }
        const uint32_t pmask = __ballot_sync(0xffffffffu, has_prefix);
        if (pmask) {
            const uint32_t first = (uint32_t)__ffs(pmask) - 1u;
            exclusive += __reduce_add_sync(0xffffffffu, lane <= first ? local : 0u);
            break;
        }
        exclusive += __reduce_add_sync(0xffffffffu, local);
        tail -= 32 * kPer;
    }
    if (lane == 0) lb_store(status + (uint64_t)tile * stride, lb_pack(epoch, kFlagPrefix, exclusive + aggregate));
    return exclusive;
}

// Per-thread look-back that keeps W predecessor loads in flight per round
// (used where every thread owns its own chain, e.g. one radix digit each).
template <int W = 8>
__device__ __forceinline__ uint32_t lookback_exclusive_w8(uint64_t* status, uint32_t tile, uint32_t aggregate,
                                                          uint32_t epoch, uint32_t* err, uint32_t site,
                                                          uint32_t stride)
{
    if (tile == 0) {
        lb_store(status, lb_pack(epoch, kFlagPrefix, aggregate));
        return 0;
    }
    lb_store(status + (uint64_t)tile * stride, lb_pack(epoch, kFlagAggregate, aggregate));
    uint32_t exclusive = 0;
    int64_t tail = (int64_t)tile - 1;
    uint32_t spins = 0;
    bool done = false;
    while (!done) {
        uint64_t s[W];
#pragma unroll
        for (int i = 0; i < W; ++i)
            s[i] = (tail - i >= 0) ? lb_load(status + (uint64_t)(tail - i) * stride)
                                   : lb_pack(epoch, kFlagPrefix, 0u);
#pragma unroll
        for (int i = 0; i < W; ++i) {
            if (done) break;
            uint32_t hi = (uint32_t)(s[i] >> 32);
            while ((hi >> 2) != epoch || (hi & 3u) == 0) {
                if (++spins > kSpinLimit) {
                    atomicCAS(err, 0u, site);
                    done = true;
                    break;
                }
                if (spins > 8) __nanosleep(100);
                s[i] = lb_load(status + (uint64_t)(tail - i) * stride);
                hi = (uint32_t)(s[i] >> 32);
            }
            if (done) break;
            exclusive += (uint32_t)s[i];
            if ((hi & 3u) == kFlagPrefix) done = true;
        }
        tail -= W;
    }
    lb_store(status + (uint64_t)tile * stride, lb_pack(epoch, kFlagPrefix, exclusive + aggregate));
    return exclusive;
}

// Warp-wide inclusive scan (shuffles).
__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// CTA-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the CTA total to *total.  `warp_sums` holds blockDim/32
// entries of shared memory.
template <int kThreads>
__device__ __forceinline__ uint32_t cta_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total)
{
    constexpr int kWarps = kThreads / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_inclusive_scan(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kWarps ? warp_sums[lane] : 0;
        const uint32_t wi = warp_inclusive_scan(w);
        if (lane < kWarps) warp_sums[lane] = wi - w;
        if (lane == kWarps - 1) warp_sums[kWarps] = wi;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + inc - v;
    *total = warp_sums[kWarps];
    __syncthreads();
    return r;
}

// The radix sort's pass plan, made by the last of the CTAs that accumulated
// the four raw 8-bit digit histograms in q->sort_hist (256 threads, after a
// fence): a digit pass is skipped when every one of the n keys has the same
// digit; the histograms become exclusive bucket offsets; the passes that run
// ping-pong between the two sort buffers, the first reading the input.
// `hist` holds the raw histograms of the first `ndig` digits; the digits
// after them are not sorted on (their passes are skipped).
__device__ __forceinline__ void sort_plan(QueryState* q, uint32_t n, uint32_t* warp_sums, const uint32_t* hist,
                                          int ndig)
{
    uint32_t* gh = &q->sort_hist[0][0];
    uint32_t run[4], hv[4];
#pragma unroll
    for (int d = 0; d < 4; ++d) hv[d] = d < ndig ? __ldcg(hist + d * 256 + threadIdx.x) : 0u;  // all in flight
    for (int d = 0; d < 4; ++d) {
        if (d >= ndig) {
            run[d] = 0;
            continue;
        }
        const uint32_t v = hv[d];
        const int full = __syncthreads_or(n > 0 && v == n);
        run[d] = (n > 0 && !full) ? 1u : 0u;
        uint32_t tot;
        const uint32_t ex = cta_exclusive_scan<256>(v, warp_sums, &tot);
        gh[d * 256 + threadIdx.x] = ex;
    }
    if (threadIdx.x == 0) {
        if (n > 0 && !(run[0] | run[1] | run[2] | run[3])) run[0] = 1;  // permutation still applies
        uint32_t cur = 0, first = 4;
        for (int d = 0; d < 4; ++d) {
            q->sort_run[d] = run[d];
            q->sort_src[d] = cur;
            if (run[d]) {
                if (first == 4) first = d;
                cur = (cur == 1u) ? 2u : 1u;
            }
        }
        q->sort_first = first;
        q->sort_final = cur == 0 ? 1u : cur;
    }
}

// Division by a run-time invariant divisor as a multiply-high and shifts
// (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994): exact for every 32-bit dividend.
struct FastDiv {
    uint32_t d, m, s;
};

__host__ __device__ inline FastDiv make_fastdiv(uint32_t d)
{
    FastDiv f{d, 0u, 0u};
    if (d > 1) {
        uint32_t l = 0;
        while ((1ull << l) < d) ++l;  // l = ceil(log2 d)
        f.m = (uint32_t)((((1ull << l) - d) << 32) / d + 1ull);
        f.s = l;
    }
    return f;
}

__host__ __device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f)
{
#ifdef __CUDA_ARCH__
    if (f.d == 1) return n;
    const uint32_t t = __umulhi(n, f.m);
#else
    if (f.d == 1) return n;
    const uint32_t t = (uint32_t)(((uint64_t)n * f.m) >> 32);
#endif
    return (t + ((n - t) >> 1)) >> (f.s - 1);
}

// block id -> (x, y, z) for a grid of nb.x * nb.y * nb.z blocks
struct BlockGrid {
    uint3 nb;
    FastDiv dx, dxy;
};

inline BlockGrid make_block_grid(uint3 nb) { return BlockGrid{nb, make_fastdiv(nb.x), make_fastdiv(nb.x * nb.y)}; }

__device__ __forceinline__ uint3 block_coords(uint32_t id, const BlockGrid& g)
{
    const uint32_t z = fdiv(id, g.dxy);
    const uint32_t r = id - z * g.nb.x * g.nb.y;
    const uint32_t y = fdiv(r, g.dx);
    return make_uint3(r - y * g.nb.x, y, z);
}

__host__ __device__ __forceinline__ uint32_t align_up(uint32_t v, uint32_t a)
{
    return (uint32_t)(((uint64_t)v + a - 1) / a * a);
}

__host__ __device__ __forceinline__ uint32_t div_up(uint32_t v, uint32_t a)
{
    return (uint32_t)(((uint64_t)v + a - 1) / a);
}

// Error helper for host code.
struct CudaError {
    cudaError_t err;
    const char* what;
};

}  // namespace bcmc

#define BCMC_CUDA(call)                                                       \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) throw ::bcmc::CudaError{e_, #call};            \
    } while (0)
