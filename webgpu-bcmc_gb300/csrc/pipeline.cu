// pipeline.cu -- device side of one isosurface query (computeSurface,
// js/compressed_marching_cubes.js:580-809) and of LRUCache.update
// (js/lru_cache.js:312-843).
//
// The reference runs ~20 dispatches with six host readbacks per query.  Here a
// query is a fixed sequence of launches that read every count from the
// QueryState on the device:
//   k_query_begin  new look-back epoch, counters cleared
//   k_active_ranges / k_active
//                  active test (compute_block_active.comp) for every block,
//                  fused with the compaction of active ids, the cache lookup
//                  (lru_cache_mark_new_items.comp's "needs caching") and the
//                  compaction of new item ids; the last tile decides the cache
//                  growth (js/lru_cache.js:510-522)
//   k_slots        age/mark/grow of every slot (lru_cache_age_slots.comp,
//                  lru_cache_mark_new_items.comp, lru_cache_init.comp) fused
//                  with the compaction of available slots and their ages, the
//                  sort keys' digit histograms and (last CTA) the sort's plan
//   sort           available slots by age, oldest first (sort.cu)
//   k_decode_new   beside k_slots and the sort (a branch of the query graph):
//                  the ZFP decode of the new blocks (zfp_decompress_block.comp)
//                  into a staging buffer
//   k_assign       lru_cache_update.comp, and the staged blocks copied into
//                  their slots
//   k_query_end    the query state the host reads, into its pinned copy
//   k_mc           marching cubes count + scan + emit in one cooperative launch
//                  (compute_block_has_vertices.comp,
//                  compute_block_voxel_num_verts.comp,
//                  compute_block_vertices.comp)
#include <algorithm>

#include "active_test.cuh"
#include "bcmc_pipeline.h"
#include "mc_common.cuh"
#include "zfp_device.cuh"

namespace bcmc {

// Starts a query: inputs come from the arguments, or, when `in` is set, from
// the host's pinned copy, read directly (a query graph reuses the pointer and
// needs no copy node for its inputs).
__global__ void k_query_begin(QueryState* q, float iso, int mc_only, uint32_t capacity, uint32_t vert_capacity,
                              const QueryInputs* in)
{
    const int t = threadIdx.x;
    if (in) {
        iso = __ldcv(&in->isovalue);
        mc_only = (int)__ldcv(&in->mc_only);
        capacity = __ldcv(&in->capacity);
        vert_capacity = __ldcv(&in->vert_capacity);
    }
    if (t == 0) {
        q->epoch += 1;
        q->capacity = capacity;
        q->vert_capacity = vert_capacity;
        q->tiles_mc = q->mc_arrived = q->tiles_emit = 0;
        q->error = 0;
        q->vert_overflow = 0;
        q->num_with_verts = 0;
        q->num_verts = 0;
        if (!mc_only) {
            q->debug_drop_tile = in ? __ldcv(&in->debug_drop_tile) : 0u;
            q->isovalue = iso;
            q->tiles_active = q->tiles_slots = q->tiles_sort_hist = 0;
            for (int i = 0; i < 4; ++i) q->tiles_sort[i] = 0;
            q->sort_arrived = 0;
            q->num_active = q->num_new = q->num_avail = 0;
            q->grow_needed = 0;
            // the sort plan of zero keys (k_slots replaces it when it sorts)
            for (int i = 0; i < 4; ++i) q->sort_run[i] = q->sort_src[i] = 0;
            q->sort_first = 4;
            q->sort_final = 1;
            q->sort_key16 = q->sort_wide = 0;
        }
    }
    if (!mc_only)
        for (int i = t; i < 1536; i += blockDim.x) (&q->sort_hist[0][0])[i] = 0;  // and sort_hist16
}

// Ends a query graph: the query state the host reads (the fields before the
// sort histograms) into the host's pinned copy, stored to mapped host memory
// by one warp instead of a copy node.
constexpr uint32_t kHostStateWords = offsetof(QueryState, sort_hist) / 4;

__global__ void k_query_end(const QueryState* q, QueryState* host)
{
    const uint32_t* src = reinterpret_cast<const uint32_t*>(q);
    uint32_t* dst = reinterpret_cast<uint32_t*>(host);
    for (uint32_t i = threadIdx.x; i < kHostStateWords; i += blockDim.x) dst[i] = __ldcg(src + i);
}

void query_end_launch(const QueryState* q, QueryState* host, cudaStream_t s)
{
    k_query_end<<<1, 64, 0, s>>>(q, host);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// k_active
// ---------------------------------------------------------------------------
constexpr int kActThreads = 256;
constexpr int kActiveItems = 4;
constexpr int kActiveTile = kActThreads * kActiveItems;  // blocks per k_active tile
constexpr int kSlotItems = 2;
constexpr int kSlotTile = kActThreads * kSlotItems;  // slots per k_slots tile

__device__ __forceinline__ uint32_t spad8(uint32_t i) { return i + (i >> 5); }

// The last tile of the active test: totals, and the cache growth decision.
__device__ __forceinline__ void active_finish(QueryState* q, uint32_t A, uint32_t N, uint32_t total)
{
    q->num_active = A;
    q->num_new = N;
    const uint32_t old = q->cache_size;
    uint32_t new_size = old;
    if (A > 0 && N > 0) {
        const uint32_t kept = A - N;
        const uint32_t avail = old - kept;
        if (avail < N) {  // js/lru_cache.js:519-522
            uint64_t grown = (uint64_t)old + (3ull * (N - avail) + 1ull) / 2ull;
            if (grown > total) grown = total;
            new_size = align_up((uint32_t)grown, 32u);
        }
        q->display_slots_available = new_size - A;
    }
    q->old_cache_size = old;
    q->new_cache_size = new_size;
    if (new_size > q->capacity) {  // host grows the buffers and re-runs the query
        q->grow_needed = new_size;
        q->num_avail = 0;
    } else {
        q->cache_size = new_size;
        q->num_avail = (A > 0 && N > 0) ? new_size - (A - N) : 0u;
    }
}

// k_active over the block ranges (the MC path), 4 consecutive blocks per
// thread, 1024 threads per tile.  The tile's ranges and all their 3x3x3 neighbours are
// staged once in shared memory as 2-bit flags (bit 0: iso >= lo, bit 1:
// iso <= hi): for each z-offset dz in {-1, 0, 1}, the window of block ids
// [B0 + dz*NX*NY - NX - 1, B0 + 2048 + dz*NX*NY + NX + 1) around the tile's
// blocks [B0, B0 + 2048) (stage_len = 2048 + 2*NX + 2 entries each).
// Neighbour (dx, dy, dz) of local block l sits at
// (dz+1)*stage_len + l + (dy+1)*NX + dx + 1.  Staging turns 27 dependent
// global loads per block into one round of independent loads per tile.
// 2048-block tiles (128 CTAs on the 256^3 volume) measured 1.5 us faster per
// query than 4096-block ones (64 CTAs), which kept the look-back to one
// window there but left most SMs idle.
constexpr int kActRThreads = 512;
constexpr int kActRItems = 4;                          // consecutive blocks per thread
constexpr int kActRTile = kActRThreads * kActRItems;  // blocks per tile
constexpr int kActRStage = 5;  // staged ranges per thread and window in one round (5 * 512 >= 2048 + 2*NX + 2 for NX <= 255)

__global__ void __launch_bounds__(kActRThreads, 1) k_active_ranges(QueryState* q, ActiveArgs a, uint32_t stage_len)
{
    __shared__ uint32_t s_warp[kActRThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_pa, s_pn;
    extern __shared__ uint8_t s_bits[];  // 3 * stage_len flag bytes
    const uint32_t total = a.total;
    const uint32_t ntiles = div_up(total, kActRTile);
    const uint32_t epoch = q->epoch;
    const float iso = q->isovalue;
    const uint3 nb = a.grid.nb;
    const uint32_t nx = nb.x, nxy = nb.x * nb.y;
    const uint32_t t = threadIdx.x;
    for (;;) {
        if (t == 0) s_tile = atomicAdd(&q->tiles_active, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        // all of a thread's loads first (up to kActRStage per window, in
        // flight together), then the flags
        for (uint32_t i0 = 0; i0 < stage_len; i0 += kActRStage * kActRThreads) {
            float2 r[3][kActRStage];
#pragma unroll
            for (int dz = 0; dz < 3; ++dz) {
                const int64_t start = (int64_t)tile * kActRTile + (int64_t)(dz - 1) * nxy - nx - 1;
#pragma unroll
                for (int k = 0; k < kActRStage; ++k) {
                    const uint32_t i = i0 + k * kActRThreads + t;
                    const int64_t id = start + i;
                    r[dz][k] = (i < stage_len && id >= 0 && id < (int64_t)total) ? __ldg(a.ranges + id)
                                                                                 : make_float2(NAN, NAN);
                }
            }
#pragma unroll
            for (int dz = 0; dz < 3; ++dz)
#pragma unroll
                for (int k = 0; k < kActRStage; ++k) {
                    const uint32_t i = i0 + k * kActRThreads + t;
                    if (i < stage_len) {
                        uint32_t ra, rb;
                        range_bits(r[dz][k], iso, ra, rb);  // NaN (outside the volume): no flags
                        s_bits[(uint32_t)dz * stage_len + i] = (uint8_t)(ra | (rb << 1));
                    }
                }
        }
        __syncthreads();
        const uint32_t l0 = kActRItems * t, b0 = tile * kActRTile + l0;
        uint32_t act = 0, need = 0;  // bit j = block b0 + j
#pragma unroll
        for (int j = 0; j < kActRItems; ++j) {
            const uint32_t b = b0 + j, l = l0 + j;
            if (b >= total) break;
            const uint3 c = block_coords(b, a.grid);
            // valid neighbour offsets per axis: bit (d + 1) for d in {-1, 0, 1}
            const uint32_t mx = (c.x > 0 ? 1u : 0u) | 2u | (c.x + 1 < nb.x ? 4u : 0u);
            const uint32_t my = (c.y > 0 ? 1u : 0u) | 2u | (c.y + 1 < nb.y ? 4u : 0u);
            const uint32_t mz = (c.z > 0 ? 1u : 0u) | 2u | (c.z + 1 < nb.z ? 4u : 0u);
            const uint32_t self = s_bits[stage_len + l + nx + 1];
            uint32_t orv = 0, anyc = 0;
#pragma unroll
            for (int dz = 0; dz < 3; ++dz)
#pragma unroll
                for (int dy = 0; dy < 3; ++dy) {
                    if (!((mz >> dz) & (my >> dy) & 1u)) continue;
                    const uint8_t* row = s_bits + (uint32_t)dz * stage_len + l + (uint32_t)dy * nx;
#pragma unroll
                    for (int dx = 0; dx < 3; ++dx) {
                        const uint32_t v = (mx >> dx) & 1u ? (uint32_t)row[dx] : 0u;
                        orv |= v;
                        anyc |= (v + 1u) >> 2;  // 1 when both flags are set
                    }
                }
            // compute_block_active.comp:24-61 (see block_is_active)
            act |= (((self & (orv >> 1)) | ((self >> 1) & orv) | anyc) & 1u) << j;
        }
        if (kActRItems == 4 && b0 + kActRItems <= total) {
            *reinterpret_cast<uint4*>(a.active_out + b0) =
                make_uint4(act & 1u, (act >> 1) & 1u, (act >> 2) & 1u, (act >> 3) & 1u);
            if (act && a.item_slots) {
                const int4 s4 = __ldg(reinterpret_cast<const int4*>(a.item_slots + b0));
                need = ((s4.x < 0 ? 1u : 0u) | (s4.y < 0 ? 2u : 0u) | (s4.z < 0 ? 4u : 0u) | (s4.w < 0 ? 8u : 0u)) & act;
            }
        } else {
            for (uint32_t j = 0; j < (uint32_t)kActRItems && b0 + j < total; ++j) {
                a.active_out[b0 + j] = (act >> j) & 1u;
                if ((act >> j & 1u) && a.item_slots && a.item_slots[b0 + j] < 0) need |= 1u << j;
            }
        }
        uint32_t tot;
        const uint32_t excl =
            cta_exclusive_scan<kActRThreads>((uint32_t)__popc(act) | ((uint32_t)__popc(need) << 16), s_warp, &tot);
        if (t < 32) {
            const uint32_t p =
                lb_dropped(q, tile) ? 0u : warp_lookback(a.status_a, tile, tot & 0xffffu, epoch, &q->error, 30u);
            if (t == 0) s_pa = p;
        } else if (t < 64) {
            const uint32_t p =
                lb_dropped(q, tile) ? 0u : warp_lookback(a.status_n, tile, tot >> 16, epoch, &q->error, 31u);
            if (t == 32) s_pn = p;
        }
        __syncthreads();
        uint32_t pa = s_pa + (excl & 0xffffu), pn = s_pn + (excl >> 16);
#pragma unroll
        for (int j = 0; j < kActRItems; ++j) {
            if (act >> j & 1u) {
                if (a.active_ids) a.active_ids[pa] = b0 + j;
                ++pa;
            }
            if (need >> j & 1u) {
                if (a.new_ids) a.new_ids[pn] = b0 + j;
                ++pn;
            }
        }
        if (tile == ntiles - 1 && t == 0) active_finish(q, s_pa + (tot & 0xffffu), s_pn + (tot >> 16), total);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kActThreads) k_active(QueryState* q, ActiveArgs a)
{
    __shared__ uint32_t s_warp[kActThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_pa, s_pn;
    const uint32_t total = a.total;
    const uint32_t ntiles = div_up(total, kActiveTile);
    const uint32_t epoch = q->epoch;
    const float iso = q->isovalue;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&q->tiles_active, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        // thread -> 4 consecutive blocks (thread-blocked order = block order)
        const uint32_t b0 = tile * kActiveTile + kActiveItems * threadIdx.x;
        uint32_t act = 0, need = 0;  // bit i = block b0 + i
        if (b0 < total) {
            const uint32_t n = min(4u, total - b0);
            if (a.ranges) {
                const uint3 c = block_coords(b0, a.grid);
                if (n == 4 && c.x + 3 < a.grid.nb.x) {
                    act = row4_active(a.ranges, a.grid, c, b0, iso);
                } else {
                    for (uint32_t i = 0; i < n; ++i) act |= block_is_active(a.ranges, a.grid, b0 + i, iso) << i;
                }
                if (n == 4)
                    *reinterpret_cast<uint4*>(a.active_out + b0) =
                        make_uint4(act & 1u, (act >> 1) & 1u, (act >> 2) & 1u, (act >> 3) & 1u);
                else
                    for (uint32_t i = 0; i < n; ++i) a.active_out[b0 + i] = (act >> i) & 1u;
            } else {
                for (uint32_t i = 0; i < n; ++i) act |= (a.item_needed[b0 + i] != 0u ? 1u : 0u) << i;
            }
            if (a.item_slots && act) {
                if (n == 4) {
                    const int4 s4 = __ldg(reinterpret_cast<const int4*>(a.item_slots + b0));
                    need = (s4.x < 0 ? 1u : 0u) | (s4.y < 0 ? 2u : 0u) | (s4.z < 0 ? 4u : 0u) | (s4.w < 0 ? 8u : 0u);
                } else {
                    for (uint32_t i = 0; i < n; ++i) need |= (a.item_slots[b0 + i] < 0 ? 1u : 0u) << i;
                }
                need &= act;
            }
        }
        const uint32_t cnt = (uint32_t)__popc(act) | ((uint32_t)__popc(need) << 16);
        uint32_t tot;
        const uint32_t excl = cta_exclusive_scan<kActThreads>(cnt, s_warp, &tot);
        if (threadIdx.x < 32) {
            const uint32_t p =
                lb_dropped(q, tile) ? 0u : warp_lookback(a.status_a, tile, tot & 0xffffu, epoch, &q->error, 30u);
            if (threadIdx.x == 0) s_pa = p;
        } else if (threadIdx.x < 64) {
            const uint32_t p =
                lb_dropped(q, tile) ? 0u : warp_lookback(a.status_n, tile, tot >> 16, epoch, &q->error, 31u);
            if (threadIdx.x == 32) s_pn = p;
        }
        __syncthreads();
        uint32_t pa = s_pa + (excl & 0xffffu), pn = s_pn + (excl >> 16);
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) {
            if (act >> i & 1u) {
                if (a.active_ids) a.active_ids[pa] = b0 + i;
                ++pa;
            }
            if (need >> i & 1u) {
                if (a.new_ids) a.new_ids[pn] = b0 + i;
                ++pn;
            }
        }
        if (tile == ntiles - 1 && threadIdx.x == 0) active_finish(q, s_pa + (tot & 0xffffu), s_pn + (tot >> 16), total);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// k_slots: age + mark + init of new slots, fused with the compaction of the
// available slots (ascending slot id) and their ages.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kActThreads) k_slots(QueryState* q, SlotArgs a)
{
    __shared__ uint8_t s_flags[kSlotTile + kSlotTile / 32];
    __shared__ uint32_t s_warp[kActThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_prefix;
    __shared__ uint32_t s_hist[6][256];  // ~age digits 0-3, then the 16-bit keys' digits 0-1
    __shared__ uint32_t s_bins[kAgeBins];  // age bins (age_bin)
    __shared__ bool s_last;
    if ((a.skip_when_inactive && q->num_active == 0) || q->grow_needed) return;
    const uint32_t old = q->old_cache_size, nsz = q->new_cache_size;
    const bool compact = q->num_new > 0;
    const bool hist = compact && a.plan != 0u;
    // the six digit histograms of the sort keys are needed unless the plan is
    // the one-pass one on the age bins; expect that when the last update's was
    // (a misprediction is repaired by the last CTA below)
    const bool digits = hist && q->sort_prev_dense == 0u;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t wide = 0;     // an age without a 16-bit key
    uint32_t binless = 0;  // an age outside the age bins
    if (hist) {
        if (digits)
            for (int i = threadIdx.x; i < 1536; i += kActThreads) (&s_hist[0][0])[i] = 0;
        for (int i = threadIdx.x; i < (int)kAgeBins; i += kActThreads) s_bins[i] = 0;
    }
    const uint32_t ntiles = div_up(nsz, kSlotTile);
    const uint32_t epoch = q->epoch;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&q->tiles_slots, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t base = tile * kSlotTile;
#pragma unroll
        for (int j = 0; j < kSlotItems; ++j) {
            const uint32_t local = j * kActThreads + threadIdx.x;
            const uint32_t s = base + local;
            uint32_t av = 0;
            if (s < old) {
                const int32_t it = a.slot_item[s];
                const bool keep = it >= 0 && a.needed[it] != 0u;
                const uint32_t age = keep ? 0u : a.slot_age[s] + 1u;
                av = keep ? 0u : 1u;
                a.slot_age[s] = age;
                a.slot_avail[s] = av;
            } else if (s < nsz) {  // lru_cache_init.comp:27-29
                a.slot_age[s] = 100000u;
                a.slot_avail[s] = 1u;
                a.slot_item[s] = -1;
                av = 1u;
            }
            s_flags[spad8(local)] = (uint8_t)av;
        }
        if (compact) {
            __syncthreads();
            uint32_t cnt = 0;
            uint8_t fl[kSlotItems];
#pragma unroll
            for (int j = 0; j < kSlotItems; ++j) {
                fl[j] = s_flags[spad8(threadIdx.x * kSlotItems + j)];
                cnt += fl[j];
            }
            uint32_t tot;
            const uint32_t excl = cta_exclusive_scan<kActThreads>(cnt, s_warp, &tot);
            if (threadIdx.x < 32) {
                const uint32_t p = warp_lookback(a.status, tile, tot, epoch, &q->error, 32u);
                if (threadIdx.x == 0) s_prefix = p;
            }
            __syncthreads();
            uint32_t p = s_prefix + excl;
            const uint32_t first = base + threadIdx.x * kSlotItems;
#pragma unroll
            for (int j = 0; j < kSlotItems; ++j) {
                uint32_t age = 0;
                if (fl[j]) {
                    const uint32_t s = first + j;
                    age = a.slot_age[s];
                    a.avail_ids[p] = s;
                    a.avail_keys[p] = age;
                    ++p;
                }
                if (hist) {  // one shared atomic per distinct digit and warp
                    const uint32_t k = ~age, k16 = ~age_key16(age);
                    const bool has16 = fl[j] && age_has_key16(age);
                    if (fl[j] && !has16) wide = 1;
                    // the joint histogram of the age bins (one shared atomic per distinct bin and warp)
                    const uint32_t bin = fl[j] ? age_bin(age) : kAgeBins + 1u;
                    if (bin == kAgeBins) binless = 1;
                    const uint32_t bp = __match_any_sync(0xffffffffu, bin);
                    if (bin < kAgeBins && lane == (uint32_t)__ffs(bp) - 1u) atomicAdd(&s_bins[bin], (uint32_t)__popc(bp));
                    if (digits) {
#pragma unroll
                        for (int d = 0; d < 6; ++d) {
                            const uint32_t digit = fl[j] ? ((d < 4 ? k : k16) >> (8 * (d & 3))) & 255u : 256u;
                            const uint32_t peers = __match_any_sync(0xffffffffu, digit);
                            if (fl[j] && lane == (uint32_t)__ffs(peers) - 1u)
                                atomicAdd(&s_hist[d][digit], (uint32_t)__popc(peers));
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
    if (!hist) return;
    // this CTA's histograms into q->sort_hist; the last CTA to finish makes
    // the sort's pass plan (what k_sort_hist's last CTA does)
    uint32_t* gh = &q->sort_hist[0][0];  // sort_hist16 follows it
    if (digits)
        for (int i = threadIdx.x; i < 1536; i += kActThreads) {
            const uint32_t c = (&s_hist[0][0])[i];
            if (c) atomicAdd(gh + i, c);
        }
    for (int i = threadIdx.x; i < (int)kAgeBins; i += kActThreads)
        if (s_bins[i]) atomicAdd(a.age_hist + i, s_bins[i]);
    if (__syncthreads_or(wide) && threadIdx.x == 0) atomicOr(&q->sort_wide, 1u);
    if (__syncthreads_or(binless) && threadIdx.x == 0) atomicOr(&q->sort_wide, 2u);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&q->tiles_sort_hist, 1u) == gridDim.x - 1u;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t flags = *reinterpret_cast<volatile uint32_t*>(&q->sort_wide);
    const bool key16 = (flags & 1u) == 0u;
    // the age bins in use (two per thread, in age order) and how many
    uint32_t cnt[2], used = 0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        cnt[k] = __ldcg(a.age_hist + 2u * threadIdx.x + k);
        used += cnt[k] ? 1u : 0u;
    }
    uint32_t distinct;
    const uint32_t below = cta_exclusive_scan<kActThreads>(used, s_warp, &distinct);
    // every age in a bin and at most 256 bins used: one sort pass on the bins'
    // dense ranks, older ages (higher bins) ranked first
    const bool dense = flags == 0u && distinct <= 256u;
    uint32_t* rank_hist = &q->sort_hist16[0][0];  // reused for the ranks' histogram
    if (dense) {
        rank_hist[threadIdx.x] = 0u;
        __syncthreads();
        uint32_t p = below;
#pragma unroll
        for (int k = 0; k < 2; ++k)
            if (cnt[k]) {
                const uint32_t rank = distinct - 1u - p++;
                a.age_rank[2u * threadIdx.x + k] = (uint8_t)rank;
                rank_hist[rank] = cnt[k];
            }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) a.age_hist[2u * threadIdx.x + k] = 0u;  // zero again for the next update
    if (!dense && !digits) {
        // the one-pass plan was expected and does not apply: the digit
        // histograms from the compacted keys, by this CTA alone (the CTAs
        // accumulated none, so q->sort_hist is still zero)
        const uint32_t n = q->num_avail;
        for (int i = threadIdx.x; i < 1536; i += kActThreads) (&s_hist[0][0])[i] = 0;
        __syncthreads();
        for (uint32_t i0 = 0; i0 < n; i0 += kActThreads) {
            const uint32_t i = i0 + threadIdx.x;
            const bool v = i < n;
            const uint32_t age = v ? __ldcg(a.avail_keys + i) : 0u;
            const uint32_t k = ~age, k16 = ~age_key16(age);
#pragma unroll
            for (int d = 0; d < 6; ++d) {
                const uint32_t digit = v ? ((d < 4 ? k : k16) >> (8 * (d & 3))) & 255u : 256u;
                const uint32_t peers = __match_any_sync(0xffffffffu, digit);
                if (v && lane == (uint32_t)__ffs(peers) - 1u) atomicAdd(&s_hist[d][digit], (uint32_t)__popc(peers));
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 1536; i += kActThreads) gh[i] = (&s_hist[0][0])[i];
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        q->sort_key16 = dense ? 2u : (key16 ? 1u : 0u);
        q->sort_prev_dense = dense ? 1u : 0u;
    }
    if (dense) sort_plan(q, q->num_avail, s_warp, rank_hist, 1);
    else if (key16) sort_plan(q, q->num_avail, s_warp, &q->sort_hist16[0][0], 2);
    else sort_plan(q, q->num_avail, s_warp, &q->sort_hist[0][0], 4);
}

// ---------------------------------------------------------------------------
// k_assign: lru_cache_update.comp:19-37 (+ the new block's data into its slot
// when `words` is set: copied from the staging buffer k_decode_new filled,
// decoded here for new-block indices past it).
// ---------------------------------------------------------------------------
constexpr int kAssignThreads = 128;

__global__ void __launch_bounds__(kAssignThreads) k_assign(QueryState* q, AssignArgs a)
{
    if (q->num_active == 0 || q->grow_needed) return;
    const uint32_t n = q->num_new;
    const uint32_t size = q->new_cache_size;
    const uint32_t* __restrict__ sorted = q->sort_final == 1 ? a.sorted_b : a.sorted_c;
    const uint32_t first_decode = a.stage ? a.stage_blocks : 0u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t item = a.new_ids[i];
        const uint32_t slot = sorted[i];
        if (slot >= size) {  // cannot happen with a consistent sort; never write out of bounds
            atomicCAS(&q->error, 0u, 50u);
            continue;
        }
        const int32_t prev = a.slot_item[slot];
        if (prev != -1) a.item_slots[prev] = -1;
        a.slot_age[slot] = 0;
        a.slot_item[slot] = (int32_t)item;
        a.slot_avail[slot] = 0;
        a.item_slots[item] = (int32_t)slot;
        if (a.words && i >= first_decode) {
            // decoded here: every new block of the standalone LRU update, the ones
            // past the staging buffer on the query path.  Rare enough on the query
            // path that the words are read in place and the plane scratch is
            // thread-local, which keeps this kernel free of shared memory for its
            // assignment and copy work.
            __align__(16) uint32_t pl[64];
            float v[64];
            zfp_decode_staged(reinterpret_cast<const uint32_t*>(a.words + (uint64_t)item * (a.max_bits / 64u)),
                              a.max_bits, pl, v);
            float4* d4 = reinterpret_cast<float4*>(a.cache + (uint64_t)slot * 64u);
#pragma unroll
            for (int k = 0; k < 16; ++k) d4[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        }
    }
    if (!a.stage) return;
    // staged blocks into their slots: 16 threads per block, 16 B each
    const uint32_t ns = n < a.stage_blocks ? n : a.stage_blocks;
    const float4* __restrict__ src = reinterpret_cast<const float4*>(a.stage);
    float4* dst = reinterpret_cast<float4*>(a.cache);
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < ns * 16u; e += gridDim.x * blockDim.x) {
        const uint32_t i = e >> 4, k = e & 15u;
        const uint32_t slot = sorted[i];
        if (slot < size) dst[(uint64_t)slot * 16u + k] = __ldcs(src + (uint64_t)i * 16u + k);
    }
}

// ---------------------------------------------------------------------------
// k_decode_new: zfp_decompress_block.comp's decode of the query's new blocks,
// by new-block index into the staging buffer.  It depends on the active test
// only, so it runs beside k_slots and the sort; k_assign then copies the
// staged blocks into the slots the sort chose.
// ---------------------------------------------------------------------------
constexpr int kDecodeNewThreads = 128;

__global__ void __launch_bounds__(kDecodeNewThreads, 5) k_decode_new(const QueryState* q, DecodeArgs a)
{
    if (q->num_active == 0 || q->grow_needed) return;
    const uint32_t n = q->num_new < a.stage_blocks ? q->num_new : a.stage_blocks;
    extern __shared__ __align__(16) uint32_t s_words[];
    const uint32_t rate = a.max_bits / 64u;
    uint32_t* pl = zfp_stage_planes(s_words, kDecodeNewThreads, rate);
    if (threadIdx.x < 4) s_words[kDecodeNewThreads * 2u * rate + threadIdx.x] = 0u;
    const uint32_t wb = threadIdx.x & ~31u;
    for (uint32_t i0 = blockIdx.x * kDecodeNewThreads; i0 < n; i0 += gridDim.x * kDecodeNewThreads) {
        const uint32_t i = i0 + threadIdx.x;
        __syncthreads();
        if (i < n) zfp_stage_block(a.words, a.new_ids[i], rate, s_words);
        __syncthreads();
        if (i0 + wb >= n) continue;  // the whole warp
        const bool mine = i < n;
        float v[64];
        if (mine) zfp_decode_staged(s_words + threadIdx.x * 2u * rate, a.max_bits, pl, v);
        zfp_store_warp(pl, v, mine, a.stage + (uint64_t)(i0 + wb) * 64u, n - (i0 + wb));
    }
}

// ---------------------------------------------------------------------------
// k_mc: marching cubes over the active blocks, 16 blocks per tile.
// ---------------------------------------------------------------------------
constexpr int kMcBlocks = 16;
constexpr int kMcThreads = 256;
constexpr int kMcCells = 64 * kMcBlocks;  // 4 consecutive cells per thread
constexpr int kMcPerSm = 6;               // resident CTAs per SM (the grid: one launch, all resident)
constexpr int kMcMaskWords = kMcCells * 15 / 32;  // a tile holds at most 15 vertices per cell

// Marching cubes over the active blocks, one cooperative launch (every CTA
// resident).  Each CTA owns one contiguous range of active blocks:
//   count pass: per 16-block tile, one parallel round of loads fetches the
//     active flags and cache slots of every block's 7 +x/+y/+z neighbours and
//     its own slot, a second round fills each block's 5^3 grid in shared
//     memory (16 B loads of 4 voxels per thread, ghost voxels alongside); a
//     thread tests its 4 corner rows once and derives the cases and vertex
//     counts of its 4 cells; block totals are kept;
//   one warp-cooperative decoupled look-back per CTA turns the CTA totals into
//     its global vertex offset and its offset in the blocks-with-vertices list;
//   the range's entries of that list and their vertex offsets (a CTA scan over
//     the block totals), then a grid barrier;
//   emit: tiles of 16 consecutive list entries, claimed from a counter by
//     whichever CTA is free -- vertex counts differ between ranges by up to
//     7x, so the emit work is balanced across the grid, not per range --
//     reloaded (from L2); a CTA scan gives each cell's offset and marks each
//     cell's first vertex in a bitmask, and the vertices are spread over the
//     CTA -- thread k takes vertex k of the tile, finds its cell from the
//     bitmask (a population count below bit k plus the cells started before
//     its word), its edge's two corners and axis in the (case, vertex) table
//     -- so lanes stay converged and stores are contiguous.
// Ranges of at most two tiles (small queries) skip the barrier: each CTA
// emits its own range's tiles of blocks with vertices.  On the 256^3 CT-like
// sweep the barrier and the tile claims cost 6-10 us on queries of under
// 30,000 active blocks and the balance saves up to 48 us on the largest.
// Output order = the reference's: active-block order, cell order, table order.
// kHost: the vertices go to page-locked host memory (a.host_verts); its own
// instantiation keeps the device path's emit loop free of the alignment shift.
template <bool kHost>
__global__ void __launch_bounds__(kMcThreads, kMcPerSm) k_mc(QueryState* q, McArgs a)
{
    // a block's 5^3 grid; rows 144 floats apart (16 mod 32 banks), so the two
    // blocks of a warp read their corner rows on complementary banks
    __shared__ float s_vol[kMcBlocks][144];
    __shared__ uint8_t s_rm[kMcBlocks][32];  // corner-row masks of each block (count_cells)
    __shared__ uint32_t s_pair[32], s_pair_sw[32];  // 5-bit row mask -> per-cell corner pairs
    __shared__ __align__(16) uint16_t s_te[256][16];  // c_tri_edges
    __shared__ __align__(16) uint32_t s_cp[64 * 8];    // c_corner_pack
    __shared__ __align__(16) uint8_t s_cnt[256];
    __shared__ __align__(16) uint8_t s_case[kMcCells];
    __shared__ uint32_t s_cells[kMcCells];          // the tile's cells with vertices in order: cell | first vertex << 16
    __shared__ uint32_t s_vmask[kMcMaskWords];      // bit k: vertex k of the tile is its cell's first
    __shared__ uint16_t s_vbase[kMcMaskWords];      // cells with vertices starting before vertex 32w
    __shared__ uint32_t s_boff[kMcBlocks];          // each block's first vertex in the tile
    __shared__ uint32_t s_id[kMcBlocks];
    __shared__ uint32_t s_slot[kMcBlocks][8];
    __shared__ uint32_t s_act[kMcBlocks];
    __shared__ uint32_t s_warp[kMcThreads / 32 + 1];
    __shared__ uint32_t s_idx[kMcBlocks];
    __shared__ uint32_t s_stop, s_with, s_pv, s_pb, s_cta_v, s_cta_b, s_rank, s_cursor;
    __shared__ uint32_t s_gdesc[64];  // ghost_desc of each ghost voxel
    __shared__ uint8_t s_nb_off[8];

    const uint32_t A = q->num_active;
    if (A == 0 || q->grow_needed) return;
    const uint32_t epoch = q->epoch;
    const float iso = q->isovalue;
    const uint32_t cap = q->vert_capacity;
    const uint32_t slots = q->cache_size;
    const uint3 nb = a.nb;
    const uint32_t t = threadIdx.x;
    const uint32_t G = gridDim.x;
    if (t == 0) s_rank = atomicAdd(&q->tiles_mc, 1u);
    __syncthreads();
    const uint32_t rank = s_rank;
    const uint32_t range = div_up(div_up(A, G), kMcBlocks) * kMcBlocks;
    const uint32_t start = min(A, rank * range), end = min(A, start + range);
    // ranks 0 .. worked - 1 own blocks; the others take part in no look-back
    // (the walk of the last rank, past every predecessor, would end the kernel)
    const uint32_t worked = div_up(A, range);
    for (uint32_t i = t; i < 512u; i += kMcThreads)
        reinterpret_cast<uint4*>(&s_te[0][0])[i] = reinterpret_cast<const uint4*>(&c_tri_edges.e[0][0])[i];
    if (t < 128) reinterpret_cast<uint4*>(s_cp)[t] = reinterpret_cast<const uint4*>(&c_corner_pack.p[0][0])[t];
    if (t < 16) reinterpret_cast<uint4*>(s_cnt)[t] = reinterpret_cast<const uint4*>(c_tri.count)[t];
    if (t == 0) {
        s_cta_v = s_cta_b = 0;
        s_pv = s_pb = 0;
        s_cursor = start;
    }
    if (t < 61) s_gdesc[t] = ghost_desc(c_ghost[t]);
    if (t < 32) {
        uint32_t w = 0, ws = 0;
#pragma unroll
        for (uint32_t x = 0; x < 4; ++x) {
            const uint32_t pr = (t >> x) & 3u;
            w |= pr << (8u * x);
            ws |= (((pr & 1u) << 1) | (pr >> 1)) << (8u * x);
        }
        s_pair[t] = w;
        s_pair_sw[t] = ws;
    }
    if (t < 7) s_nb_off[t] = c_nb_off[t];
    const uint32_t j = t >> 4, u = t & 15u, ry = u & 3u, rz = u >> 2;

    auto load_tile = [&]() -> uint32_t {
        if (t < kMcBlocks * 8) {
            const uint32_t jb = t >> 3, k = t & 7u, id = s_id[jb];
            uint32_t slot = 0xffffffffu, act = 0;
            if (id != 0xffffffffu) {
                const uint3 bc = block_coords(id, a.grid);
                const uint32_t bx = bc.x, by = bc.y, bz = bc.z;
                if (k == kNbSelf) {
                    slot = (uint32_t)__ldg(a.item_slots + id);
                    act = (bx + 1 < nb.x ? 0x100u : 0u) | (by + 1 < nb.y ? 0x200u : 0u) |
                          (bz + 1 < nb.z ? 0x400u : 0u);
                } else {
                    const uint32_t o = s_nb_off[k], ox = o & 1u, oy = (o >> 1) & 1u, oz = o >> 2;
                    if (bx + ox < nb.x && by + oy < nb.y && bz + oz < nb.z) {
                        const uint32_t nid = id + ox + nb.x * (oy + nb.y * oz);
                        act = __ldg(a.active + nid) != 0u ? 1u : 0u;
                        slot = (uint32_t)__ldg(a.item_slots + nid);
                    }
                }
            }
            s_slot[jb][k] = slot;
            const uint32_t bits = __ballot_sync(0xffffffffu, (act & 1u) != 0u);
            if (k == kNbSelf) s_act[jb] = ((bits >> (t & 24u)) & 0x7fu) | act;
        }
        __syncthreads();
        const uint32_t id = s_id[j];
        uint32_t dims = 0;
        if (id != 0xffffffffu) {
            const uint32_t act = s_act[j];
            dims = block_dims_with_ghost(act, (act & 0x100u) != 0u, (act & 0x200u) != 0u, (act & 0x400u) != 0u);
            const uint32_t slot = s_slot[j][kNbSelf];
            float4 v4 = make_float4(0.f, 0.f, 0.f, 0.f);
            if (slot < slots) v4 = __ldg(reinterpret_cast<const float4*>(a.cache + (uint64_t)slot * 64u) + u);
            else atomicCAS(&q->error, 0u, 51u);
            const uint32_t has = ghost_axes(dims);
            float gv[4];
            uint32_t gaddr[4];
#pragma unroll
            for (uint32_t r = 0; r < 4; ++r) {
                const uint32_t gi = u + 16u * r;
                gv[r] = 0.0f;
                gaddr[r] = 0xffffffffu;
                if (gi < 61) {
                    const uint32_t d = s_gdesc[gi];
                    if ((d & 7u & ~has) == 0u) {
                        const uint32_t nslot = s_slot[j][d >> 16];
                        if (nslot < slots) {
                            gv[r] = __ldg(a.cache + (uint64_t)nslot * 64u + ((d >> 3) & 63u));
                            gaddr[r] = (d >> 9) & 127u;
                        } else {
                            atomicCAS(&q->error, 0u, 52u);
                        }
                    }
                }
            }
            float* row = &s_vol[j][5u * (ry + 5u * rz)];
            row[0] = v4.x;
            row[1] = v4.y;
            row[2] = v4.z;
            row[3] = v4.w;
#pragma unroll
            for (uint32_t r = 0; r < 4; ++r)
                if (gaddr[r] != 0xffffffffu) s_vol[j][gaddr[r]] = gv[r];
        }
        __syncthreads();
        return dims;
    };
    // cases and counts of cells 4u..4u+3 (compute_block_has_vertices.comp:28-51):
    // the 4 corner rows (y, z), (y+1, z), (y, z+1), (y+1, z+1) are tested once each
    auto count_cells = [&](uint32_t dims, uint32_t nv[4], uint32_t& cs4) -> uint32_t {
        const uint32_t dx = dims & 15u, dy = (dims >> 4) & 15u, dz = dims >> 8;
        const bool row_ok = s_id[j] != 0xffffffffu && ry + 1 < dy && rz + 1 < dz;
        // the 25 corner rows (y, z) of the block's grid, row y + 5z, two per
        // thread of the block's 16 (one warp half): masks of value <= iso
#pragma unroll
        for (uint32_t h = 0; h < 2; ++h) {
            const uint32_t i = u + 16u * h;
            if (i < 25u) {
                const float* p = &s_vol[j][5u * i];
                uint32_t m = 0;
#pragma unroll
                for (uint32_t x = 0; x < 5; ++x) m |= (p[x] <= iso ? 1u : 0u) << x;
                s_rm[j][i] = (uint8_t)m;
            }
        }
        __syncwarp();
        const uint32_t r0 = ry + 5u * rz;
        // the four cases at once, one byte per cell: s_pair[m] puts bits x and
        // x+1 of a row mask into byte x, s_pair_sw the same pair swapped; the
        // corner order of the case (compute_vertex_values.comp:48-57) is
        // (x,y,z) (x+1,y,z) (x+1,y+1,z) (x,y+1,z), then the same at z+1
        cs4 = s_pair[s_rm[j][r0]] | (s_pair_sw[s_rm[j][r0 + 1u]] << 2) | (s_pair[s_rm[j][r0 + 5u]] << 4) |
              (s_pair_sw[s_rm[j][r0 + 6u]] << 6);
        // cells past the grid (the last one when dims.x is 4) or in rows past it: no case
        cs4 &= row_ok ? (dx == 5u ? 0xffffffffu : 0x00ffffffu) : 0u;
        uint32_t sum = 0;
#pragma unroll
        for (uint32_t x = 0; x < 4; ++x) {
            nv[x] = s_cnt[(cs4 >> (8u * x)) & 255u];
            sum += nv[x];
        }
        return sum;
    };

    // a tile's cases and counts into the emit's tables: one CTA scan gives each
    // thread's first vertex and first rank among the cells with vertices; each
    // such cell sets its start bit, takes its place in s_cells and, for the one
    // 32-vertex word whose first vertex falls in its range (it has at most 15),
    // records the cells starting before that word (s_vmask is zeroed when the
    // tile is claimed).  Returns the tile's vertex count; ends with a barrier.
    auto prep_tile = [&](const uint32_t* nv, const uint32_t cs4, const uint32_t mysum) -> uint32_t {
        const uint32_t ne = (nv[0] != 0u) + (nv[1] != 0u) + (nv[2] != 0u) + (nv[3] != 0u);
        uint32_t tot;
        const uint32_t ex = cta_exclusive_scan<kMcThreads>(mysum | (ne << 16), s_warp, &tot);
        uint32_t run = ex & 0xffffu, rank = ex >> 16;
        *reinterpret_cast<uint32_t*>(&s_case[4u * t]) = cs4;
        if ((t & 15u) == 0u) s_boff[t >> 4] = run;
        if (t == 0) s_vbase[0] = 0;
#pragma unroll
        for (uint32_t x = 0; x < 4; ++x) {
            if (nv[x]) {
                atomicOr(&s_vmask[run >> 5], 1u << (run & 31u));
                s_cells[rank] = (4u * t + x) | (run << 16);
                const uint32_t w = (run + nv[x]) >> 5;
                if ((w << 5) > run && w < (uint32_t)kMcMaskWords) s_vbase[w] = (uint16_t)(rank + 1u);
                ++rank;
            }
            run += nv[x];
        }
        __syncthreads();
        return tot & 0xffffu;
    };

    // the vertices of the tile in shared memory (s_vol, s_case, s_cells,
    // s_vmask, s_vbase, s_id), vertex k of the tile to out[k], out = a.verts + pv
    auto emit_tile = [&](const uint32_t pv, const uint32_t tile_v) {
        uint2* out = a.verts + pv;
        const auto emit = [&](const uint32_t k) {
            // vertex k's cell: the last cell starting at or before k, counted
            // through the start bits of k's word
            const uint32_t w = k >> 5;
            const uint32_t r = s_vbase[w] + (uint32_t)__popc(s_vmask[w] & (0xffffffffu >> (31u - (k & 31u)))) - 1u;
            const uint32_t e = s_cells[r], cell = e & 0xffffu, jb = cell >> 6;
            out[k] = make_uint2(mc_vertex(s_te[s_case[cell]][k - (e >> 16)], cell & 63u, s_vol[jb], s_cp, iso),
                                s_id[jb]);
        };
        if constexpr (kHost) {
            // into host memory, j = k + shift puts each warp's 32 stores in
            // one 256 B-aligned window: stores over the host link run ~20 %
            // faster aligned (device memory gains less than the extra round
            // costs)
            const uint32_t shift = (uint32_t)(reinterpret_cast<uintptr_t>(out) >> 3) & 31u;
            for (uint32_t j = t; j < tile_v + shift; j += kMcThreads)
                if (j >= shift) emit(j - shift);
        } else {
            for (uint32_t k = t; k < tile_v; k += kMcThreads) emit(k);
        }
    };

    // ---- count pass
    for (uint32_t base = start; base < end; base += kMcBlocks) {
        __syncthreads();
        if (t < kMcBlocks) {
            const uint32_t idx = base + t;
            s_id[t] = idx < end ? __ldg(a.active_ids + idx) : 0xffffffffu;
        }
        __syncthreads();
        const uint32_t dims = load_tile();
        uint32_t nv[4], cs4;
        uint32_t bsum = count_cells(dims, nv, cs4);
#pragma unroll
        for (int o = 8; o; o >>= 1) bsum += __shfl_xor_sync(0xffffffffu, bsum, o);
        if (u == 0 && s_id[j] != 0xffffffffu) {
            a.block_counts[base + j] = bsum;
            if (bsum) {
                atomicAdd(&s_cta_v, bsum);
                atomicAdd(&s_cta_b, 1u);
            }
        }
    }
    __syncthreads();
    if (t < 64 && rank < worked) {
        if (t < 32) {
            const uint32_t p = warp_lookback(a.status_v, rank, s_cta_v, epoch, &q->error, 40u);
            if (t == 0) {
                s_pv = p;
                if (rank == worked - 1) q->num_verts = p + s_cta_v;
            }
        } else {
            const uint32_t p = warp_lookback(a.status_b, rank, s_cta_b, epoch, &q->error, 41u);
            if (t == 32) {
                s_pb = p;
                if (rank == worked - 1) q->num_with_verts = p + s_cta_b;
            }
        }
    }
    __syncthreads();
    uint32_t pv = s_pv, pb = s_pb;
    const bool fits = (uint64_t)pv + s_cta_v <= cap;
    if (!fits && t == 0) atomicOr(&q->vert_overflow, 1u);
    if (range <= 2u * kMcBlocks) {
        // short ranges (small queries): each CTA emits its own range, tiles of
        // its next 16 blocks that have vertices (a warp ballot over the counts
        // skips the others); the imbalance costs less here than the barrier
        if (!fits) return;
        const uint32_t lane = t & 31u;
        for (;;) {
            __syncthreads();
            for (uint32_t i = t; i < (uint32_t)kMcMaskWords; i += kMcThreads) s_vmask[i] = 0u;
            if (t < 32) {
                uint32_t cur = s_cursor, filled = 0;
                while (filled < kMcBlocks && cur < end) {
                    const uint32_t i = cur + lane;
                    const uint32_t c = i < end ? a.block_counts[i] : 0u;
                    const uint32_t m = __ballot_sync(0xffffffffu, c != 0u);
                    const uint32_t nz = __popc(m), take = min(nz, kMcBlocks - filled);
                    const uint32_t r = __popc(m & ((1u << lane) - 1u));
                    if (c != 0u && r < take) s_idx[filled + r] = i;
                    if (take < nz) {
                        uint32_t mm = m;
                        for (uint32_t k = 0; k < take; ++k) mm &= mm - 1u;
                        cur += (uint32_t)__ffs(mm) - 1u;
                    } else {
                        cur += 32u;
                    }
                    filled += take;
                }
                __syncwarp();
                if (lane < kMcBlocks) s_id[lane] = lane < filled ? __ldg(a.active_ids + s_idx[lane]) : 0xffffffffu;
                if (lane == 0) {
                    s_stop = filled;
                    s_cursor = min(cur, end);
                }
            }
            __syncthreads();
            const uint32_t n_sel = s_stop;
            if (n_sel == 0) break;
            const uint32_t dims = load_tile();
            uint32_t nv[4], cs4;
            const uint32_t mysum = count_cells(dims, nv, cs4);
            const uint32_t tile_v = prep_tile(nv, cs4, mysum);
            if (t < n_sel) {
                a.with_verts[pb + t] = s_idx[t];
                a.vert_offsets[pb + t] = pv + s_boff[t];
            }
            emit_tile(pv, tile_v);
            pv += tile_v;
            pb += n_sel;
        }
        return;
    }
    // the range's blocks with vertices: their list entries and vertex offsets
    if (fits)
        for (uint32_t b0 = start; b0 < end; b0 += kMcThreads) {
            const uint32_t i = b0 + t;
            const uint32_t c = i < end ? a.block_counts[i] : 0u;  // <= 64 cells x 15 vertices
            uint32_t tot;
            const uint32_t ex = cta_exclusive_scan<kMcThreads>(c | (c ? 1u << 18 : 0u), s_warp, &tot);
            if (c) {
                const uint32_t r = pb + (ex >> 18);
                a.with_verts[r] = i;
                a.vert_offsets[r] = pv + (ex & 0x3ffffu);
            }
            pv += tot & 0x3ffffu;
            pb += tot >> 18;
        }
    // grid barrier (the launch is cooperative: every CTA is resident)
    __syncthreads();
    if (t == 0) {
        __threadfence();
        atomicAdd(&q->mc_arrived, 1u);
        uint32_t spins = 0;
        while (*reinterpret_cast<volatile uint32_t*>(&q->mc_arrived) < G) {
            if (++spins > kSpinLimit) {
                atomicCAS(&q->error, 0u, 42u);
                break;
            }
            if (spins > 8) __nanosleep(100);
        }
        __threadfence();
        s_stop = *reinterpret_cast<volatile uint32_t*>(&q->error) | *reinterpret_cast<volatile uint32_t*>(&q->vert_overflow);
        s_with = *reinterpret_cast<volatile uint32_t*>(&q->num_with_verts);
    }
    __syncthreads();
    if (s_stop) return;
    // emit: tiles of 16 consecutive list entries, claimed by whichever CTA is free
    const uint32_t W = s_with, ntiles = div_up(W, kMcBlocks);
    for (;;) {
        __syncthreads();
        if (t == 0) s_rank = atomicAdd(&q->tiles_emit, 1u);
        for (uint32_t i = t; i < (uint32_t)kMcMaskWords; i += kMcThreads) s_vmask[i] = 0u;
        __syncthreads();
        const uint32_t tile = s_rank;
        if (tile >= ntiles) break;
        const uint32_t first = tile * kMcBlocks;
        if (t < kMcBlocks)
            s_id[t] = first + t < W ? __ldg(a.active_ids + __ldcg(a.with_verts + first + t)) : 0xffffffffu;
        if (t == 0) s_pv = __ldcg(a.vert_offsets + first);
        __syncthreads();
        const uint32_t dims = load_tile();
        uint32_t nv[4], cs4;
        const uint32_t mysum = count_cells(dims, nv, cs4);
        const uint32_t tile_v = prep_tile(nv, cs4, mysum);
        emit_tile(s_pv, tile_v);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int pgrid(bcmc_ctx* ctx, uint32_t tiles, uint32_t per_sm)
{
    const uint32_t r = (uint32_t)ctx->num_sms * per_sm;
    return (int)(tiles < r ? (tiles ? tiles : 1) : r);
}

void query_begin_launch(QueryState* q, float iso, int mc_only, uint32_t capacity, uint32_t vert_capacity,
                        cudaStream_t s, const QueryInputs* in)
{
    k_query_begin<<<1, 256, 0, s>>>(q, iso, mc_only, capacity, vert_capacity, in);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void active_launch(bcmc_ctx* ctx, QueryState* q, const ActiveArgs& a, cudaStream_t s)
{
    // the staged kernel within the 48 KB of dynamic shared memory a launch
    // gets without opting in: 3 windows of kActRTile + 2*NX + 2 bytes
    const uint32_t stage_len = kActRTile + 2u * a.grid.nb.x + 2u;
    if (a.ranges && 3u * stage_len <= 48u * 1024u) {
        k_active_ranges<<<pgrid(ctx, div_up(a.total, kActRTile), 2), kActRThreads, 3u * stage_len, s>>>(q, a,
                                                                                                        stage_len);
        count_launches(1);
        BCMC_CUDA(cudaGetLastError());
        return;
    }
    k_active<<<pgrid(ctx, div_up(a.total, kActiveTile), 8), kActThreads, 0, s>>>(q, a);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void slots_launch(bcmc_ctx* ctx, QueryState* q, const SlotArgs& a, uint32_t max_slots, cudaStream_t s)
{
    k_slots<<<pgrid(ctx, div_up(max_slots, kSlotTile), 8), kActThreads, 0, s>>>(q, a);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void assign_launch(bcmc_ctx* ctx, QueryState* q, const AssignArgs& a, uint32_t max_new, cudaStream_t s)
{
    k_assign<<<pgrid(ctx, div_up(max_new, (uint32_t)kAssignThreads), 16), kAssignThreads, 0, s>>>(q, a);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void decode_new_launch(bcmc_ctx* ctx, const QueryState* q, const DecodeArgs& a, cudaStream_t s)
{
    // two CTAs per SM: the branch it runs on must leave room for the slot
    // selection's CTAs, the critical path beside it
    const size_t smem = zfp_stage_smem(kDecodeNewThreads, a.max_bits / 64u);
    allow_smem(k_decode_new, smem);
    k_decode_new<<<pgrid(ctx, div_up(a.stage_blocks ? a.stage_blocks : 1u, (uint32_t)kDecodeNewThreads), 2),
                   kDecodeNewThreads, smem, s>>>(q, a);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

// CTAs of k_mc resident per SM: the bound of its cooperative grid
static uint32_t mc_per_sm()
{
    static const uint32_t n = [] {
        int a = 0, b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_mc<false>, kMcThreads, 0) != cudaSuccess) a = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_mc<true>, kMcThreads, 0) != cudaSuccess) b = 1;
        const int m = std::min(std::min(a, b), kMcPerSm);
        return (uint32_t)(m > 0 ? m : 1);
    }();
    return n;
}

void mc_launch(bcmc_ctx* ctx, QueryState* q, const McArgs& a, uint32_t max_active, cudaStream_t s)
{
    // cooperative: the kernel's grid barrier needs every CTA resident
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(mc_grid(ctx, max_active));
    cfg.blockDim = dim3(kMcThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeCooperative;
    attr.val.cooperative = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    if (a.host_verts) BCMC_CUDA(cudaLaunchKernelEx(&cfg, k_mc<true>, q, a));
    else BCMC_CUDA(cudaLaunchKernelEx(&cfg, k_mc<false>, q, a));
    count_launches(1);
}

uint32_t active_tiles(uint32_t total) { return div_up(total, kActiveTile); }
uint32_t slot_tiles(uint32_t slots) { return div_up(slots, kSlotTile); }
// one CTA per range of active blocks, every CTA resident
uint32_t mc_grid(bcmc_ctx* ctx, uint32_t max_active)
{
    const uint32_t r = (uint32_t)ctx->num_sms * mc_per_sm(), tiles = div_up(max_active ? max_active : 1, kMcBlocks);
    return tiles < r ? tiles : r;
}

}  // namespace bcmc
