// pipeline.cu -- device side of one isosurface query (computeSurface,
// js/compressed_marching_cubes.js:580-809) and of LRUCache.update
// (js/lru_cache.js:312-843).
//
// The reference runs ~20 dispatches with six host readbacks per query.  Here a
// query is a fixed sequence of launches that read every count from the
// QueryState on the device:
//   k_query_begin  new look-back epoch, counters cleared
//   k_active       active test (compute_block_active.comp) for every block,
//                  fused with the compaction of active ids, the cache lookup
//                  (lru_cache_mark_new_items.comp's "needs caching") and the
//                  compaction of new item ids; the last tile decides the cache
//                  growth (js/lru_cache.js:510-522)
//   k_slots        age/mark/grow of every slot (lru_cache_age_slots.comp,
//                  lru_cache_mark_new_items.comp, lru_cache_init.comp) fused
//                  with the compaction of available slots and their ages
//   sort           available slots by age, oldest first (sort.cu)
//   k_assign       lru_cache_update.comp fused with the ZFP decode of the new
//                  block into its slot (zfp_decompress_block.comp)
//   k_mc           marching cubes count + scan + emit in one pass
//                  (compute_block_has_vertices.comp,
//                  compute_block_voxel_num_verts.comp,
//                  compute_block_vertices.comp)
#include "bcmc_pipeline.h"
#include "zfp_device.cuh"

namespace bcmc {

#define BCMC_TABLE_QUALIFIER __constant__
#include "mc_tables.inc"
#undef BCMC_TABLE_QUALIFIER

// corner i of a cell (compute_vertex_values.comp:48-57), packed x|y<<1|z<<2
__constant__ uint8_t c_corner[8] = {0, 1, 3, 2, 4, 5, 7, 6};
// cube edge -> its two corners (compute_block_vertices.comp:10-23)
__constant__ uint8_t c_edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {6, 5},
                                      {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

__global__ void k_query_begin(QueryState* q, float iso, int mc_only, uint32_t capacity, uint32_t vert_capacity)
{
    const int t = threadIdx.x;
    if (t == 0) {
        q->epoch += 1;
        q->capacity = capacity;
        q->vert_capacity = vert_capacity;
        q->tiles_mc = 0;
        q->error = 0;
        q->vert_overflow = 0;
        q->num_with_verts = 0;
        q->num_verts = 0;
        if (!mc_only) {
            q->isovalue = iso;
            q->tiles_active = q->tiles_slots = q->tiles_sort_hist = 0;
            for (int i = 0; i < 4; ++i) q->tiles_sort[i] = 0;
            q->num_active = q->num_new = q->num_avail = 0;
            q->grow_needed = 0;
        }
    }
    if (!mc_only)
        for (int i = t; i < 1024; i += blockDim.x) (&q->sort_hist[0][0])[i] = 0;
}

// ---------------------------------------------------------------------------
// k_active
// ---------------------------------------------------------------------------
constexpr int kActThreads = 256;
constexpr int kActItems = 8;
constexpr int kActTile = kActThreads * kActItems;

__device__ __forceinline__ uint32_t spad8(uint32_t i) { return i + (i >> 5); }

// compute_block_active.comp:24-61
__device__ __forceinline__ uint32_t block_is_active(const float2* __restrict__ ranges, uint3 nb, uint32_t b,
                                                    float iso)
{
    const float2 r = ranges[b];
    if (iso >= r.x && iso <= r.y) return 1u;
    const int bx = (int)(b % nb.x), by = (int)((b / nb.x) % nb.y), bz = (int)(b / (nb.x * nb.y));
    for (int k = -1; k < 2; ++k)
        for (int j = -1; j < 2; ++j)
            for (int i = -1; i < 2; ++i) {
                const int cx = bx + i, cy = by + j, cz = bz + k;
                if ((i == 0 && j == 0 && k == 0) || cx < 0 || cy < 0 || cz < 0 || cx >= (int)nb.x ||
                    cy >= (int)nb.y || cz >= (int)nb.z)
                    continue;
                const float2 n = ranges[(uint32_t)cx + nb.x * ((uint32_t)cy + nb.y * (uint32_t)cz)];
                const float lo = n.x < r.x ? n.x : r.x;  // GLSL min(range.x, n.x)
                const float hi = r.y < n.y ? n.y : r.y;  // GLSL max(range.y, n.y)
                if (iso >= lo && iso <= hi) return 1u;
            }
    return 0u;
}

__global__ void __launch_bounds__(kActThreads) k_active(QueryState* q, ActiveArgs a)
{
    __shared__ uint8_t s_flags[kActTile + kActTile / 32];
    __shared__ uint32_t s_warp[kActThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_pa, s_pn;
    const uint32_t total = a.total;
    const uint32_t ntiles = div_up(total, kActTile);
    const uint32_t epoch = q->epoch;
    const float iso = q->isovalue;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&q->tiles_active, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t base = tile * kActTile;
#pragma unroll
        for (int j = 0; j < kActItems; ++j) {
            const uint32_t local = j * kActThreads + threadIdx.x;
            const uint32_t b = base + local;
            uint32_t f = 0;
            if (b < total) {
                uint32_t act;
                if (a.ranges) {
                    act = block_is_active(a.ranges, a.nb, b, iso);
                    a.active_out[b] = act;
                } else {
                    act = a.item_needed[b] != 0u ? 1u : 0u;
                }
                const uint32_t need = (act && a.item_slots && a.item_slots[b] < 0) ? 1u : 0u;
                f = act | (need << 1);
            }
            s_flags[spad8(local)] = (uint8_t)f;
        }
        __syncthreads();
        uint32_t cnt = 0;
        uint8_t fl[kActItems];
#pragma unroll
        for (int j = 0; j < kActItems; ++j) {
            fl[j] = s_flags[spad8(threadIdx.x * kActItems + j)];
            cnt += (fl[j] & 1u) | ((uint32_t)(fl[j] >> 1) << 16);
        }
        uint32_t tot;
        const uint32_t excl = cta_exclusive_scan<kActThreads>(cnt, s_warp, &tot);
        if (threadIdx.x == 0) s_pa = lookback_exclusive(a.status_a, tile, tot & 0xffffu, epoch, &q->error, 30u);
        if (threadIdx.x == 32) s_pn = lookback_exclusive(a.status_n, tile, tot >> 16, epoch, &q->error, 31u);
        __syncthreads();
        uint32_t pa = s_pa + (excl & 0xffffu), pn = s_pn + (excl >> 16);
        const uint32_t first = base + threadIdx.x * kActItems;
#pragma unroll
        for (int j = 0; j < kActItems; ++j) {
            if (fl[j] & 1u) {
                if (a.active_ids) a.active_ids[pa] = first + j;
                ++pa;
            }
            if (fl[j] & 2u) {
                if (a.new_ids) a.new_ids[pn] = first + j;
                ++pn;
            }
        }
        if (tile == ntiles - 1 && threadIdx.x == 0) {
            const uint32_t A = s_pa + (tot & 0xffffu), N = s_pn + (tot >> 16);
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
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// k_slots: age + mark + init of new slots, fused with the compaction of the
// available slots (ascending slot id) and their ages.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kActThreads) k_slots(QueryState* q, SlotArgs a)
{
    __shared__ uint8_t s_flags[kActTile + kActTile / 32];
    __shared__ uint32_t s_warp[kActThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_prefix;
    if ((a.skip_when_inactive && q->num_active == 0) || q->grow_needed) return;
    const uint32_t old = q->old_cache_size, nsz = q->new_cache_size;
    const bool compact = q->num_new > 0;
    const uint32_t ntiles = div_up(nsz, kActTile);
    const uint32_t epoch = q->epoch;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&q->tiles_slots, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t base = tile * kActTile;
#pragma unroll
        for (int j = 0; j < kActItems; ++j) {
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
            uint8_t fl[kActItems];
#pragma unroll
            for (int j = 0; j < kActItems; ++j) {
                fl[j] = s_flags[spad8(threadIdx.x * kActItems + j)];
                cnt += fl[j];
            }
            uint32_t tot;
            const uint32_t excl = cta_exclusive_scan<kActThreads>(cnt, s_warp, &tot);
            if (threadIdx.x == 0) s_prefix = lookback_exclusive(a.status, tile, tot, epoch, &q->error, 32u);
            __syncthreads();
            uint32_t p = s_prefix + excl;
            const uint32_t first = base + threadIdx.x * kActItems;
#pragma unroll
            for (int j = 0; j < kActItems; ++j)
                if (fl[j]) {
                    const uint32_t s = first + j;
                    a.avail_ids[p] = s;
                    a.avail_keys[p] = a.slot_age[s];
                    ++p;
                }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// k_assign: lru_cache_update.comp:19-37 (+ decode of the new block into its
// slot when `words` is set).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_assign(QueryState* q, AssignArgs a)
{
    if (q->num_active == 0 || q->grow_needed) return;
    const uint32_t n = q->num_new;
    const uint32_t size = q->new_cache_size;
    const uint32_t* __restrict__ sorted = q->sort_final == 1 ? a.sorted_b : a.sorted_c;
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
        if (a.words) {
            float v[64];
            zfp_decode_block(a.words, (uint64_t)item * a.max_bits, a.max_bits, v);
            float4* d4 = reinterpret_cast<float4*>(a.cache + (uint64_t)slot * 64u);
#pragma unroll
            for (int k = 0; k < 16; ++k) d4[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        }
    }
}

// ---------------------------------------------------------------------------
// k_mc: marching cubes over the active blocks, 4 blocks (256 cells) per tile.
// ---------------------------------------------------------------------------
constexpr int kMcBlocks = 4;
constexpr int kMcThreads = 64 * kMcBlocks;

// ghost voxel positions of a 5^3 block (some coordinate == 4), packed x|y<<4|z<<8
__constant__ uint16_t c_ghost[61] = {
#define G(x, y, z) (uint16_t)((x) | ((y) << 4) | ((z) << 8))
    G(4, 0, 0), G(4, 1, 0), G(4, 2, 0), G(4, 3, 0), G(0, 4, 0), G(1, 4, 0), G(2, 4, 0), G(3, 4, 0), G(4, 4, 0),
    G(4, 0, 1), G(4, 1, 1), G(4, 2, 1), G(4, 3, 1), G(0, 4, 1), G(1, 4, 1), G(2, 4, 1), G(3, 4, 1), G(4, 4, 1),
    G(4, 0, 2), G(4, 1, 2), G(4, 2, 2), G(4, 3, 2), G(0, 4, 2), G(1, 4, 2), G(2, 4, 2), G(3, 4, 2), G(4, 4, 2),
    G(4, 0, 3), G(4, 1, 3), G(4, 2, 3), G(4, 3, 3), G(0, 4, 3), G(1, 4, 3), G(2, 4, 3), G(3, 4, 3), G(4, 4, 3),
    G(0, 0, 4), G(1, 0, 4), G(2, 0, 4), G(3, 0, 4), G(4, 0, 4), G(0, 1, 4), G(1, 1, 4), G(2, 1, 4), G(3, 1, 4),
    G(4, 1, 4), G(0, 2, 4), G(1, 2, 4), G(2, 2, 4), G(3, 2, 4), G(4, 2, 4), G(0, 3, 4), G(1, 3, 4), G(2, 3, 4),
    G(3, 3, 4), G(4, 3, 4), G(0, 4, 4), G(1, 4, 4), G(2, 4, 4), G(3, 4, 4), G(4, 4, 4)
#undef G
};

// compute_vertex_values.comp:96-156: grid extent of the block plus the ghost
// layer taken from active +x/+y/+z neighbours, tested corner, edges, faces.
__device__ __forceinline__ uint32_t block_dims_with_ghost(const uint32_t* __restrict__ active, uint3 nb,
                                                          uint32_t bx, uint32_t by, uint32_t bz)
{
    auto act = [&](uint32_t x, uint32_t y, uint32_t z) { return active[x + nb.x * (y + nb.y * z)] != 0u; };
    uint32_t dx = bx + 1 < nb.x ? 5 : 4, dy = by + 1 < nb.y ? 5 : 4, dz = bz + 1 < nb.z ? 5 : 4;
    if (dx == 5 && dy == 5 && dz == 5 && !act(bx + 1, by + 1, bz + 1)) dx = dy = dz = 4;
    if (dx == 5 && dy == 5 && !act(bx + 1, by + 1, bz)) dx = dy = 4;
    if (dx == 5 && dz == 5 && !act(bx + 1, by, bz + 1)) dx = dz = 4;
    if (dy == 5 && dz == 5 && !act(bx, by + 1, bz + 1)) dy = dz = 4;
    if (dx == 5 && !act(bx + 1, by, bz)) dx = 4;
    if (dy == 5 && !act(bx, by + 1, bz)) dy = 4;
    if (dz == 5 && !act(bx, by, bz + 1)) dz = 4;
    return dx | (dy << 4) | (dz << 8);
}

// block_vertex_position.comp:9-17 with the f32 operations of
// compute_block_vertices.comp:62-74,161-162 in the reference's order, each
// rounded on its own (no contraction).
__device__ __forceinline__ uint32_t quantize(float p)
{
    const float f = __fmul_rn(__fmul_rn(__fsub_rn(p, 0.5f), 0.25f), 1023.0f);
    return __float2uint_rz(f) & 0x3ffu;  // saturating float->uint, as WGSL u32()
}

__global__ void __launch_bounds__(kMcThreads) k_mc(QueryState* q, McArgs a)
{
    __shared__ float s_vol[kMcBlocks][128];
    __shared__ int8_t s_tri[256][16];
    __shared__ uint32_t s_dims[kMcBlocks], s_id[kMcBlocks];
    __shared__ uint32_t s_wsum[kMcThreads / 32];
    __shared__ uint32_t s_tile, s_pv, s_pb;

    const uint32_t A = q->num_active;
    if (A == 0 || q->grow_needed) return;
    const uint32_t ntiles = div_up(A, kMcBlocks);
    const uint32_t epoch = q->epoch;
    const float iso = q->isovalue;
    const uint32_t cap = q->vert_capacity;
    const uint32_t slots = q->cache_size;
    {
        const uint4* src = reinterpret_cast<const uint4*>(&kTriEdges[0][0]);
        uint4* dst = reinterpret_cast<uint4*>(&s_tri[0][0]);
        for (int i = threadIdx.x; i < 256; i += kMcThreads) dst[i] = src[i];
    }
    const uint32_t j = threadIdx.x >> 6, c = threadIdx.x & 63u;
    const uint32_t cx = c & 3u, cy = (c >> 2) & 3u, cz = c >> 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&q->tiles_mc, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t idx = tile * kMcBlocks + j;
        const bool valid = idx < A;
        if (c == 0) {
            uint32_t id = 0, dims = 0;
            if (valid) {
                id = a.active_ids[idx];
                dims = block_dims_with_ghost(a.active, a.nb, id % a.nb.x, (id / a.nb.x) % a.nb.y,
                                             id / (a.nb.x * a.nb.y));
            }
            s_id[j] = id;
            s_dims[j] = dims;
        }
        __syncthreads();
        const uint32_t id = s_id[j], dims = s_dims[j];
        const uint32_t dx = dims & 15u, dy = (dims >> 4) & 15u, dz = dims >> 8;
        if (valid) {
            // every active block is cached; a slot outside the cache would be a
            // logic error, reported instead of read
            const uint32_t slot = (uint32_t)a.item_slots[id];
            if (slot < slots) s_vol[j][cx + 5u * (cy + 5u * cz)] = __ldg(a.cache + (uint64_t)slot * 64u + c);
            else atomicCAS(&q->error, 0u, 51u);
            if (c < 61) {
                const uint32_t g = c_ghost[c];
                const uint32_t gx = g & 15u, gy = (g >> 4) & 15u, gz = g >> 8;
                if (gx < dx && gy < dy && gz < dz) {
                    const uint32_t nid = id + (gx >> 2) + a.nb.x * ((gy >> 2) + a.nb.y * (gz >> 2));
                    const uint32_t nslot = (uint32_t)a.item_slots[nid];
                    if (nslot < slots)
                        s_vol[j][gx + 5u * (gy + 5u * gz)] =
                            __ldg(a.cache + (uint64_t)nslot * 64u + (gx & 3u) + 4u * ((gy & 3u) + 4u * (gz & 3u)));
                    else atomicCAS(&q->error, 0u, 52u);
                }
            }
        }
        __syncthreads();
        // per-cell case and vertex count
        float val[8];
        uint32_t cs = 0, nv = 0;
        if (valid && cx + 1 < dx && cy + 1 < dy && cz + 1 < dz) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const uint32_t o = c_corner[i];
                val[i] = s_vol[j][(cx + (o & 1u)) + 5u * ((cy + ((o >> 1) & 1u)) + 5u * (cz + (o >> 2)))];
                cs |= (val[i] <= iso ? 1u : 0u) << i;
            }
            const int8_t* row = s_tri[cs];
            while (nv < 16 && row[nv] != -1) ++nv;
        }
        // block-local exclusive scan (two warps per block)
        const uint32_t inc = warp_inclusive_scan(nv);
        if (lane == 31) s_wsum[warp] = inc;
        __syncthreads();
        const uint32_t local = inc - nv + ((warp & 1) ? s_wsum[warp - 1] : 0u);
        uint32_t btot[kMcBlocks], boff[kMcBlocks], bwv_rank[kMcBlocks];
        uint32_t tile_v = 0, tile_b = 0;
#pragma unroll
        for (int k = 0; k < kMcBlocks; ++k) {
            btot[k] = s_wsum[2 * k] + s_wsum[2 * k + 1];
            boff[k] = tile_v;
            bwv_rank[k] = tile_b;
            tile_v += btot[k];
            tile_b += btot[k] > 0 ? 1u : 0u;
        }
        if (threadIdx.x == 0) s_pv = lookback_exclusive(a.status_v, tile, tile_v, epoch, &q->error, 40u);
        if (threadIdx.x == 32) s_pb = lookback_exclusive(a.status_b, tile, tile_b, epoch, &q->error, 41u);
        __syncthreads();
        const uint32_t pv = s_pv, pb = s_pb;
        if (tile == ntiles - 1 && threadIdx.x == 0) {
            q->num_verts = pv + tile_v;
            q->num_with_verts = pb + tile_b;
        }
        if (c == 0 && valid && btot[j] > 0 && pb + bwv_rank[j] < A) {
            a.with_verts[pb + bwv_rank[j]] = idx;
            a.vert_offsets[pb + bwv_rank[j]] = pv + boff[j];
        }
        if ((uint64_t)pv + tile_v > cap) {
            if (threadIdx.x == 0) atomicOr(&q->vert_overflow, 1u);
        } else if (nv) {
            uint2* out = a.verts + pv + boff[j] + local;
            const int8_t* row = s_tri[cs];
            const float fx = (float)cx, fy = (float)cy, fz = (float)cz;
            for (uint32_t t = 0; t < nv; ++t) {
                const uint32_t e = (uint32_t)row[t];
                const uint32_t v0 = c_edge[e][0], v1 = c_edge[e][1];
                const float fa = val[v0], fb = val[v1];
                float tt = 0.0f;
                if (!(fabsf(__fsub_rn(fa, fb)) < 0.001f)) tt = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
                const uint32_t o0 = c_corner[v0], o1 = c_corner[v1];
                const int ax = (int)(o0 & 1u), ay = (int)((o0 >> 1) & 1u), az = (int)(o0 >> 2);
                const int bx = (int)(o1 & 1u), by = (int)((o1 >> 1) & 1u), bz = (int)(o1 >> 2);
                const float px = __fadd_rn(__fadd_rn(__fadd_rn((float)ax, __fmul_rn(tt, (float)(bx - ax))), fx), 0.5f);
                const float py = __fadd_rn(__fadd_rn(__fadd_rn((float)ay, __fmul_rn(tt, (float)(by - ay))), fy), 0.5f);
                const float pz = __fadd_rn(__fadd_rn(__fadd_rn((float)az, __fmul_rn(tt, (float)(bz - az))), fz), 0.5f);
                out[t] = make_uint2((quantize(px) << 20) | (quantize(py) << 10) | quantize(pz), id);
            }
        }
        __syncthreads();
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
                        cudaStream_t s)
{
    k_query_begin<<<1, 256, 0, s>>>(q, iso, mc_only, capacity, vert_capacity);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void active_launch(bcmc_ctx* ctx, QueryState* q, const ActiveArgs& a, cudaStream_t s)
{
    k_active<<<pgrid(ctx, div_up(a.total, kActTile), 4), kActThreads, 0, s>>>(q, a);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void slots_launch(bcmc_ctx* ctx, QueryState* q, const SlotArgs& a, uint32_t max_slots, cudaStream_t s)
{
    k_slots<<<pgrid(ctx, div_up(max_slots, kActTile), 4), kActThreads, 0, s>>>(q, a);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void assign_launch(bcmc_ctx* ctx, QueryState* q, const AssignArgs& a, uint32_t max_new, cudaStream_t s)
{
    k_assign<<<pgrid(ctx, div_up(max_new, 128u), 16), 128, 0, s>>>(q, a);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void mc_launch(bcmc_ctx* ctx, QueryState* q, const McArgs& a, uint32_t max_active, cudaStream_t s)
{
    k_mc<<<pgrid(ctx, div_up(max_active, kMcBlocks), 8), kMcThreads, 0, s>>>(q, a);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

uint32_t active_tiles(uint32_t total) { return div_up(total, kActTile); }
uint32_t mc_tiles(uint32_t total) { return div_up(total, kMcBlocks); }

}  // namespace bcmc
