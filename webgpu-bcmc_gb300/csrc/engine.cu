// engine.cu -- batched isosurface queries over several resident volumes with
// one shared pool of decoded-block slots (bcmc_engine_* in include/bcmc.h).
//
// A launch sequence answers up to max_batch (volume, isovalue) queries:
//   k_bbegin   new look-back epoch, counters cleared
//   k_bactive  every query's active test over its volume's blocks, as one
//              stream of 1024-block tiles (query-major).  A tile whose
//              extended value range (its blocks and their 26 neighbours, from
//              volume load) excludes the isovalue is skipped whole.  Active
//              flags go to a per-query bitmap; active (query, block) entries
//              are compacted in query-major, block-ascending order by one
//              decoupled look-back over all tiles; blocks no slot holds are
//              claimed (one claim per block across the batch) and given a
//              slot from the pool's free list
//   k_bdecode  ZFP decode of every claimed block into its slot
//   k_bmc      marching cubes over all entries: the per-query kernel's
//              range-per-CTA count pass, one look-back per CTA, the list of
//              entries with vertices, a grid barrier (cooperative launch) and
//              emit tiles claimed by whichever CTA is free;
//              per-block isovalue, volume and neighbour flags come from the
//              entry's query; every query's vertices come out contiguous and
//              in the plain path's order
//   k_bfinish  per-query vertex offsets and counts
// replayed as one CUDA graph per batch-size bucket.  The host reads the batch
// state once at the end and re-runs only when a capacity was exceeded (entry
// list, slot pool -> eviction of slots the batch does not use, vertex buffer).
#include <algorithm>
#include <map>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "active_test.cuh"
#include "bcmc_impl.h"
#include "mc_common.cuh"
#include "zfp_device.cuh"

namespace bcmc {
namespace {

constexpr int kEngThreads = 256;
constexpr uint32_t kEngTile = 1024;  // blocks per active tile (4 per thread)
// k_bmc tiles: kBlocks active blocks per tile, 16 threads per block (4 cells
// each); 1536 threads per SM resident whatever the tile (6 CTAs of 16 blocks)
constexpr int kBmcThreadsPerSm = 1536;
constexpr int kBmcPerSm = 6;        // CTAs per SM of the default 16-block tile
constexpr int kBmcMaxPerSm = 12;    // of the 8-block tile: sizes the MC look-back status words
constexpr uint32_t kMaxVolumes = 4096;

struct EngVolDev {
    const uint64_t* words;
    const float2* ranges;
    const float2* tile_ext;  // extended range of each 1024-block tile
    int32_t* item_slots;     // slot of each block, -1 none, -2 claimed by this batch
    BlockGrid grid;
    uint32_t total;
    uint32_t max_bits;
};

struct EngQuery {
    uint32_t vol;
    float iso;
    uint32_t tile0;  // first tile of this query in the batch's tile stream
    uint32_t bit0;   // first word of its active bitmap
};

struct EngResult {
    unsigned long long vstart;
    uint32_t nverts;
    uint32_t nactive;
};

// Batch state: written by the host before a sequence (inputs) and by the
// kernels (counters, outputs), read back once at the end.
struct EngState {
    // inputs
    uint32_t nq, ntiles, entry_capacity, use_epoch;
    unsigned long long vert_capacity, vert_base;
    // device-side
    uint32_t epoch, tiles_active, tiles_mc, num_entries;
    uint32_t num_decode, pool_exhausted, entry_overflow, vert_overflow;
    uint32_t error, mc_arrived;  // mc_arrived: k_bmc's grid barrier
    uint32_t tiles_emit, with_verts;  // k_bmc's emit tiles claimed, entries with vertices
    unsigned long long num_verts;  // this sequence's vertices (64-bit, from the per-query totals)
};

// Free list of pool slots: slots free_list[head % cap .. tail % cap) are free.
struct EngPool {
    uint32_t capacity;
    uint32_t head;  // advanced by allocations (may overshoot tail; the host clamps)
    uint32_t tail;  // advanced by evictions
    uint32_t pad;
};

struct BatchArgs {
    const EngVolDev* vols;
    const EngQuery* queries;
    EngResult* results;
    EngState* st;
    EngPool* pool;
    uint32_t* free_list;
    uint32_t* last_use;
    uint32_t* owner_vol;
    uint32_t* owner_block;
    float* cache;
    uint32_t* bitmap;
    uint32_t* ent_id;
    uint32_t* ent_q;
    uint32_t* block_counts;
    uint32_t* wv_list;  // entries with vertices, in entry order (k_bmc)
    uint32_t* wv_off;   // their vertex offsets (32-bit, from vert_base)
    uint32_t* q_nactive;
    uint32_t* q_nverts;
    uint32_t* dec_vol;
    uint32_t* dec_block;
    uint32_t* dec_slot;
    uint2* verts;
    uint64_t* status_a;  // look-back over active tiles
    uint64_t* status_v;  // look-back over MC CTAs (vertices)
    uint64_t* status_b;  // look-back over MC CTAs (entries with vertices)
};

// ---------------------------------------------------------------------------
// volume set-up: extended range of every 1024-block tile
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kEngThreads) k_tile_ext(const float2* __restrict__ ranges, BlockGrid g,
                                                         uint32_t total, float2* __restrict__ ext)
{
    __shared__ float s_lo[kEngThreads / 32], s_hi[kEngThreads / 32];
    const uint32_t tile = blockIdx.x;
    float lo = INFINITY, hi = -INFINITY;
    for (uint32_t i = threadIdx.x; i < kEngTile; i += kEngThreads) {
        const uint32_t b = tile * kEngTile + i;
        if (b >= total) break;
        const uint3 c = block_coords(b, g);
        for (int dz = -1; dz < 2; ++dz)
            for (int dy = -1; dy < 2; ++dy)
                for (int dx = -1; dx < 2; ++dx) {
                    const int x = (int)c.x + dx, y = (int)c.y + dy, z = (int)c.z + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= (int)g.nb.x || y >= (int)g.nb.y || z >= (int)g.nb.z)
                        continue;
                    const float2 r = __ldg(ranges + ((uint32_t)x + g.nb.x * ((uint32_t)y + g.nb.y * (uint32_t)z)));
                    lo = fminf(lo, r.x);  // NaN ranges never make a block active: ignored
                    hi = fmaxf(hi, r.y);
                }
    }
    for (int o = 16; o; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31u) == 0) {
        s_lo[threadIdx.x >> 5] = lo;
        s_hi[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kEngThreads / 32; ++w) {
            lo = fminf(lo, s_lo[w]);
            hi = fmaxf(hi, s_hi[w]);
        }
        ext[tile] = make_float2(lo, hi);
    }
}

// ---------------------------------------------------------------------------
// k_bbegin
// ---------------------------------------------------------------------------
__global__ void k_bbegin(EngState* st, uint32_t* q_nverts, uint32_t* q_nactive, uint32_t nq)
{
    if (threadIdx.x == 0) {
        st->epoch += 1;
        st->tiles_active = st->tiles_mc = st->mc_arrived = st->tiles_emit = st->with_verts = 0;
        st->num_entries = st->num_decode = 0;
        st->pool_exhausted = st->entry_overflow = st->vert_overflow = 0;
        st->error = 0;
        st->num_verts = 0;
    }
    for (uint32_t i = threadIdx.x; i < nq; i += blockDim.x) q_nverts[i] = q_nactive[i] = 0;
}

// ---------------------------------------------------------------------------
// k_bactive
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t find_query(const EngQuery* __restrict__ qs, uint32_t nq, uint32_t tile)
{
    uint32_t lo = 0, hi = nq;  // last q with tile0 <= tile
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&qs[mid].tile0) <= tile) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Claims block b of volume v for this batch and gives it a slot from the free
// list; when the pool has no free slot the claim is released and the batch
// flagged (the host evicts and re-runs).
__device__ __forceinline__ void claim_block(const BatchArgs& a, uint32_t v, int32_t* item_slots, uint32_t b,
                                            uint32_t use_epoch)
{
    if (atomicCAS(item_slots + b, -1, -2) != -1) return;  // cached meanwhile, or claimed by another query
    EngPool* pool = a.pool;
    const uint32_t idx = atomicAdd(&pool->head, 1u);
    const uint32_t tail = *(volatile uint32_t*)&pool->tail;
    if ((int32_t)(idx - tail) >= 0) {  // no free slot: release the claim
        atomicExch(item_slots + b, -1);
        atomicOr(&a.st->pool_exhausted, 1u);
        return;
    }
    const uint32_t slot = a.free_list[idx % pool->capacity];
    a.last_use[slot] = use_epoch;
    const uint32_t d = atomicAdd(&a.st->num_decode, 1u);
    a.dec_vol[d] = v;
    a.dec_block[d] = b;
    a.dec_slot[d] = slot;
}

__global__ void __launch_bounds__(kEngThreads) k_bactive(BatchArgs a)
{
    __shared__ uint32_t s_warp[kEngThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_q, s_p;
    EngState* st = a.st;
    const uint32_t ntiles = st->ntiles, nq = st->nq, epoch = st->epoch, cap = st->entry_capacity;
    const uint32_t use_epoch = st->use_epoch;
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t tile = atomicAdd(&st->tiles_active, 1u);
            s_tile = tile;
            s_q = tile < ntiles ? find_query(a.queries, nq, tile) : 0u;
        }
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t qi = s_q;
        const EngQuery Q = a.queries[qi];
        const EngVolDev& V = a.vols[Q.vol];
        const uint32_t lt = tile - Q.tile0;
        const uint32_t total = V.total;
        const float iso = Q.iso;
        const uint32_t b0 = lt * kEngTile + 4u * threadIdx.x;
        uint32_t act = 0;
        const float2 ext = __ldg(V.tile_ext + lt);
        if (iso >= ext.x && iso <= ext.y && b0 < total) {
            const uint32_t n = min(4u, total - b0);
            const uint3 c = block_coords(b0, V.grid);
            if (n == 4 && c.x + 3 < V.grid.nb.x) {
                act = row4_active(V.ranges, V.grid, c, b0, iso);
            } else {
                for (uint32_t i = 0; i < n; ++i) act |= block_is_active(V.ranges, V.grid, b0 + i, iso) << i;
            }
            // cache lookup: mark use, claim what no slot holds
            for (uint32_t i = 0; i < 4; ++i) {
                if (!(act >> i & 1u)) continue;
                const int32_t s = *(volatile int32_t*)(V.item_slots + b0 + i);
                if (s >= 0) a.last_use[s] = use_epoch;
                else if (s == -1) claim_block(a, Q.vol, V.item_slots, b0 + i, use_epoch);
            }
        }
        // active bitmap: 8 threads (32 blocks) per word
        uint32_t word = act << (4u * (threadIdx.x & 7u));
        word |= __shfl_xor_sync(0xffffffffu, word, 1);
        word |= __shfl_xor_sync(0xffffffffu, word, 2);
        word |= __shfl_xor_sync(0xffffffffu, word, 4);
        if ((threadIdx.x & 7u) == 0) a.bitmap[Q.bit0 + lt * (kEngTile / 32) + (threadIdx.x >> 3)] = word;
        // compaction of (block, query) entries over the whole tile stream
        uint32_t tot;
        const uint32_t excl = cta_exclusive_scan<kEngThreads>((uint32_t)__popc(act), s_warp, &tot);
        if (threadIdx.x < 32) {
            const uint32_t p = warp_lookback(a.status_a, tile, tot, epoch, &st->error, 60u);
            if (threadIdx.x == 0) {
                s_p = p;
                if (tot) atomicAdd(a.q_nactive + qi, tot);
                if (tile == ntiles - 1) {
                    st->num_entries = p + tot;
                    if (p + tot > cap) st->entry_overflow = 1;
                }
            }
        }
        __syncthreads();
        uint32_t pos = s_p + excl;
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) {
            if (act >> i & 1u) {
                if (pos < cap) {
                    a.ent_id[pos] = b0 + i;
                    a.ent_q[pos] = qi;
                }
                ++pos;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// k_bdecode: claimed blocks into their slots, then publish the slot
// ---------------------------------------------------------------------------
// Volumes of a batch differ in rate: the staged words of one CTA are laid out
// at the largest rate of the resident volumes (`max_rate` u64 words per block).

template <int kThreads>
__global__ void __launch_bounds__(kThreads, 640 / kThreads) k_bdecode(BatchArgs a, uint32_t max_rate)
{
    extern __shared__ __align__(16) uint32_t s_words[];
    uint32_t* pl = zfp_stage_planes(s_words, kThreads, max_rate);
    if (threadIdx.x < 4) s_words[kThreads * 2u * max_rate + threadIdx.x] = 0u;
    const uint32_t n = a.st->num_decode;
    for (uint32_t i0 = blockIdx.x * kThreads; i0 < n; i0 += gridDim.x * kThreads) {
        const uint32_t i = i0 + threadIdx.x;
        uint32_t v = 0, b = 0, slot = 0;
        __syncthreads();
        if (i < n) {
            v = a.dec_vol[i];
            b = a.dec_block[i];
            slot = a.dec_slot[i];
            const EngVolDev& V = a.vols[v];
            // this thread's slot of the staged words, at the CTA's stride
            uint2* dst = reinterpret_cast<uint2*>(s_words + threadIdx.x * 2u * max_rate);
            const uint32_t rate = V.max_bits / 64u;
            for (uint32_t k = 0; k < rate; ++k) {
                const uint64_t x = __ldg(V.words + (uint64_t)b * rate + k);
                dst[k] = make_uint2((uint32_t)x, (uint32_t)(x >> 32));
            }
        }
        __syncthreads();
        if (i >= n) continue;
        const EngVolDev& V = a.vols[v];
        float out[64];
        zfp_decode_staged(s_words + threadIdx.x * 2u * max_rate, V.max_bits, pl, out);
        float4* d4 = reinterpret_cast<float4*>(a.cache + (uint64_t)slot * 64u);
#pragma unroll
        for (int k = 0; k < 16; ++k) d4[k] = make_float4(out[4 * k], out[4 * k + 1], out[4 * k + 2], out[4 * k + 3]);
        a.owner_vol[slot] = v;
        a.owner_block[slot] = b;
        V.item_slots[b] = (int32_t)slot;
    }
}

// The autotuner's decode probe: k_bdecode's inner loop into a scratch buffer.
template <int kThreads>
__global__ void __launch_bounds__(kThreads, 640 / kThreads) k_decode_probe(const uint64_t* __restrict__ words, uint32_t rate,
                                                           uint32_t n, float* __restrict__ scratch)
{
    extern __shared__ __align__(16) uint32_t s_words[];
    uint32_t* pl = zfp_stage_planes(s_words, kThreads, rate);
    const uint32_t wb = threadIdx.x & ~31u;
    for (uint32_t i0 = blockIdx.x * kThreads; i0 < n; i0 += gridDim.x * kThreads) {
        const uint32_t nb = n - i0 < (uint32_t)kThreads ? n - i0 : (uint32_t)kThreads;
        __syncthreads();
        zfp_stage_run(words, i0, nb, rate, s_words);
        __syncthreads();
        if (wb >= nb) continue;
        const bool mine = threadIdx.x < nb;
        float out[64];
        if (mine) zfp_decode_staged(s_words + threadIdx.x * 2u * rate, 64u * rate, pl, out);
        zfp_store_warp(pl, out, mine, scratch + (uint64_t)(i0 + wb) * 64u, nb - wb);
    }
}

// ---------------------------------------------------------------------------
// k_bmc: the per-query MC kernel (pipeline.cu, k_mc) over a batch's entries
// ---------------------------------------------------------------------------
template <int kBmcBlocks>
__global__ void __launch_bounds__(16 * kBmcBlocks, kBmcThreadsPerSm / (16 * kBmcBlocks)) k_bmc(BatchArgs a)
{
    constexpr int kBmcThreads = 16 * kBmcBlocks;
    constexpr int kBmcCells = 64 * kBmcBlocks;
    // a block's 5^3 grid; rows 144 floats apart (16 mod 32 banks), so the two
    // blocks of a warp read their corner rows on complementary banks
    __shared__ float s_vol[kBmcBlocks][144];
    __shared__ uint8_t s_rm[kBmcBlocks][32];  // corner-row masks of each block (count_cells)
    __shared__ uint32_t s_pair[32], s_pair_sw[32];  // 5-bit row mask -> per-cell corner pairs
    __shared__ __align__(16) uint16_t s_te[256][16];  // c_tri_edges
    __shared__ __align__(16) uint32_t s_cp[64 * 8];    // c_corner_pack
    __shared__ __align__(16) uint8_t s_cnt[256];
    __shared__ __align__(16) uint8_t s_case[kBmcCells];
    constexpr int kMaskWords = kBmcCells * 15 / 32;  // a tile holds at most 15 vertices per cell
    __shared__ uint32_t s_cells[kBmcCells];    // the tile's cells with vertices in order: cell | first vertex << 16
    __shared__ uint32_t s_vmask[kMaskWords];   // bit k: vertex k of the tile is its cell's first
    __shared__ uint16_t s_vbase[kMaskWords];   // cells with vertices starting before vertex 32w
    __shared__ uint32_t s_id[kBmcBlocks];
    __shared__ uint32_t s_qi[kBmcBlocks];
    __shared__ float s_iso[kBmcBlocks];
    __shared__ uint32_t s_slot[kBmcBlocks][8];
    __shared__ uint32_t s_act[kBmcBlocks];
    __shared__ uint32_t s_warp[kBmcThreads / 32 + 1];
    __shared__ uint32_t s_stop, s_with, s_pv, s_pb, s_cta_v, s_cta_b, s_rank;
    __shared__ uint32_t s_gdesc[64];  // ghost_desc of each ghost voxel
    __shared__ uint8_t s_nb_off[8];

    EngState* st = a.st;
    const uint32_t A = min(st->num_entries, st->entry_capacity);
    if (A == 0 || st->entry_overflow || st->pool_exhausted) return;
    const uint32_t epoch = st->epoch;
    const uint64_t cap = st->vert_capacity, vbase = st->vert_base;
    const uint32_t slots = a.pool->capacity;
    const uint32_t t = threadIdx.x;
    const uint32_t G = gridDim.x;
    if (t == 0) s_rank = atomicAdd(&st->tiles_mc, 1u);
    __syncthreads();
    const uint32_t rank = s_rank;
    const uint32_t range = div_up(div_up(A, G), kBmcBlocks) * kBmcBlocks;
    const uint32_t start = min(A, rank * range), end = min(A, start + range);
    // ranks 0 .. worked - 1 own entries; the others take part in no look-back
    const uint32_t worked = div_up(A, range);
    for (uint32_t i = t; i < 512u; i += kBmcThreads)
        reinterpret_cast<uint4*>(&s_te[0][0])[i] = reinterpret_cast<const uint4*>(&c_tri_edges.e[0][0])[i];
    for (uint32_t i = t; i < 128u; i += kBmcThreads)
        reinterpret_cast<uint4*>(s_cp)[i] = reinterpret_cast<const uint4*>(&c_corner_pack.p[0][0])[i];
    if (t < 16) reinterpret_cast<uint4*>(s_cnt)[t] = reinterpret_cast<const uint4*>(c_tri.count)[t];
    if (t == 0) s_cta_v = s_cta_b = s_pv = s_pb = 0;
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
        if (t < kBmcBlocks * 8) {
            const uint32_t jb = t >> 3, k = t & 7u, id = s_id[jb];
            uint32_t slot = 0xffffffffu, act = 0;
            if (id != 0xffffffffu) {
                const EngQuery* Q = a.queries + s_qi[jb];
                const EngVolDev& V = a.vols[__ldg(&Q->vol)];
                const uint3 nb = V.grid.nb;
                const uint3 bc = block_coords(id, V.grid);
                const uint32_t bx = bc.x, by = bc.y, bz = bc.z;
                if (k == kNbSelf) {
                    slot = (uint32_t)__ldg(V.item_slots + id);
                    act = (bx + 1 < nb.x ? 0x100u : 0u) | (by + 1 < nb.y ? 0x200u : 0u) |
                          (bz + 1 < nb.z ? 0x400u : 0u);
                } else {
                    const uint32_t o = s_nb_off[k], ox = o & 1u, oy = (o >> 1) & 1u, oz = o >> 2;
                    if (bx + ox < nb.x && by + oy < nb.y && bz + oz < nb.z) {
                        const uint32_t nid = id + ox + nb.x * (oy + nb.y * oz);
                        const uint32_t w = __ldg(a.bitmap + __ldg(&Q->bit0) + (nid >> 5));
                        act = (w >> (nid & 31u)) & 1u;
                        slot = (uint32_t)__ldg(V.item_slots + nid);
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
            else atomicCAS(&st->error, 0u, 62u);
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
                            atomicCAS(&st->error, 0u, 63u);
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
        const float iso = s_iso[j];
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

    // ---- count pass
    for (uint32_t base = start; base < end; base += kBmcBlocks) {
        __syncthreads();
        if (t < kBmcBlocks) {
            const uint32_t idx = base + t;
            uint32_t id = 0xffffffffu, qi = 0;
            if (idx < end) {
                id = __ldg(a.ent_id + idx);
                qi = __ldg(a.ent_q + idx);
            }
            s_id[t] = id;
            s_qi[t] = qi;
            s_iso[t] = __ldg(&a.queries[qi].iso);
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
                atomicAdd(a.q_nverts + s_qi[j], bsum);
            }
        }
    }
    __syncthreads();
    if (t < 64 && rank < worked) {
        if (t < 32) {
            const uint32_t p = warp_lookback(a.status_v, rank, s_cta_v, epoch, &st->error, 61u);
            if (t == 0) s_pv = p;
        } else {
            const uint32_t p = warp_lookback(a.status_b, rank, s_cta_b, epoch, &st->error, 64u);
            if (t == 32) {
                s_pb = p;
                if (rank == worked - 1) st->with_verts = p + s_cta_b;
            }
        }
    }
    __syncthreads();
    // 32-bit prefix: a sequence over 2^32 vertices wraps here; k_bfinish
    // detects it from the 64-bit per-query totals and the host splits
    uint32_t pv = s_pv, pb = s_pb;
    const bool fits = vbase + pv + s_cta_v <= cap;
    if (!fits && t == 0) atomicOr(&st->vert_overflow, 1u);
    // the range's entries with vertices: list positions and vertex offsets
    if (fits)
        for (uint32_t b0 = start; b0 < end; b0 += kBmcThreads) {
            const uint32_t i = b0 + t;
            const uint32_t c = i < end ? a.block_counts[i] : 0u;  // <= 64 cells x 15 vertices
            uint32_t tot;
            const uint32_t ex = cta_exclusive_scan<kBmcThreads>(c | (c ? 1u << 18 : 0u), s_warp, &tot);
            if (c) {
                const uint32_t r = pb + (ex >> 18);
                a.wv_list[r] = i;
                a.wv_off[r] = pv + (ex & 0x3ffffu);
            }
            pv += tot & 0x3ffffu;
            pb += tot >> 18;
        }
    // grid barrier (the launch is cooperative: every CTA is resident)
    __syncthreads();
    if (t == 0) {
        __threadfence();
        atomicAdd(&st->mc_arrived, 1u);
        uint32_t spins = 0;
        while (*reinterpret_cast<volatile uint32_t*>(&st->mc_arrived) < G) {
            if (++spins > kSpinLimit) {
                atomicCAS(&st->error, 0u, 65u);
                break;
            }
            if (spins > 8) __nanosleep(100);
        }
        __threadfence();
        s_stop = *reinterpret_cast<volatile uint32_t*>(&st->error) | *reinterpret_cast<volatile uint32_t*>(&st->vert_overflow);
        s_with = *reinterpret_cast<volatile uint32_t*>(&st->with_verts);
    }
    __syncthreads();
    if (s_stop) return;
    // emit: tiles of kBmcBlocks consecutive list entries, claimed by whichever CTA is free
    const uint32_t W = s_with, ntiles = div_up(W, (uint32_t)kBmcBlocks);
    for (;;) {
        __syncthreads();
        if (t == 0) s_rank = atomicAdd(&st->tiles_emit, 1u);
        for (uint32_t i = t; i < (uint32_t)kMaskWords; i += kBmcThreads) s_vmask[i] = 0u;
        __syncthreads();
        const uint32_t tile = s_rank;
        if (tile >= ntiles) break;
        const uint32_t first = tile * kBmcBlocks;
        if (t < kBmcBlocks) {
            uint32_t id = 0xffffffffu, qi = 0;
            if (first + t < W) {
                const uint32_t e = __ldcg(a.wv_list + first + t);
                id = __ldg(a.ent_id + e);
                qi = __ldg(a.ent_q + e);
            }
            s_id[t] = id;
            s_qi[t] = qi;
            s_iso[t] = __ldg(&a.queries[qi].iso);
        }
        if (t == 0) s_pv = __ldcg(a.wv_off + first);
        __syncthreads();
        const uint32_t dims = load_tile();
        uint32_t nv[4], cs4;
        const uint32_t mysum = count_cells(dims, nv, cs4);
        // the emit's tables (as k_mc's prep_tile): each cell with vertices sets
        // its start bit, takes its place in s_cells and records, for the one
        // 32-vertex word whose first vertex falls in its range, the cells
        // starting before that word
        const uint32_t ne = (nv[0] != 0u) + (nv[1] != 0u) + (nv[2] != 0u) + (nv[3] != 0u);
        uint32_t tot;
        const uint32_t ex = cta_exclusive_scan<kBmcThreads>(mysum | (ne << 16), s_warp, &tot);
        const uint32_t tile_v = tot & 0xffffu;
        uint32_t run = ex & 0xffffu, rank = ex >> 16;
        *reinterpret_cast<uint32_t*>(&s_case[4u * t]) = cs4;
        if (t == 0) s_vbase[0] = 0;
#pragma unroll
        for (uint32_t x = 0; x < 4; ++x) {
            if (nv[x]) {
                atomicOr(&s_vmask[run >> 5], 1u << (run & 31u));
                s_cells[rank] = (4u * t + x) | (run << 16);
                const uint32_t w = (run + nv[x]) >> 5;
                if ((w << 5) > run && w < (uint32_t)kMaskWords) s_vbase[w] = (uint16_t)(rank + 1u);
                ++rank;
            }
            run += nv[x];
        }
        __syncthreads();
        uint2* out = a.verts + vbase + s_pv;
        for (uint32_t k = t; k < tile_v; k += kBmcThreads) {
            const uint32_t w = k >> 5;
            const uint32_t r = s_vbase[w] + (uint32_t)__popc(s_vmask[w] & (0xffffffffu >> (31u - (k & 31u)))) - 1u;
            const uint32_t e = s_cells[r], cell = e & 0xffffu, jb = cell >> 6;
            out[k] = make_uint2(mc_vertex(s_te[s_case[cell]][k - (e >> 16)], cell & 63u, s_vol[jb], s_cp, s_iso[jb]),
                                s_id[jb]);
        }
    }
}

// ---------------------------------------------------------------------------
// k_bfinish: per-query results (one CTA; queries in order)
// ---------------------------------------------------------------------------
constexpr int kFinThreads = 1024;
__global__ void __launch_bounds__(kFinThreads) k_bfinish(BatchArgs a)
{
    __shared__ unsigned long long s_sum[kFinThreads / 32 + 1];
    EngState* st = a.st;
    const uint32_t nq = st->nq;
    const uint64_t vbase = st->vert_base;
    unsigned long long carry = 0;
    for (uint32_t b0 = 0; b0 < nq; b0 += kFinThreads) {
        const uint32_t i = b0 + threadIdx.x;
        const unsigned long long v = i < nq ? a.q_nverts[i] : 0ull;
        // inclusive scan in 64 bits: warp shuffles, then the warp totals
        unsigned long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31u) >= (uint32_t)o) x += y;
        }
        if ((threadIdx.x & 31u) == 31u) s_sum[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long r = 0;
            for (int w = 0; w < kFinThreads / 32; ++w) {
                const unsigned long long tw = s_sum[w];
                s_sum[w] = r;
                r += tw;
            }
            s_sum[kFinThreads / 32] = r;
        }
        __syncthreads();
        const unsigned long long excl = carry + s_sum[threadIdx.x >> 5] + x - v;
        if (i < nq) {
            EngResult r;
            r.vstart = vbase + excl;
            r.nverts = (uint32_t)v;
            r.nactive = a.q_nactive[i];
            a.results[i] = r;
        }
        carry += s_sum[kFinThreads / 32];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        st->num_verts = carry;
        if (vbase + carry > st->vert_capacity || carry >= (1ull << 32)) st->vert_overflow = 1;
    }
}

// ---------------------------------------------------------------------------
// k_bevict: free every slot the current batch does not use
// ---------------------------------------------------------------------------
__global__ void k_bevict(BatchArgs a, uint32_t use_epoch, uint32_t nslots, unsigned long long* evicted)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < nslots; s += gridDim.x * blockDim.x) {
        const uint32_t v = a.owner_vol[s];
        if (v == 0xffffffffu || a.last_use[s] == use_epoch) continue;
        a.vols[v].item_slots[a.owner_block[s]] = -1;
        a.owner_vol[s] = 0xffffffffu;
        const uint32_t pos = atomicAdd(&a.pool->tail, 1u);
        a.free_list[pos % a.pool->capacity] = s;
        atomicAdd(evicted, 1ull);
    }
}

__global__ void k_fill_u32(uint32_t* p, uint64_t n, uint32_t v)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}
__global__ void k_iota(uint32_t* p, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

}  // namespace
}  // namespace bcmc

using namespace bcmc;

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct EngVolume {
    uint32_t dims[3];
    uint32_t rate;
    uint64_t* words = nullptr;
    size_t words_bytes = 0;
    float2* ranges = nullptr;
    float2* tile_ext = nullptr;
    int32_t* item_slots = nullptr;
    uint32_t total = 0, tiles = 0;
    BlockGrid grid;
};

// Launch parameters the autotuner chooses per batch-size bucket (the kernels'
// tile shapes are compile-time; these are the runtime knobs).
struct EngConfig {
    int act_per_sm = 8;      // k_bactive CTAs per SM
    int dec_threads = 128;   // k_bdecode threads per CTA (64, 128, 256)
    int dec_per_sm = 16;     // k_bdecode CTAs per SM
    int mc_per_sm = kBmcPerSm;  // k_bmc CTAs per SM of the 16-block tile (<= its residency, 6); scaled
                                // by 16 / mc_blocks for the other tiles
    int mc_blocks = 16;         // k_bmc active blocks per tile (8, 16, 32)
};

// The buffers of one batch in flight.  Two lanes let the server keep two
// batches on the device at once: the next batch's active test, claims and
// decode (phase 1) run while the current batch's marching cubes (phase 2) do.
struct EngLane {
    bool ready = false;  // buffers allocated
    EngQuery* d_queries = nullptr;
    EngQuery* h_queries = nullptr;  // pinned
    EngResult* d_results = nullptr;
    EngResult* h_results = nullptr;  // pinned
    EngState* d_st = nullptr;
    EngState* h_st = nullptr;  // pinned
    uint32_t *q_nactive = nullptr, *q_nverts = nullptr;
    uint32_t* bitmap = nullptr;
    uint64_t bitmap_words = 0;
    uint32_t *ent_id = nullptr, *ent_q = nullptr, *block_counts = nullptr, *wv_list = nullptr, *wv_off = nullptr;
    uint32_t entry_cap = 0;
    uint2* verts = nullptr;
    uint64_t vert_cap = 0, vert_used = 0;
    uint64_t* status = nullptr;
    uint64_t status_words = 0;
    uint64_t status_a_words = 0;
    uint64_t epoch_calls = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // one graph per batch-size bucket, rebuilt when buffers move
    struct Graph {
        cudaGraphExec_t exec = nullptr;        // the whole sequence on one stream
        cudaGraphExec_t front = nullptr;       // phase 1 (pipelined runs)
        cudaGraphExec_t back = nullptr;        // phase 2 (pipelined runs)
        uint64_t generation = 0, split_generation = 0;
        int cfg_key = -1, split_cfg_key = -1;  // the launch parameters they were captured with
    };
    std::map<uint32_t, Graph> graphs;
    uint64_t generation = 1;
    // pipelined batch in flight on this lane
    cudaEvent_t ev_front = nullptr;  // its phase 1 finished
    cudaEvent_t ev_done = nullptr;   // its phase 2 and the state copies finished
    bool in_flight = false;
    uint32_t batch_epoch = 0;        // use epoch of its sequence (protected from eviction)
    uint32_t n = 0, bucket = 0;
    std::vector<bcmc_query> queries;
};

struct bcmc_engine {
    bcmc_ctx* ctx = nullptr;
    cudaStream_t stream = nullptr;       // every synchronous run; phase 1 of pipelined runs
    cudaStream_t stream_back = nullptr;  // phase 2 of pipelined runs
    cudaStream_t stream_copy = nullptr;  // vertex copies of completed pipelined batches
    bcmc_engine_opts opts{};
    std::vector<EngVolume> vols;
    EngVolDev* d_vols = nullptr;
    uint32_t d_vols_cap = 0;
    // pool
    uint64_t pool_slots = 0;
    float* cache = nullptr;
    uint32_t *free_list = nullptr, *last_use = nullptr, *owner_vol = nullptr, *owner_block = nullptr;
    EngPool* d_pool = nullptr;
    EngPool* h_pool = nullptr;
    unsigned long long* d_evicted = nullptr;
    // the decode list of a sequence's claims: written and read in phase 1 only,
    // which runs one batch at a time, so both lanes share it
    uint32_t *dec_vol = nullptr, *dec_block = nullptr, *dec_slot = nullptr;
    uint32_t dec_cap = 0;
    uint32_t max_batch = 0;
    uint32_t max_rate = 1;  // largest rate of the resident volumes (k_bdecode's staging stride)
    uint32_t use_epoch = 0;
    EngLane lanes[2];
    EngLane* L = &lanes[0];  // the lane the next sequence runs on, and whose vertices the API returns
    std::map<uint32_t, EngConfig> tuned;  // per bucket
    EngConfig cfg;                        // of the sequence being enqueued
    bcmc_engine_stats stats{};
    uint64_t overlapped = 0;  // pipelined batches launched while another was in flight
};

namespace {

int eng_grid_mc_max(bcmc_engine* e) { return e->ctx->num_sms * kBmcMaxPerSm; }  // sizes the status words
// k_bmc<kB> CTAs resident per SM: the bound of its cooperative grid
template <int kB>
int bmc_resident()
{
    static const int n = [] {
        int r = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_bmc<kB>, 16 * kB, 0) != cudaSuccess || r < 1) r = 1;
        return r;
    }();
    return n;
}
int eng_grid_mc(bcmc_engine* e)
{
    const int kb = e->cfg.mc_blocks;
    const int resident = kb == 8 ? bmc_resident<8>() : (kb == 32 ? bmc_resident<32>() : bmc_resident<16>());
    const int per_sm = std::min(std::min(e->cfg.mc_per_sm, kBmcPerSm) * 16 / kb, resident);
    return e->ctx->num_sms * std::max(per_sm, 1);
}
int eng_grid_act(bcmc_engine* e) { return e->ctx->num_sms * e->cfg.act_per_sm; }
int eng_grid_dec(bcmc_engine* e) { return e->ctx->num_sms * e->cfg.dec_per_sm; }

template <typename T>
void eng_realloc(bcmc_engine* e, T*& p, uint64_t old_n, uint64_t new_n)
{
    dev_free(e->ctx, p, old_n * sizeof(T));
    p = nullptr;
    p = (T*)dev_alloc(e->ctx, new_n * sizeof(T));
}

BatchArgs eng_args(bcmc_engine* e)
{
    BatchArgs a;
    a.vols = e->d_vols;
    a.queries = e->L->d_queries;
    a.results = e->L->d_results;
    a.st = e->L->d_st;
    a.pool = e->d_pool;
    a.free_list = e->free_list;
    a.last_use = e->last_use;
    a.owner_vol = e->owner_vol;
    a.owner_block = e->owner_block;
    a.cache = e->cache;
    a.bitmap = e->L->bitmap;
    a.ent_id = e->L->ent_id;
    a.ent_q = e->L->ent_q;
    a.block_counts = e->L->block_counts;
    a.wv_list = e->L->wv_list;
    a.wv_off = e->L->wv_off;
    a.q_nactive = e->L->q_nactive;
    a.q_nverts = e->L->q_nverts;
    a.dec_vol = e->dec_vol;
    a.dec_block = e->dec_block;
    a.dec_slot = e->dec_slot;
    a.verts = e->L->verts;
    a.status_a = e->L->status;
    a.status_v = e->L->status + e->L->status_a_words;
    a.status_b = a.status_v + eng_grid_mc_max(e) + 1;
    return a;
}

void eng_ensure_status(bcmc_engine* e, uint64_t active_tiles)
{
    const uint64_t need_a = std::max<uint64_t>(active_tiles + 1, 1024);
    const uint64_t mc_words = 2 * ((uint64_t)eng_grid_mc_max(e) + 1);  // status_v, status_b
    const uint64_t need = need_a + mc_words;
    if (need_a <= e->L->status_a_words && need <= e->L->status_words) return;
    BCMC_CUDA(cudaStreamSynchronize(e->stream));
    const uint64_t words = std::max<uint64_t>(need_a * 2, 4096) + mc_words;
    eng_realloc(e, e->L->status, e->L->status_words, words);
    BCMC_CUDA(cudaMemsetAsync(e->L->status, 0, words * 8, e->stream));
    e->L->status_words = words;
    e->L->status_a_words = words - mc_words;
    ++e->L->generation;
}

// Every 2^26 sequences the look-back epoch restarts over cleared status words.
void eng_epoch_tick(bcmc_engine* e)
{
    if (++e->L->epoch_calls < (1ull << 26)) return;
    BCMC_CUDA(cudaMemsetAsync(e->L->status, 0, e->L->status_words * 8, e->stream));
    BCMC_CUDA(cudaMemsetAsync(&e->L->d_st->epoch, 0, 4, e->stream));
    e->L->epoch_calls = 0;
}

void eng_upload_vols(bcmc_engine* e)
{
    const uint32_t n = (uint32_t)e->vols.size();
    if (n > e->d_vols_cap) {
        eng_realloc(e, e->d_vols, e->d_vols_cap, std::max<uint32_t>(n * 2, 8));
        e->d_vols_cap = std::max<uint32_t>(n * 2, 8);
        for (EngLane& l : e->lanes) ++l.generation;
    }
    std::vector<EngVolDev> h(n);
    for (uint32_t i = 0; i < n; ++i) {
        const EngVolume& v = e->vols[i];
        h[i] = EngVolDev{v.words, v.ranges, v.tile_ext, v.item_slots, v.grid, v.total, 64u * v.rate};
    }
    BCMC_CUDA(cudaMemcpyAsync(e->d_vols, h.data(), n * sizeof(EngVolDev), cudaMemcpyHostToDevice, e->stream));
    BCMC_CUDA(cudaStreamSynchronize(e->stream));
}

void eng_alloc_pool(bcmc_engine* e, uint64_t slots)
{
    if (slots == 0 || slots > 0xffffffffull) throw std::invalid_argument("pool_slots out of range");
    e->pool_slots = slots;
    e->cache = (float*)dev_alloc(e->ctx, slots * 256);
    e->free_list = (uint32_t*)dev_alloc(e->ctx, slots * 4);
    e->last_use = (uint32_t*)dev_alloc(e->ctx, slots * 4);
    e->owner_vol = (uint32_t*)dev_alloc(e->ctx, slots * 4);
    e->owner_block = (uint32_t*)dev_alloc(e->ctx, slots * 4);
    // every successful claim of a batch takes a free slot: the decode list
    // never needs more entries than the pool has slots
    e->dec_vol = (uint32_t*)dev_alloc(e->ctx, slots * 4);
    e->dec_block = (uint32_t*)dev_alloc(e->ctx, slots * 4);
    e->dec_slot = (uint32_t*)dev_alloc(e->ctx, slots * 4);
    e->dec_cap = (uint32_t)slots;
    const int grid = e->ctx->num_sms * 8;
    k_iota<<<grid, 256, 0, e->stream>>>(e->free_list, (uint32_t)slots);
    k_fill_u32<<<grid, 256, 0, e->stream>>>(e->owner_vol, slots, 0xffffffffu);
    k_fill_u32<<<grid, 256, 0, e->stream>>>(e->last_use, slots, 0u);
    count_launches(3);
    e->h_pool->capacity = (uint32_t)slots;
    e->h_pool->head = 0;
    e->h_pool->tail = (uint32_t)slots;
    BCMC_CUDA(cudaMemcpyAsync(e->d_pool, e->h_pool, sizeof(EngPool), cudaMemcpyHostToDevice, e->stream));
    BCMC_CUDA(cudaStreamSynchronize(e->stream));
    for (EngLane& l : e->lanes) ++l.generation;
}

void eng_ensure_batch(bcmc_engine* e, uint64_t bitmap_words, uint32_t entries)
{
    if (bitmap_words > e->L->bitmap_words) {
        BCMC_CUDA(cudaStreamSynchronize(e->stream));
        const uint64_t n = std::max<uint64_t>(bitmap_words + bitmap_words / 2, 1u << 16);
        eng_realloc(e, e->L->bitmap, e->L->bitmap_words, n);
        e->L->bitmap_words = n;
        ++e->L->generation;
    }
    if (entries > e->L->entry_cap) {
        BCMC_CUDA(cudaStreamSynchronize(e->stream));
        const uint64_t n64 = std::min<uint64_t>((uint64_t)entries + entries / 2, 0xffffffffull);
        const uint32_t n = (uint32_t)std::max<uint64_t>(n64, 1u << 16);
        eng_realloc(e, e->L->ent_id, e->L->entry_cap, n);
        eng_realloc(e, e->L->ent_q, e->L->entry_cap, n);
        eng_realloc(e, e->L->block_counts, e->L->entry_cap, n);
        eng_realloc(e, e->L->wv_list, e->L->entry_cap, n);
        eng_realloc(e, e->L->wv_off, e->L->entry_cap, n);
        e->L->entry_cap = n;
        ++e->L->generation;
    }
}

void eng_ensure_verts(bcmc_engine* e, uint64_t need)
{
    if (need <= e->L->vert_cap) return;
    BCMC_CUDA(cudaStreamSynchronize(e->stream));
    uint64_t n = std::max<uint64_t>(need + need / 2, 1u << 20);
    if (e->opts.vertex_budget) n = std::max<uint64_t>(need, std::min<uint64_t>(n, e->opts.vertex_budget));
    // keep the vertices already written by earlier sequences of this run
    uint2* nv = (uint2*)dev_alloc(e->ctx, n * sizeof(uint2));
    if (e->L->vert_used)
        BCMC_CUDA(cudaMemcpyAsync(nv, e->L->verts, e->L->vert_used * sizeof(uint2), cudaMemcpyDeviceToDevice, e->stream));
    BCMC_CUDA(cudaStreamSynchronize(e->stream));
    dev_free(e->ctx, e->L->verts, e->L->vert_cap * sizeof(uint2));
    e->L->verts = nv;
    e->L->vert_cap = n;
    ++e->L->generation;
}

// Allocates lane k's buffers (lane 0 at creation; lane 1 on the first
// pipelined run) and makes k the current lane.
void eng_lane_init(bcmc_engine* e, int k)
{
    EngLane& l = e->lanes[k];
    e->L = &l;
    if (l.ready) return;
    bcmc_ctx* ctx = e->ctx;
    BCMC_CUDA(cudaEventCreate(&l.ev0));
    BCMC_CUDA(cudaEventCreate(&l.ev1));
    BCMC_CUDA(cudaEventCreateWithFlags(&l.ev_front, cudaEventDisableTiming));
    BCMC_CUDA(cudaEventCreateWithFlags(&l.ev_done, cudaEventDisableTiming));
    BCMC_CUDA(cudaMallocHost(&l.h_queries, e->max_batch * sizeof(EngQuery)));
    BCMC_CUDA(cudaMallocHost(&l.h_results, e->max_batch * sizeof(EngResult)));
    BCMC_CUDA(cudaMallocHost(&l.h_st, sizeof(EngState)));
    memset(l.h_st, 0, sizeof(EngState));
    l.d_queries = (EngQuery*)dev_alloc(ctx, e->max_batch * sizeof(EngQuery));
    l.d_results = (EngResult*)dev_alloc(ctx, e->max_batch * sizeof(EngResult));
    l.d_st = (EngState*)dev_alloc(ctx, sizeof(EngState));
    BCMC_CUDA(cudaMemsetAsync(l.d_st, 0, sizeof(EngState), e->stream));
    l.q_nactive = (uint32_t*)dev_alloc(ctx, e->max_batch * 4);
    l.q_nverts = (uint32_t*)dev_alloc(ctx, e->max_batch * 4);
    l.ready = true;
    // with a vertex budget the buffer is sized for it once, up front
    eng_ensure_verts(e, e->opts.vertex_budget ? e->opts.vertex_budget
                                              : (e->opts.vertex_capacity ? e->opts.vertex_capacity : (1ull << 24)));
    eng_ensure_status(e, 1024);
    eng_ensure_batch(e, 1u << 16, 1u << 16);
    BCMC_CUDA(cudaStreamSynchronize(e->stream));
}

void eng_lane_free(bcmc_engine* e, EngLane& l)
{
    bcmc_ctx* ctx = e->ctx;
    for (auto& kv : l.graphs) {
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        if (kv.second.front) cudaGraphExecDestroy(kv.second.front);
        if (kv.second.back) cudaGraphExecDestroy(kv.second.back);
    }
    l.graphs.clear();
    dev_free(ctx, l.d_queries, e->max_batch * sizeof(EngQuery));
    dev_free(ctx, l.d_results, e->max_batch * sizeof(EngResult));
    dev_free(ctx, l.d_st, sizeof(EngState));
    dev_free(ctx, l.q_nactive, e->max_batch * 4);
    dev_free(ctx, l.q_nverts, e->max_batch * 4);
    dev_free(ctx, l.bitmap, l.bitmap_words * 4);
    dev_free(ctx, l.ent_id, (size_t)l.entry_cap * 4);
    dev_free(ctx, l.ent_q, (size_t)l.entry_cap * 4);
    dev_free(ctx, l.block_counts, (size_t)l.entry_cap * 4);
    dev_free(ctx, l.wv_list, (size_t)l.entry_cap * 4);
    dev_free(ctx, l.wv_off, (size_t)l.entry_cap * 4);
    dev_free(ctx, l.verts, l.vert_cap * sizeof(uint2));
    dev_free(ctx, l.status, l.status_words * 8);
    if (l.h_queries) cudaFreeHost(l.h_queries);
    if (l.h_results) cudaFreeHost(l.h_results);
    if (l.h_st) cudaFreeHost(l.h_st);
    if (l.ev0) cudaEventDestroy(l.ev0);
    if (l.ev1) cudaEventDestroy(l.ev1);
    if (l.ev_front) cudaEventDestroy(l.ev_front);
    if (l.ev_done) cudaEventDestroy(l.ev_done);
    l = EngLane{};
}

// The launch sequence of one batch (also what a graph captures).
// Phase 1 of a batch: inputs in, active test, claims, decode of the claimed
// blocks into their slots.
void eng_enqueue_front(bcmc_engine* e, uint32_t bucket, cudaStream_t s)
{
    const BatchArgs a = eng_args(e);
    BCMC_CUDA(cudaMemcpyAsync(e->L->d_queries, e->L->h_queries, bucket * sizeof(EngQuery), cudaMemcpyHostToDevice, s));
    BCMC_CUDA(cudaMemcpyAsync(e->L->d_st, e->L->h_st, offsetof(EngState, epoch), cudaMemcpyHostToDevice, s));
    BCMC_CUDA(cudaEventRecordWithFlags(e->L->ev0, s, cudaEventRecordExternal));
    k_bbegin<<<1, 1024, 0, s>>>(e->L->d_st, e->L->q_nverts, e->L->q_nactive, bucket);
    k_bactive<<<eng_grid_act(e), kEngThreads, 0, s>>>(a);
    const uint32_t r = e->max_rate;
    if (e->cfg.dec_threads == 64) {
        const size_t smem = zfp_stage_smem(64, r);
        allow_smem(k_bdecode<64>, smem);
        k_bdecode<64><<<eng_grid_dec(e), 64, smem, s>>>(a, r);
    } else if (e->cfg.dec_threads == 256) {
        const size_t smem = zfp_stage_smem(256, r);
        allow_smem(k_bdecode<256>, smem);
        k_bdecode<256><<<eng_grid_dec(e), 256, smem, s>>>(a, r);
    } else {
        const size_t smem = zfp_stage_smem(128, r);
        allow_smem(k_bdecode<128>, smem);
        k_bdecode<128><<<eng_grid_dec(e), 128, smem, s>>>(a, r);
    }
    count_launches(3);
    BCMC_CUDA(cudaGetLastError());
}

// Phase 2: marching cubes over the batch's entries, per-query results, state out.
void eng_enqueue_back(bcmc_engine* e, uint32_t bucket, cudaStream_t s)
{
    const BatchArgs a = eng_args(e);
    // cooperative: k_bmc's grid barrier needs every CTA resident
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(eng_grid_mc(e));
    cfg.blockDim = dim3(16 * e->cfg.mc_blocks);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeCooperative;
    attr.val.cooperative = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    if (e->cfg.mc_blocks == 8) BCMC_CUDA(cudaLaunchKernelEx(&cfg, k_bmc<8>, a));
    else if (e->cfg.mc_blocks == 32) BCMC_CUDA(cudaLaunchKernelEx(&cfg, k_bmc<32>, a));
    else BCMC_CUDA(cudaLaunchKernelEx(&cfg, k_bmc<16>, a));
    k_bfinish<<<1, kFinThreads, 0, s>>>(a);
    count_launches(2);
    BCMC_CUDA(cudaGetLastError());
    BCMC_CUDA(cudaEventRecordWithFlags(e->L->ev1, s, cudaEventRecordExternal));
    BCMC_CUDA(cudaMemcpyAsync(e->L->h_st, e->L->d_st, sizeof(EngState), cudaMemcpyDeviceToHost, s));
    BCMC_CUDA(cudaMemcpyAsync(e->L->h_results, e->L->d_results, bucket * sizeof(EngResult), cudaMemcpyDeviceToHost, s));
}

// The launch sequence of one batch on one stream (also what a graph captures).
void eng_enqueue(bcmc_engine* e, uint32_t bucket)
{
    eng_enqueue_front(e, bucket, e->stream);
    eng_enqueue_back(e, bucket, e->stream);
}

int eng_cfg_key(const EngConfig& c)
{
    const int log_blocks = c.mc_blocks == 8 ? 3 : (c.mc_blocks == 32 ? 5 : 4);
    return c.act_per_sm | (c.dec_threads << 8) | (c.dec_per_sm << 18) | (c.mc_per_sm << 24) | (log_blocks << 27);
}

// Captures what `enqueue` issues on stream s into a graph.
template <typename F>
cudaGraphExec_t eng_capture(cudaStream_t s, F&& enqueue)
{
    cudaGraph_t graph = nullptr;
    const uint64_t before = g_kernel_launches.load();
    BCMC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
        enqueue();
    } catch (...) {
        cudaStreamEndCapture(s, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
    }
    BCMC_CUDA(cudaStreamEndCapture(s, &graph));
    g_kernel_launches.store(before);  // captured, not launched
    cudaGraphExec_t exec = nullptr;
    const cudaError_t err = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    BCMC_CUDA(err);
    return exec;
}

void eng_launch(bcmc_engine* e, uint32_t bucket)
{
    auto it = e->tuned.find(bucket);
    e->cfg = it != e->tuned.end() ? it->second : EngConfig{};
    auto& g = e->L->graphs[bucket];
    const int key = eng_cfg_key(e->cfg);
    if (!g.exec || g.generation != e->L->generation || g.cfg_key != key) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        g.exec = eng_capture(e->stream, [&] { eng_enqueue(e, bucket); });
        g.generation = e->L->generation;
        g.cfg_key = key;
    }
    BCMC_CUDA(cudaGraphLaunch(g.exec, e->stream));
    count_launches(5);
}

// Pipelined launch: phase 1 on the front stream, phase 2 on the back stream
// after it.  The next batch's phase 1 (front stream) can then run while this
// batch's phase 2 does.
void eng_launch_split(bcmc_engine* e, uint32_t bucket)
{
    auto it = e->tuned.find(bucket);
    e->cfg = it != e->tuned.end() ? it->second : EngConfig{};
    auto& g = e->L->graphs[bucket];
    const int key = eng_cfg_key(e->cfg);
    if (!g.front || g.split_generation != e->L->generation || g.split_cfg_key != key) {
        if (g.front) cudaGraphExecDestroy(g.front);
        if (g.back) cudaGraphExecDestroy(g.back);
        g.front = g.back = nullptr;
        g.front = eng_capture(e->stream, [&] { eng_enqueue_front(e, bucket, e->stream); });
        g.back = eng_capture(e->stream_back, [&] { eng_enqueue_back(e, bucket, e->stream_back); });
        g.split_generation = e->L->generation;
        g.split_cfg_key = key;
    }
    BCMC_CUDA(cudaGraphLaunch(g.front, e->stream));
    BCMC_CUDA(cudaEventRecord(e->L->ev_front, e->stream));
    BCMC_CUDA(cudaStreamWaitEvent(e->stream_back, e->L->ev_front, 0));
    BCMC_CUDA(cudaGraphLaunch(g.back, e->stream_back));
    count_launches(5);
}

uint32_t bucket_of(uint32_t n)
{
    uint32_t b = 1;
    while (b < n) b <<= 1;
    return b;
}

// Refusal of a launch sequence by the vertex budget: only its first `fit`
// queries fit (their counts are known from the count pass).
struct AdmitPrefix : std::length_error {
    uint32_t fit;
    explicit AdmitPrefix(uint32_t f) : std::length_error("batch above the vertex budget"), fit(f) {}
};

// Runs queries[0..n) (n <= max_batch) as one launch sequence; results go to out.
// Throws std::length_error when the pool cannot hold the sequence's active blocks.
struct SeqShape {
    uint32_t bucket;
    uint64_t tiles, words;
};

// The current lane's query table for queries[0..n), padded to the batch-size
// bucket, and its buffers sized for it.
SeqShape eng_prepare(bcmc_engine* e, const bcmc_query* queries, uint32_t n)
{
    SeqShape sh{std::min(bucket_of(n), e->max_batch), 0, 0};
    for (uint32_t i = 0; i < sh.bucket; ++i) {
        EngQuery q{};
        if (i < n) {
            if (queries[i].volume >= e->vols.size()) throw std::invalid_argument("unknown volume id");
            const EngVolume& v = e->vols[queries[i].volume];
            q.vol = queries[i].volume;
            q.iso = queries[i].isovalue;
            q.tile0 = (uint32_t)sh.tiles;
            q.bit0 = (uint32_t)sh.words;
            sh.tiles += v.tiles;
            sh.words += (uint64_t)v.tiles * (kEngTile / 32);
        } else {  // padding queries of the bucket: no tiles
            q.vol = 0;
            q.iso = 0.0f;
            q.tile0 = (uint32_t)sh.tiles;
            q.bit0 = (uint32_t)sh.words;
        }
        e->L->h_queries[i] = q;
    }
    if (sh.tiles >= 0xffffffffull || sh.words >= 0xffffffffull) throw std::invalid_argument("batch too large");
    eng_ensure_status(e, sh.tiles);
    eng_ensure_batch(e, sh.words, std::max<uint32_t>(e->L->entry_cap, 1u << 16));
    return sh;
}

// The current lane's batch inputs for one launch of the sequence.
void eng_set_inputs(bcmc_engine* e, const SeqShape& sh)
{
    EngState& st = *e->L->h_st;
    st.nq = sh.bucket;
    st.ntiles = (uint32_t)sh.tiles;
    st.entry_capacity = e->L->entry_cap;
    st.use_epoch = e->use_epoch;
    st.vert_capacity = e->L->vert_cap;
    st.vert_base = e->L->vert_used;
}

void eng_take_results(bcmc_engine* e, uint32_t n, bcmc_query_result* out)
{
    for (uint32_t i = 0; i < n; ++i) {
        out[i].vertex_offset = e->L->h_results[i].vstart;
        out[i].num_vertices = e->L->h_results[i].nverts;
        out[i].num_active_blocks = e->L->h_results[i].nactive;
    }
    e->L->vert_used += e->L->h_st->num_verts;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, e->L->ev0, e->L->ev1) == cudaSuccess) e->stats.last_batch_ms = ms;
    e->stats.queries += n;
}

// Runs queries[0..n) (n <= max_batch) as one launch sequence; results go to out.
// Throws std::length_error when the pool cannot hold the sequence's active blocks.
void eng_run_sequence(bcmc_engine* e, const bcmc_query* queries, uint32_t n, bcmc_query_result* out)
{
    const SeqShape sh = eng_prepare(e, queries, n);
    const uint32_t bucket = sh.bucket;
    const uint64_t words = sh.words;
    ++e->use_epoch;
    for (int attempt = 0;; ++attempt) {
        if (attempt > 8) throw std::runtime_error("batch did not converge");
        eng_ensure_verts(e, e->L->vert_used + 1);
        EngState& st = *e->L->h_st;
        eng_set_inputs(e, sh);
        eng_epoch_tick(e);
        eng_launch(e, bucket);
        BCMC_CUDA(cudaStreamSynchronize(e->stream));
        ++e->stats.launch_sequences;
        if (st.error) throw std::runtime_error("device wait timed out in the batched engine");
        e->stats.decoded_blocks += st.num_decode;
        if (st.entry_overflow) {
            eng_ensure_batch(e, words, st.num_entries);
            continue;
        }
        if (st.pool_exhausted) {
            // the pool's head overshot its tail: clamp, then free what this batch does not use
            BCMC_CUDA(cudaMemcpyAsync(e->h_pool, e->d_pool, sizeof(EngPool), cudaMemcpyDeviceToHost, e->stream));
            BCMC_CUDA(cudaStreamSynchronize(e->stream));
            e->h_pool->head = e->h_pool->tail;
            BCMC_CUDA(cudaMemcpyAsync(e->d_pool, e->h_pool, sizeof(EngPool), cudaMemcpyHostToDevice, e->stream));
            BCMC_CUDA(cudaMemsetAsync(e->d_evicted, 0, 8, e->stream));
            k_bevict<<<e->ctx->num_sms * 8, 256, 0, e->stream>>>(eng_args(e), e->use_epoch, (uint32_t)e->pool_slots,
                                                                 e->d_evicted);
            count_launches(1);
            unsigned long long ev = 0;
            BCMC_CUDA(cudaMemcpyAsync(&ev, e->d_evicted, 8, cudaMemcpyDeviceToHost, e->stream));
            BCMC_CUDA(cudaStreamSynchronize(e->stream));
            e->stats.evicted_blocks += ev;
            if (ev == 0) throw std::length_error("the slot pool cannot hold one batch's active blocks");
            continue;
        }
        // vertex admission from the count pass: per-query totals are complete
        // even when the emit pass was refused for lack of room
        const uint64_t limit_seq = std::min<uint64_t>(
            (1ull << 32) - 1, e->opts.vertex_budget ? e->opts.vertex_budget - std::min(e->opts.vertex_budget, e->L->vert_used)
                                                    : ~0ull);
        if (st.vert_overflow || st.num_verts > limit_seq) {
            uint64_t cum = 0;
            uint32_t fit = 0;
            for (; fit < n; ++fit) {
                const uint64_t v = e->L->h_results[fit].nverts;
                if (cum + v > limit_seq) break;
                cum += v;
            }
            if (fit < n) throw AdmitPrefix(fit);
            eng_ensure_verts(e, e->L->vert_used + cum);
            continue;  // the re-run finds every block cached: no decode work repeats
        }
        break;
    }
    eng_take_results(e, n, out);
}

// Admission by slot memory: a batch whose active blocks do not fit the pool
// (even after evicting every slot it does not use) runs as two halves.
void eng_run_chunk(bcmc_engine* e, const bcmc_query* queries, uint32_t n, bcmc_query_result* out)
{
    try {
        eng_run_sequence(e, queries, n, out);
    } catch (const std::length_error&) {
        if (n < 2) throw;
        const uint32_t h = n / 2;
        eng_run_chunk(e, queries, h, out);
        eng_run_chunk(e, queries + h, n - h, out + h);
    }
}

void eng_free(bcmc_engine* e)
{
    bcmc_ctx* ctx = e->ctx;
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->stream_back) cudaStreamSynchronize(e->stream_back);
    if (e->stream_copy) cudaStreamSynchronize(e->stream_copy);
    for (EngLane& l : e->lanes) eng_lane_free(e, l);
    for (auto& v : e->vols) {
        dev_free(ctx, v.words, v.words_bytes);
        dev_free(ctx, v.ranges, (size_t)v.total * 8);
        dev_free(ctx, v.tile_ext, (size_t)v.tiles * 8);
        dev_free(ctx, v.item_slots, (size_t)v.total * 4);
    }
    dev_free(ctx, e->d_vols, e->d_vols_cap * sizeof(EngVolDev));
    dev_free(ctx, e->cache, e->pool_slots * 256);
    dev_free(ctx, e->free_list, e->pool_slots * 4);
    dev_free(ctx, e->last_use, e->pool_slots * 4);
    dev_free(ctx, e->owner_vol, e->pool_slots * 4);
    dev_free(ctx, e->owner_block, e->pool_slots * 4);
    dev_free(ctx, e->d_pool, sizeof(EngPool));
    dev_free(ctx, e->d_evicted, 8);
    dev_free(ctx, e->dec_vol, (size_t)e->dec_cap * 4);
    dev_free(ctx, e->dec_block, (size_t)e->dec_cap * 4);
    dev_free(ctx, e->dec_slot, (size_t)e->dec_cap * 4);
    if (e->h_pool) cudaFreeHost(e->h_pool);
    if (e->stream) cudaStreamDestroy(e->stream);
    if (e->stream_back) cudaStreamDestroy(e->stream_back);
    if (e->stream_copy) cudaStreamDestroy(e->stream_copy);
    delete e;
    ctx_child_removed(ctx);
}

template <typename F>
bcmc_status eng_guarded(bcmc_engine* e, F&& f)
{
    try {
        return f();
    } catch (const CudaError& x) {
        e->ctx->last_error = std::string(x.what) + ": " + cudaGetErrorString(x.err);
        return x.err == cudaErrorMemoryAllocation ? BCMC_E_OOM : BCMC_E_CUDA;
    } catch (const std::invalid_argument& x) {
        e->ctx->last_error = x.what();
        return BCMC_E_ARG;
    } catch (const std::length_error& x) {
        e->ctx->last_error = x.what();
        return BCMC_E_ADMISSION;
    } catch (const std::bad_alloc&) {
        e->ctx->last_error = "host allocation failed";
        return BCMC_E_OOM;
    } catch (const std::exception& x) {
        e->ctx->last_error = x.what();
        return BCMC_E_CUDA;
    }
}

}  // namespace

extern "C" bcmc_status bcmc_engine_create(bcmc_ctx* ctx, const bcmc_engine_opts* opts, bcmc_engine** out)
{
    if (!ctx || !out) return BCMC_E_ARG;
    *out = nullptr;
    bcmc_engine* e = new (std::nothrow) bcmc_engine();
    if (!e) return BCMC_E_OOM;
    e->ctx = ctx;
    if (opts) e->opts = *opts;
    if (e->opts.flags != 0) {
        delete e;
        return BCMC_E_ARG;
    }
    ctx_child_added(ctx);  // eng_free removes it, also on the error path below
    const bcmc_status st = eng_guarded(e, [&]() -> bcmc_status {
        BCMC_CUDA(cudaSetDevice(ctx->device));
        BCMC_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        BCMC_CUDA(cudaStreamCreateWithFlags(&e->stream_back, cudaStreamNonBlocking));
        BCMC_CUDA(cudaStreamCreateWithFlags(&e->stream_copy, cudaStreamNonBlocking));
        e->max_batch = bucket_of(e->opts.max_batch ? std::min<uint32_t>(e->opts.max_batch, 1u << 16) : 1024u);
        BCMC_CUDA(cudaMallocHost(&e->h_pool, sizeof(EngPool)));
        e->d_pool = (EngPool*)dev_alloc(ctx, sizeof(EngPool));
        e->d_evicted = (unsigned long long*)dev_alloc(ctx, 8);
        eng_lane_init(e, 0);
        BCMC_CUDA(cudaStreamSynchronize(e->stream));
        return BCMC_OK;
    });
    if (st != BCMC_OK) {
        eng_free(e);
        return st;
    }
    *out = e;
    return BCMC_OK;
}

extern "C" void bcmc_engine_destroy(bcmc_engine* e)
{
    if (e) eng_free(e);
}

extern "C" bcmc_status bcmc_engine_add_volume(bcmc_engine* e, const uint8_t* zfp, size_t len, uint32_t rate,
                                              const uint32_t dims[3], uint32_t* volume)
{
    if (!e || !zfp || !dims || !volume || rate == 0 || rate > 32 || !dims[0] || !dims[1] || !dims[2])
        return BCMC_E_ARG;
    if (e->vols.size() >= kMaxVolumes) return BCMC_E_ARG;
    if (e->pool_slots) return BCMC_E_STATE;  // volumes are added before the first run sizes the pool
    return eng_guarded(e, [&]() -> bcmc_status {
        EngVolume v;
        for (int i = 0; i < 3; ++i) v.dims[i] = dims[i];
        v.rate = rate;
        const uint3 nb = make_uint3(div_up(dims[0], 4u), div_up(dims[1], 4u), div_up(dims[2], 4u));
        const uint64_t total = (uint64_t)nb.x * nb.y * nb.z;
        if (total >= (1ull << 31)) throw std::invalid_argument("volume too large");
        const uint64_t need = (total * 64u * rate + 7) / 8;
        if (len < need) throw std::invalid_argument("compressed stream shorter than the volume needs");
        v.total = (uint32_t)total;
        v.tiles = div_up(v.total, kEngTile);
        v.grid = make_block_grid(nb);
        const uint64_t words = (need + 7) / 8 + 2;
        v.words_bytes = words * 8;
        v.words = (uint64_t*)dev_alloc(e->ctx, v.words_bytes);
        BCMC_CUDA(cudaMemsetAsync(v.words, 0, v.words_bytes, e->stream));
        BCMC_CUDA(cudaMemcpyAsync(v.words, zfp, need, cudaMemcpyHostToDevice, e->stream));
        v.ranges = (float2*)dev_alloc(e->ctx, (size_t)v.total * 8);
        v.tile_ext = (float2*)dev_alloc(e->ctx, (size_t)v.tiles * 8);
        v.item_slots = (int32_t*)dev_alloc(e->ctx, (size_t)v.total * 4);
        BCMC_CUDA(cudaMemsetAsync(v.item_slots, 0xff, (size_t)v.total * 4, e->stream));  // -1
        zfp_ranges_launch(e->ctx, v.words, dims, 64u * rate, reinterpret_cast<float*>(v.ranges), e->stream);
        k_tile_ext<<<v.tiles, kEngThreads, 0, e->stream>>>(v.ranges, v.grid, v.total, v.tile_ext);
        count_launches(1);
        BCMC_CUDA(cudaGetLastError());
        BCMC_CUDA(cudaStreamSynchronize(e->stream));
        *volume = (uint32_t)e->vols.size();
        e->vols.push_back(v);
        if (rate > e->max_rate) {
            e->max_rate = rate;
            for (EngLane& l : e->lanes) ++l.generation;  // graphs captured k_bdecode's staging size
        }
        eng_upload_vols(e);
        return BCMC_OK;
    });
}

extern "C" bcmc_status bcmc_engine_run(bcmc_engine* e, const bcmc_query* queries, uint32_t n,
                                       bcmc_query_result* results)
{
    if (!e || (n && (!queries || !results))) return BCMC_E_ARG;
    if (e->vols.empty()) return BCMC_E_STATE;
    return eng_guarded(e, [&]() -> bcmc_status {
        if (!e->pool_slots) {
            uint64_t all = 0;
            for (auto& v : e->vols) all += v.total;
            eng_alloc_pool(e, e->opts.pool_slots ? e->opts.pool_slots : all);
        }
        e->L->vert_used = 0;
        for (uint32_t i = 0; i < n; i += e->max_batch) {
            const uint32_t m = std::min(e->max_batch, n - i);
            eng_run_chunk(e, queries + i, m, results + i);
        }
        ++e->stats.batches;
        return BCMC_OK;
    });
}

namespace {
// Runs the longest prefix of queries[0..n) that the slot pool and the vertex
// budget admit (halving on refusal); returns its length.  Throws
// std::length_error when not even queries[0] alone fits.
uint32_t eng_run_prefix(bcmc_engine* e, const bcmc_query* queries, uint32_t n, bcmc_query_result* out)
{
    try {
        eng_run_sequence(e, queries, n, out);
        return n;
    } catch (const AdmitPrefix& x) {  // the count pass says how many fit
        if (x.fit == 0) throw;
        return eng_run_prefix(e, queries, x.fit, out);
    } catch (const std::length_error&) {  // the slot pool: halve
        if (n < 2) throw;
        return eng_run_prefix(e, queries, n / 2, out);
    }
}
}  // namespace

namespace {
// device time of one launch sequence under the current tuned config: best of 3
double eng_time_sequence(bcmc_engine* e, const bcmc_query* qs, uint32_t n, bcmc_query_result* out)
{
    double best = 1e30;
    for (int r = 0; r < 3; ++r) {
        e->L->vert_used = 0;
        eng_run_sequence(e, qs, n, out);
        best = std::min(best, e->stats.last_batch_ms);
    }
    return best;
}

double eng_time_decode(bcmc_engine* e, const EngVolume& v, uint32_t nblk, float* scratch, int threads, int per_sm)
{
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
        BCMC_CUDA(cudaEventRecord(e->L->ev0, e->stream));
        const int grid = e->ctx->num_sms * per_sm;
        const size_t smem = zfp_stage_smem((uint32_t)threads, v.rate);
        if (threads == 64) {
            allow_smem(k_decode_probe<64>, smem);
            k_decode_probe<64><<<grid, 64, smem, e->stream>>>(v.words, v.rate, nblk, scratch);
        } else if (threads == 256) {
            allow_smem(k_decode_probe<256>, smem);
            k_decode_probe<256><<<grid, 256, smem, e->stream>>>(v.words, v.rate, nblk, scratch);
        } else {
            allow_smem(k_decode_probe<128>, smem);
            k_decode_probe<128><<<grid, 128, smem, e->stream>>>(v.words, v.rate, nblk, scratch);
        }
        count_launches(1);
        BCMC_CUDA(cudaGetLastError());
        BCMC_CUDA(cudaEventRecord(e->L->ev1, e->stream));
        BCMC_CUDA(cudaEventSynchronize(e->L->ev1));
        float ms = 0.0f;
        BCMC_CUDA(cudaEventElapsedTime(&ms, e->L->ev0, e->L->ev1));
        best = std::min(best, ms);
    }
    return best;
}
}  // namespace

extern "C" bcmc_status bcmc_engine_autotune(bcmc_engine* e, const bcmc_query* queries, uint32_t n,
                                            bcmc_tune_report* out)
{
    if (!e || !queries || !n || !out) return BCMC_E_ARG;
    if (e->vols.empty()) return BCMC_E_STATE;
    return eng_guarded(e, [&]() -> bcmc_status {
        if (!e->pool_slots) {
            uint64_t all = 0;
            for (auto& v : e->vols) all += v.total;
            eng_alloc_pool(e, e->opts.pool_slots ? e->opts.pool_slots : all);
        }
        const uint32_t m = std::min(n, e->max_batch);
        const uint32_t bucket = std::min(bucket_of(m), e->max_batch);
        std::vector<bcmc_query_result> res(m);
        e->tuned.erase(bucket);
        e->L->vert_used = 0;
        eng_run_sequence(e, queries, m, res.data());  // warm-up: decodes, buffer growth, graph
        EngConfig best{};
        e->tuned[bucket] = best;
        double t_best = eng_time_sequence(e, queries, m, res.data());
        out->batch_ms_default = t_best;
        // coordinate descent over the sequence's launch parameters
        for (int mb : {8, 32}) {  // MC tile: active blocks per CTA tile
            EngConfig c = best;
            c.mc_blocks = mb;
            e->tuned[bucket] = c;
            const double t = eng_time_sequence(e, queries, m, res.data());
            if (t < t_best) best = c, t_best = t;
        }
        for (int mc : {4, 5}) {
            EngConfig c = best;
            c.mc_per_sm = mc;
            e->tuned[bucket] = c;
            const double t = eng_time_sequence(e, queries, m, res.data());
            if (t < t_best) best = c, t_best = t;
        }
        for (int act : {4, 8, 16}) {
            EngConfig c = best;
            c.act_per_sm = act;
            e->tuned[bucket] = c;
            const double t = eng_time_sequence(e, queries, m, res.data());
            if (t < t_best) best = c, t_best = t;
        }
        out->batch_ms_tuned = t_best;
        // decode: a probe over (up to 2^18) blocks of the largest volume
        const EngVolume* big = &e->vols[0];
        for (auto& v : e->vols)
            if (v.total > big->total) big = &v;
        const uint32_t nblk = std::min<uint32_t>(big->total, 1u << 18);
        float* scratch = (float*)dev_alloc(e->ctx, (size_t)nblk * 256);
        double d_best = 1e30, d_default = 0.0;
        try {
            for (int thr : {64, 128, 256})
                for (int per_sm : {8, 16, 32}) {
                    const double t = eng_time_decode(e, *big, nblk, scratch, thr, per_sm);
                    if (thr == 128 && per_sm == 16) d_default = t;
                    if (t < d_best) {
                        d_best = t;
                        best.dec_threads = thr;
                        best.dec_per_sm = per_sm;
                    }
                }
        } catch (...) {
            dev_free(e->ctx, scratch, (size_t)nblk * 256);
            throw;
        }
        dev_free(e->ctx, scratch, (size_t)nblk * 256);
        e->tuned[bucket] = best;
        out->decode_ms_default = d_default;
        out->decode_ms_tuned = d_best;
        out->act_ctas_per_sm = best.act_per_sm;
        out->decode_threads = best.dec_threads;
        out->decode_ctas_per_sm = best.dec_per_sm;
        out->mc_ctas_per_sm = best.mc_per_sm;
        out->mc_blocks_per_tile = best.mc_blocks;
        out->bucket = bucket;
        return BCMC_OK;
    });
}

extern "C" bcmc_status bcmc_engine_set_tuning(bcmc_engine* e, const bcmc_tune_report* c)
{
    if (!e || !c) return BCMC_E_ARG;
    const uint32_t b = c->bucket;
    const auto in = [](int v, std::initializer_list<int> ok) { return std::find(ok.begin(), ok.end(), v) != ok.end(); };
    if (b == 0 || (b & (b - 1)) != 0 || b > e->max_batch || !in(c->act_ctas_per_sm, {4, 8, 16}) ||
        !in(c->decode_threads, {64, 128, 256}) || !in(c->decode_ctas_per_sm, {8, 16, 32}) ||
        !in(c->mc_ctas_per_sm, {4, 5, 6}) || !in(c->mc_blocks_per_tile, {8, 16, 32}))
        return BCMC_E_ARG;
    EngConfig cfg;
    cfg.act_per_sm = c->act_ctas_per_sm;
    cfg.dec_threads = c->decode_threads;
    cfg.dec_per_sm = c->decode_ctas_per_sm;
    cfg.mc_per_sm = c->mc_ctas_per_sm;
    cfg.mc_blocks = c->mc_blocks_per_tile;
    e->tuned[b] = cfg;
    return BCMC_OK;
}

extern "C" bcmc_status bcmc_engine_run_admit(bcmc_engine* e, const bcmc_query* queries, uint32_t n,
                                             bcmc_query_result* results, uint32_t* admitted)
{
    if (!e || !admitted || (n && (!queries || !results))) return BCMC_E_ARG;
    if (e->vols.empty()) return BCMC_E_STATE;
    *admitted = 0;
    return eng_guarded(e, [&]() -> bcmc_status {
        if (!e->pool_slots) {
            uint64_t all = 0;
            for (auto& v : e->vols) all += v.total;
            eng_alloc_pool(e, e->opts.pool_slots ? e->opts.pool_slots : all);
        }
        e->L->vert_used = 0;
        uint32_t done = 0;
        while (done < n) {
            const uint32_t m = std::min(e->max_batch, n - done);
            uint32_t got;
            try {
                got = eng_run_prefix(e, queries + done, m, results + done);
            } catch (const std::length_error&) {
                if (done) break;  // the rest waits for the next run
                throw;
            }
            done += got;
            if (got < m) break;
        }
        *admitted = done;
        ++e->stats.batches;
        return BCMC_OK;
    });
}

extern "C" bcmc_status bcmc_engine_vertices(bcmc_engine* e, const void** d_vertices, uint64_t* count)
{
    if (!e || !d_vertices || !count) return BCMC_E_ARG;
    *d_vertices = e->L->verts;
    *count = e->L->vert_used;
    return BCMC_OK;
}

extern "C" bcmc_status bcmc_engine_copy_vertices(bcmc_engine* e, uint64_t first, uint64_t count, void* host)
{
    if (!e || (count && !host) || first > e->L->vert_used || count > e->L->vert_used - first) return BCMC_E_ARG;
    return eng_guarded(e, [&]() -> bcmc_status {
        if (count)
            BCMC_CUDA(cudaMemcpyAsync(host, e->L->verts + first, count * sizeof(uint2), cudaMemcpyDeviceToHost, e->stream));
        BCMC_CUDA(cudaStreamSynchronize(e->stream));
        return BCMC_OK;
    });
}

extern "C" bcmc_status bcmc_engine_stats_get(bcmc_engine* e, bcmc_engine_stats* out)
{
    if (!e || !out) return BCMC_E_ARG;
    return eng_guarded(e, [&]() -> bcmc_status {
        bcmc_engine_stats s = e->stats;
        s.pool_slots = e->pool_slots;
        if (e->pool_slots) {
            BCMC_CUDA(cudaMemcpyAsync(e->h_pool, e->d_pool, sizeof(EngPool), cudaMemcpyDeviceToHost, e->stream));
            BCMC_CUDA(cudaStreamSynchronize(e->stream));
            const uint32_t head = std::min(e->h_pool->head, e->h_pool->tail);
            s.pool_used = e->pool_slots - (e->h_pool->tail - head);
        }
        s.vertex_capacity = e->L->vert_cap;
        s.overlapped_batches = e->overlapped;
        s.device_bytes = e->ctx->device_bytes;
        *out = s;
        return BCMC_OK;
    });
}

namespace bcmc {
namespace {
void eng_ensure_pool(bcmc_engine* e)
{
    if (e->pool_slots) return;
    uint64_t all = 0;
    for (auto& v : e->vols) all += v.total;
    eng_alloc_pool(e, e->opts.pool_slots ? e->opts.pool_slots : all);
}
}  // namespace

bcmc_status engine_submit(bcmc_engine* e, int k, const bcmc_query* queries, uint32_t n, void (*on_done)(void*),
                          void* arg)
{
    if (!e || k < 0 || k > 1 || !n || !queries || n > e->max_batch) return BCMC_E_ARG;
    if (e->vols.empty() || e->lanes[k].in_flight) return BCMC_E_STATE;
    return eng_guarded(e, [&]() -> bcmc_status {
        eng_ensure_pool(e);
        eng_lane_init(e, k);
        EngLane& me = *e->L;
        me.vert_used = 0;
        const SeqShape sh = eng_prepare(e, queries, n);
        ++e->use_epoch;
        eng_ensure_verts(e, 1);
        eng_set_inputs(e, sh);
        eng_epoch_tick(e);
        eng_launch_split(e, sh.bucket);
        BCMC_CUDA(cudaEventRecord(me.ev_done, e->stream_back));
        if (on_done) BCMC_CUDA(cudaLaunchHostFunc(e->stream_back, on_done, arg));
        me.in_flight = true;
        me.n = n;
        me.bucket = sh.bucket;
        me.batch_epoch = e->use_epoch;
        me.queries.assign(queries, queries + n);
        if (e->lanes[1 - k].in_flight) ++e->overlapped;
        ++e->stats.launch_sequences;
        ++e->stats.batches;
        return BCMC_OK;
    });
}

bcmc_status engine_complete(bcmc_engine* e, int k, bcmc_query_result* out, uint32_t* admitted)
{
    if (!e || k < 0 || k > 1 || !out || !admitted) return BCMC_E_ARG;
    EngLane& me = e->lanes[k];
    if (!me.in_flight) return BCMC_E_STATE;
    *admitted = 0;
    me.in_flight = false;
    return eng_guarded(e, [&]() -> bcmc_status {
        e->L = &me;
        BCMC_CUDA(cudaEventSynchronize(me.ev_done));
        const EngState& st = *me.h_st;
        e->stats.decoded_blocks += st.num_decode;
        if (st.error) throw std::runtime_error("device wait timed out in the batched engine");
        const uint64_t limit = std::min<uint64_t>((1ull << 32) - 1, e->opts.vertex_budget ? e->opts.vertex_budget : ~0ull);
        if (st.entry_overflow || st.pool_exhausted || st.vert_overflow || st.num_verts > limit) {
            // buffer growth, eviction or admission: run this batch again on its
            // own, after both streams have drained (an eviction must not free a
            // slot the other lane's batch still reads)
            BCMC_CUDA(cudaStreamSynchronize(e->stream));
            BCMC_CUDA(cudaStreamSynchronize(e->stream_back));
            me.vert_used = 0;
            *admitted = eng_run_prefix(e, me.queries.data(), me.n, out);
            return BCMC_OK;
        }
        eng_take_results(e, me.n, out);
        *admitted = me.n;
        return BCMC_OK;
    });
}

bcmc_status engine_copy_lane_vertices(bcmc_engine* e, int k, uint64_t first, uint64_t count, void* host)
{
    if (!e || k < 0 || k > 1 || (count && !host)) return BCMC_E_ARG;
    EngLane& l = e->lanes[k];
    if (first > l.vert_used || count > l.vert_used - first) return BCMC_E_ARG;
    return eng_guarded(e, [&]() -> bcmc_status {
        if (count) {
            BCMC_CUDA(cudaMemcpyAsync(host, l.verts + first, count * sizeof(uint2), cudaMemcpyDeviceToHost,
                                      e->stream_copy));
            BCMC_CUDA(cudaStreamSynchronize(e->stream_copy));
        }
        return BCMC_OK;
    });
}

void engine_drain(bcmc_engine* e)
{
    cudaStreamSynchronize(e->stream);
    cudaStreamSynchronize(e->stream_back);  // also waits for its host callbacks
    cudaStreamSynchronize(e->stream_copy);
}

uint32_t engine_max_batch(bcmc_engine* e) { return e->max_batch; }
uint32_t engine_num_volumes(bcmc_engine* e) { return (uint32_t)e->vols.size(); }

int engine_device(bcmc_engine* e) { return e->ctx->device; }
uint64_t engine_vertex_budget(bcmc_engine* e) { return e->opts.vertex_budget; }
bcmc_ctx* engine_ctx(bcmc_engine* e) { return e->ctx; }
}  // namespace bcmc
