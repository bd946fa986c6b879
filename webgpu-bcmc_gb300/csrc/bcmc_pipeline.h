// bcmc_pipeline.h -- argument blocks and launchers of the query pipeline
// kernels (pipeline.cu).  Internal to libbcmc_gb300.
#pragma once

#include "bcmc_impl.h"

namespace bcmc {

struct ActiveArgs {
    const float2* ranges;     // set: test ranges against the isovalue (MC path)
    uint3 nb;                 // blocks per axis
    BlockGrid grid;           // id -> (x, y, z) without integer division
    const uint32_t* item_needed;  // set instead of ranges: standalone LRU update
    uint32_t* active_out;     // per-block active flags (MC path)
    const int32_t* item_slots;  // cachedItemSlots
    uint32_t total;           // blocks / items
    uint32_t* active_ids;     // compacted active ids (nullable)
    uint32_t* new_ids;        // compacted ids that need caching
    uint64_t* status_a;
    uint64_t* status_n;
};

struct SlotArgs {
    const uint32_t* needed;   // per item: 1 if needed this update
    uint32_t* slot_age;
    uint32_t* slot_avail;
    int32_t* slot_item;
    uint32_t* avail_ids;      // compacted available slots (ascending)
    uint32_t* avail_keys;     // their ages
    uint64_t* status;
    // computeSurface skips the cache update when no block is active
    // (compressed_marching_cubes.js:630-641); LRUCache.update itself always ages
    uint32_t skip_when_inactive;
    // 1: also accumulate the digit histograms of ~age (the descending sort's
    // keys) and make the sort's pass plan in the last CTA, so the sort that
    // follows runs without its histogram kernel
    uint32_t plan;
    // the joint histogram of the 16-bit age keys whose age is below 256 in
    // its class (kAgeBins bins: class, low byte), zero between updates, and
    // the dense rank of each bin, for a one-pass sort when every key is such
    // and at most 256 bins are used
    uint32_t* age_hist;
    uint8_t* age_rank;
};

struct AssignArgs {
    const uint32_t* new_ids;
    const uint32_t* sorted_b;  // sorted slot ids in sort buffer b or c
    const uint32_t* sorted_c;
    uint32_t* slot_age;
    uint32_t* slot_avail;
    int32_t* slot_item;
    int32_t* item_slots;
    const uint64_t* words;    // set: decode each new block into its slot
    uint32_t max_bits;
    float* cache;
    // set: new blocks [0, stage_blocks) were decoded into stage (one element
    // per new-block index) by k_decode_new and are copied into their slots
    const float* stage;
    uint32_t stage_blocks;
};

// k_decode_new: the new blocks' ZFP decode, run beside the LRU's slot
// selection (it needs only the new ids) into a staging buffer.
struct DecodeArgs {
    const uint32_t* new_ids;
    const uint64_t* words;
    uint32_t max_bits;
    float* stage;           // stage_blocks * 64 floats
    uint32_t stage_blocks;
};

struct McArgs {
    const uint32_t* active;
    const uint32_t* active_ids;
    const int32_t* item_slots;
    const float* cache;
    uint3 nb;
    BlockGrid grid;
    uint32_t* with_verts;
    uint32_t* vert_offsets;
    uint32_t* block_counts;  // vertices of each active block (count pass -> list entries)
    uint2* verts;
    uint64_t* status_v;
    uint64_t* status_b;
    // 1: verts is page-locked host memory; each warp's vertex stores then
    // cover one 256 B-aligned window, which such stores need for full speed
    uint32_t host_verts;
};

void query_begin_launch(QueryState* q, float iso, int mc_only, uint32_t capacity, uint32_t vert_capacity,
                        cudaStream_t s, const QueryInputs* in = nullptr);
void query_end_launch(const QueryState* q, QueryState* host, cudaStream_t s);
void active_launch(bcmc_ctx* ctx, QueryState* q, const ActiveArgs& a, cudaStream_t s);
void slots_launch(bcmc_ctx* ctx, QueryState* q, const SlotArgs& a, uint32_t max_slots, cudaStream_t s);
void assign_launch(bcmc_ctx* ctx, QueryState* q, const AssignArgs& a, uint32_t max_new, cudaStream_t s);
void decode_new_launch(bcmc_ctx* ctx, const QueryState* q, const DecodeArgs& a, cudaStream_t s);
void mc_launch(bcmc_ctx* ctx, QueryState* q, const McArgs& a, uint32_t max_active, cudaStream_t s);
uint32_t active_tiles(uint32_t total);
uint32_t slot_tiles(uint32_t slots);
uint32_t mc_grid(bcmc_ctx* ctx, uint32_t max_active);

}  // namespace bcmc
