/*
 * bcmc_oracle.h -- CPU oracle for the block-compressed marching-cubes path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * compute shaders and JavaScript orchestration (Twinklebear/webgpu-bcmc), used
 * to check the CUDA implementation bit for bit and timed as the CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * it; the product library never links it.
 *
 * Every function names the reference file:line it follows.  The ZFP encoder has
 * no counterpart in the reference (it only decodes); it is written from the
 * published fixed-rate method (Lindstrom 2014, "Fixed-Rate Compressed
 * Floating-Point Arrays", IEEE TVCG 20(12)) and produces the stream layout that
 * shaders/zfp_decompress.comp reads.
 */
#ifndef BCMC_ORACLE_H
#define BCMC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- stream geometry ---------------------------------------------------- */
/* Number of 64-bit words of a fixed-rate stream for `dims`, plus one zero pad
 * word (the reference's reader may fetch one word past the last block,
 * shaders/zfp_decompress.comp:212-217). */
uint64_t bcmc_oracle_stream_words(const uint32_t dims[3], uint32_t max_bits);

/* ---- ZFP fixed-rate encoder (published method, not in the reference) ----- */
int bcmc_oracle_zfp_encode(const float* field, const uint32_t dims[3], uint32_t max_bits,
                           uint64_t* words);

/* ---- decoder: shaders/zfp_decompress.comp:195-384 ------------------------ */
/* Decode block `block_index` with the reference's emulated-uint64 reader.
 * emulate_u32_offset=1 reproduces the reference's 32-bit `block_index*max_bits`
 * (zfp_decompress.comp:199), which wraps beyond 2^32 bits. */
void bcmc_oracle_decode_block(const uint64_t* words, uint64_t block_index, uint32_t max_bits,
                              int emulate_u32_offset, float out[64]);
/* Same decode with a native 64-bit reader (checks the emulation). */
void bcmc_oracle_decode_block_native(const uint64_t* words, uint64_t block_index,
                                     uint32_t max_bits, float out[64]);
/* Decoded integer coefficients (after decode_ints, before un-permute). */
void bcmc_oracle_decode_block_ints(const uint64_t* words, uint64_t block_index, uint32_t max_bits,
                                   uint32_t out[64], uint32_t* s_cont, int32_t* emax);
/* Decode every block of the volume into out[nblocks*64] (block order). */
void bcmc_oracle_decode_volume(const uint64_t* words, uint64_t nblocks, uint32_t max_bits,
                               float* out);

/* ---- zfp_compute_block_range.comp:19-61 ---------------------------------- */
void bcmc_oracle_block_ranges(const uint64_t* words, const uint32_t dims[3], uint32_t max_bits,
                              float* ranges /* [2*nblocks] */);

/* ---- mc_isosurface.vert:51-60: world (3 floats) and clip (4 floats) ------- */
void bcmc_oracle_unpack_vertices(const uint32_t* verts, uint64_t n, const uint32_t dims[3], const float scale[3],
                                 const float* proj_view, float* world, float* clip);

/* ---- the render pass, headless (js/bcmc.js:174-190,237-265,377-391) ------ */
/* mc_isosurface.vert:35-49 (DRAW_FOG): per vertex the distance along the eye
 * ray where it enters the box [-scale/2, scale/2], at least 0. */
void bcmc_oracle_fog_enter(const float* world, uint64_t n, const float eye[3], const float scale[3], float* tenter);
/* mc_isosurface.frag:15-40 for one fragment (tri_world: the triangle's 3
 * world vertices, whose edges give the flat normal). */
void bcmc_oracle_shade(const float wp[3], float t_enter, const float eye[3], const float* tri_world, int fog,
                       float rgba[4]);
/* n packed vertices drawn as n/3 triangles into width x height: rgba (4 per
 * pixel), depth and triangle (may be NULL; 0xFFFFFFFF = background).
 * Returns 0, or -1 when a host allocation fails. */
int bcmc_oracle_render(const uint32_t* verts, uint64_t n, const uint32_t dims[3], const float scale[3],
                       const float proj_view[16], const float eye[3], int fog, uint32_t width, uint32_t height,
                       float* rgba, float* depth, uint32_t* triangle);

/* ---- compute_block_active.comp:24-61 ------------------------------------- */
void bcmc_oracle_block_active(const float* ranges, const uint32_t dims[3], float isovalue,
                              uint32_t* active);

/* ---- exclusive_scan.js:178-295 (+ prefix_sum/block_prefix_sum/add_block_sums)
 * In-place exclusive scan of data[0..n); when n < aligned_n, data[n] receives
 * the total.  Returns the total (mod 2^32). */
uint32_t bcmc_oracle_exclusive_scan(uint32_t* data, uint32_t n, uint32_t aligned_n);

/* ---- stream_compact.comp:26-32, stream_compact.js:56-165 ----------------- */
void bcmc_oracle_compact(const uint32_t* flags, const uint32_t* offsets, uint32_t n,
                         uint32_t* out);

/* ---- radix_sort_by_key.js:155-400 --------------------------------------- */
uint32_t bcmc_oracle_sort_aligned_size(uint32_t n);
/* keys/values hold aligned_size(n) entries; sorted values land in values[0..n). */
void bcmc_oracle_sort_by_key(uint32_t* keys, uint32_t* values, uint32_t n, int reverse);

/* ---- LRU cache: lru_cache.js:4-903 -------------------------------------- */
typedef struct bcmc_oracle_lru bcmc_oracle_lru;
bcmc_oracle_lru* bcmc_oracle_lru_create(uint32_t initial_size, uint32_t element_size,
                                        uint32_t total_elements);
void bcmc_oracle_lru_destroy(bcmc_oracle_lru* c);
/* Returns numNewItems; new_item_ids receives them (capacity total_elements). */
uint32_t bcmc_oracle_lru_update(bcmc_oracle_lru* c, const uint32_t* item_needed,
                                uint32_t* new_item_ids);
void bcmc_oracle_lru_reset(bcmc_oracle_lru* c);
uint32_t bcmc_oracle_lru_cache_size(const bcmc_oracle_lru* c);
uint32_t bcmc_oracle_lru_slots_available(const bcmc_oracle_lru* c); /* displayNumSlotsAvailable */
const int32_t* bcmc_oracle_lru_item_slots(const bcmc_oracle_lru* c);  /* [total] */
const uint32_t* bcmc_oracle_lru_slot_age(const bcmc_oracle_lru* c);   /* [cache_size] */
const uint32_t* bcmc_oracle_lru_slot_avail(const bcmc_oracle_lru* c); /* [cache_size] */
const int32_t* bcmc_oracle_lru_slot_item(const bcmc_oracle_lru* c);   /* [cache_size] */
float* bcmc_oracle_lru_cache_data(bcmc_oracle_lru* c);               /* [cache_size*64] */
/* Sorted available slot ids of the last update that had new items. */
const uint32_t* bcmc_oracle_lru_last_sorted(const bcmc_oracle_lru* c, uint32_t* n);

/* ---- CompressedMarchingCubes: compressed_marching_cubes.js:1-1122 -------- */
typedef struct bcmc_oracle_mc bcmc_oracle_mc;
bcmc_oracle_mc* bcmc_oracle_mc_create(const uint64_t* words, uint64_t nwords,
                                      uint32_t compression_rate, const uint32_t dims[3],
                                      const float scale[3], double initial_cache_fraction);
void bcmc_oracle_mc_destroy(bcmc_oracle_mc* m);
uint32_t bcmc_oracle_mc_compute_surface(bcmc_oracle_mc* m, float isovalue);
void bcmc_oracle_mc_cache_reset(bcmc_oracle_mc* m);
bcmc_oracle_lru* bcmc_oracle_mc_lru(bcmc_oracle_mc* m);
const uint32_t* bcmc_oracle_mc_vertices(const bcmc_oracle_mc* m);  /* uvec2 per vertex */
const float* bcmc_oracle_mc_ranges(const bcmc_oracle_mc* m);
const uint32_t* bcmc_oracle_mc_active(const bcmc_oracle_mc* m);
const uint32_t* bcmc_oracle_mc_active_ids(const bcmc_oracle_mc* m);
const uint32_t* bcmc_oracle_mc_with_verts(const bcmc_oracle_mc* m);   /* indices into active ids */
const uint32_t* bcmc_oracle_mc_vert_offsets(const bcmc_oracle_mc* m); /* per block with verts */
const uint32_t* bcmc_oracle_mc_new_items(const bcmc_oracle_mc* m);
/* stats[0..6] = totalBlocks, numActiveBlocks, newDecompressed,
 * numBlocksWithVertices, numVertices, cacheSize, slotsAvailable */
void bcmc_oracle_mc_stats(const bcmc_oracle_mc* m, uint32_t stats[7]);

/* ---- per-cell counts for the 256-case table sweep ------------------------- */
uint32_t bcmc_oracle_case_vertex_count(uint32_t case_index);
const int32_t* bcmc_oracle_tri_table(void); /* 256*16 */

/* threads the OpenMP build uses (1 without OpenMP) */
int bcmc_oracle_threads(void);

#ifdef __cplusplus
}
#endif
#endif
