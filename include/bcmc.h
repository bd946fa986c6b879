/*
 * bcmc.h -- C ABI of the GB300 block-compressed marching-cubes library
 * (libbcmc_gb300.so, CUDA for sm_103a).
 *
 * Drop-in for the compute path of Twinklebear/webgpu-bcmc: the
 * CompressedMarchingCubes pipeline (js/compressed_marching_cubes.js) and the
 * GPU primitives it is built from (js/lru_cache.js, js/exclusive_scan.js,
 * js/stream_compact.js, js/radix_sort_by_key.js).  Every entry point names the
 * reference interface it replaces.  Plain pointers and sizes only; no C++
 * exceptions cross this boundary.  `stream` arguments are cudaStream_t values
 * passed as void* (NULL = the context's own stream).  Device pointers are
 * plain CUDA device addresses on the context's device.
 *
 * Threading: a context and the objects made from it are used by one host
 * thread at a time.
 */
#ifndef BCMC_H
#define BCMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BCMC_ABI_VERSION 1

/* Status codes.  The reference reports errors with alert()/console.log
 * (js/lru_cache.js:315-317, js/exclusive_scan.js:117-119, js/util.js:29-31). */
typedef enum {
    BCMC_OK = 0,
    BCMC_E_ARG = 1,       /* invalid argument (sizes, null pointers, rate)      */
    BCMC_E_OOM = 2,       /* device or host allocation failed                   */
    BCMC_E_CUDA = 3,      /* a CUDA call failed; see bcmc_last_error()          */
    BCMC_E_TIMEOUT = 4,   /* a device-side wait hit its iteration limit         */
    BCMC_E_ADMISSION = 5, /* a request does not fit the configured memory       */
    BCMC_E_STATE = 6,     /* call order violated (e.g. no surface computed yet) */
    BCMC_E_LIMIT = 7      /* size above a fixed compile-time limit of the call  */
} bcmc_status;

typedef struct bcmc_ctx bcmc_ctx;
typedef struct bcmc_vol bcmc_vol;
typedef struct bcmc_lru bcmc_lru;

/* Context options.  Defaults (bcmc_opts_default): device 0,
 * initial cache 5 % of the blocks (compressed_marching_cubes.js:446). */
typedef struct {
    int device;                    /* CUDA device ordinal                          */
    double initial_cache_fraction; /* LRU initial size as a fraction of blocks     */
    uint32_t flags;                /* BCMC_FLAG_* bits, 0 = the reference's behaviour */
} bcmc_opts;

void bcmc_opts_default(bcmc_opts* opts);

/* bcmc_opts.flags bits.
 * BCMC_FLAG_FULL_RANGES: compute the value range of every block.  By default
 * block ranges follow the reference exactly: zfp_compute_block_range.comp:22
 * counts the blocks as (padded x * padded y) / 64 * padded z in 32-bit integers,
 * which truncates when (x/4)*(y/4) is not a multiple of 4, and the ranges of the
 * blocks past that count stay at the zero of the freshly created buffer
 * (compressed_marching_cubes.js:526-529). */
#define BCMC_FLAG_FULL_RANGES 1u

/* ---- context ------------------------------------------------------------ */
/* Replaces the WebGPU device handed to `new CompressedMarchingCubes(device)`
 * (js/compressed_marching_cubes.js:1, js/bcmc.js:2-13). */
bcmc_status bcmc_ctx_create(const bcmc_opts* opts, bcmc_ctx** out);
void bcmc_ctx_destroy(bcmc_ctx* ctx);
const char* bcmc_last_error(const bcmc_ctx* ctx);
/* The context's CUDA stream (cudaStream_t as void*). */
void* bcmc_ctx_stream(bcmc_ctx* ctx);
/* Wait for all work the context queued. */
bcmc_status bcmc_ctx_synchronize(bcmc_ctx* ctx);
/* CUDA kernels this library has launched in this process (all contexts).
 * No reference counterpart: lets callers account for the GPU work behind a
 * call (e.g. kernels per query). */
uint64_t bcmc_kernel_launches(void);
/* Test hook, no reference counterpart (the reference's only guards are alerts,
 * js/lru_cache.js:315-317, js/exclusive_scan.js:117-119).  With
 * tile_plus_one = t + 1, tile t of the active test of every later query on
 * this context, and of its primitive scans (bcmc_scan_exclusive_u32[_async],
 * bcmc_select_ids), publishes no decoupled look-back status: the tiles after
 * it wait on a status word that nothing sets until their bounded spin runs
 * out (about a second), and the call returns BCMC_E_TIMEOUT.  A query that
 * times out resets its volume's cache (the slot arrays are not trusted after
 * a wait gave up), so the next query starts from an empty cache.  0 turns the
 * hook off.  Nothing faults or hangs: the waits are bounded. */
bcmc_status bcmc_debug_drop_tile(bcmc_ctx* ctx, uint32_t tile_plus_one);

/* ---- CompressedMarchingCubes -------------------------------------------- */
/* setCompressedVolume(volume, compressionRate, volumeDims, volumeScale)
 * (js/compressed_marching_cubes.js:432-520): uploads the fixed-rate ZFP stream
 * (host bytes, 64*rate bits per 4^3 block, x-fastest block order) and computes
 * every block's value range (computeBlockRanges, :522-578). */
bcmc_status bcmc_volume_create(bcmc_ctx* ctx, const uint8_t* zfp, size_t len, uint32_t rate,
                               const uint32_t dims[3], const float scale[3], bcmc_vol** out);
/* Same, from a stream already resident on the device (copied device-to-device). */
bcmc_status bcmc_volume_create_device(bcmc_ctx* ctx, const void* d_zfp, size_t len, uint32_t rate,
                                      const uint32_t dims[3], const float scale[3],
                                      bcmc_vol** out);
void bcmc_volume_destroy(bcmc_vol* vol);

/* Per-stage device times in milliseconds, keyed like the reference's
 * perfTracker (compressed_marching_cubes.js:593-610). */
typedef struct {
    float computeActiveBlocks; /* active test + compaction + cache lookup        */
    float cacheUpdate;         /* LRU age/mark/grow/sort                         */
    float decompression;       /* slot assignment and the new blocks' data into
                                * their slots; their ZFP decode runs beside the
                                * cache update, so only what is left of it after
                                * the sort is counted here                       */
    float computeVertices;     /* MC count + scan + emit                         */
    float total;
} bcmc_perf;

/* computeSurface(isovalue, perfTracker) -> numVertices
 * (js/compressed_marching_cubes.js:580-809).  Blocks until the vertex count is
 * known.  `perf` may be NULL (no per-stage timing); passing one adds the
 * stage-timing events to the query (some tens of microseconds).  Vertex
 * counts are 32-bit, as the reference's: a query of 2^32 or more vertices
 * returns BCMC_E_STATE (its mesh is not produced). */
bcmc_status bcmc_compute_surface(bcmc_vol* vol, float isovalue, bcmc_perf* perf,
                                 uint32_t* num_vertices);

/* The same query with the vertices written by the kernels straight into host
 * memory: host_vertices must be page-locked (cudaMallocHost or
 * cudaHostRegister) and 8-byte aligned, with room for `capacity` vertices.
 * The device-to-host transfer overlaps the vertex computation, which a
 * bcmc_compute_surface + bcmc_copy_vertices pair runs one after the other.
 * The volume's device vertex buffer is not written: bcmc_vertices and
 * bcmc_copy_vertices return BCMC_E_STATE until the next bcmc_compute_surface.
 * When the query has more than `capacity` vertices, returns BCMC_E_LIMIT with
 * *num_vertices set to the count needed (the buffer's contents are then
 * unspecified); the cache state has advanced as for a completed query.
 * No counterpart in the reference, whose vertices stay in a GPU buffer. */
bcmc_status bcmc_compute_surface_host(bcmc_vol* vol, float isovalue, void* host_vertices, uint64_t capacity,
                                      uint32_t* num_vertices);

/* n queries run in order on the volume (the cache state advances exactly as
 * n bcmc_compute_surface calls would), their vertices delivered back to back
 * into one page-locked, 8-byte aligned host buffer of `capacity` vertices:
 * query i's num_vertices[i] vertices start at vertex sum(num_vertices[0..i-1]).
 * Each query computes into one of two device vertex buffers while the
 * previous query's vertices are copied out of the other, so a sweep runs at
 * the rate of the slower of computation and transfer.  Returns once every
 * transfer has completed.  When query i does not fit in what is left of the
 * buffer: BCMC_E_LIMIT, num_vertices[i] = its count, later queries are not run
 * (their counts are 0) and the cache state has advanced through query i.
 * Afterwards bcmc_vertices gives query n-1's vertices on the device.
 * No counterpart in the reference, whose vertices stay in a GPU buffer. */
bcmc_status bcmc_compute_surfaces_host(bcmc_vol* vol, const float* isovalues, uint32_t n, void* host_vertices,
                                       uint64_t capacity, uint32_t* num_vertices);

/* The vertex buffer (this.vertexBuffer, :781-784): numVertices entries of
 * 8 bytes, {uint32 packed 10:10:10 position within the block, uint32 block id}
 * (compute_block_vertices.comp:164).  The pointer stays valid until the next
 * bcmc_compute_surface on this volume; BCMC_E_STATE after a
 * bcmc_compute_surface_host. */
bcmc_status bcmc_vertices(bcmc_vol* vol, const void** d_vertices, uint64_t* bytes);
/* Copies the vertex buffer into host memory (bytes <= 8*numVertices). */
bcmc_status bcmc_copy_vertices(bcmc_vol* vol, void* host, uint64_t bytes);

/* Fields the reference object exposes to its UI (js/bcmc.js:77-100),
 * updated at the same points of computeSurface as the reference updates them. */
typedef struct {
    uint32_t totalBlocks;
    uint32_t numActiveBlocks;
    uint32_t newDecompressed;
    uint32_t numBlocksWithVertices;
    uint32_t numVertices;
    uint32_t cacheSize;                /* lruCache.cacheSize                    */
    uint32_t displayNumSlotsAvailable; /* lruCache.displayNumSlotsAvailable     */
    uint32_t lastNumVertices;          /* return value of the last query        */
} bcmc_stats;
bcmc_status bcmc_stats_get(bcmc_vol* vol, bcmc_stats* out);

/* reportMemoryUse() (js/compressed_marching_cubes.js:366-430): bytes per
 * buffer class, plus what this implementation actually holds on the device. */
typedef struct {
    uint64_t compressedData, vertexBuffer, blockActive, blockRanges, activeBlockIDs,
        blocksWithVertices, blockVertexOffsets, cache, cachedItemSlots, slotData, scratch,
        deviceTotal;
} bcmc_memory;
bcmc_status bcmc_memory_report(bcmc_vol* vol, bcmc_memory* out);

/* lruCache.reset() (js/lru_cache.js:846-903). */
bcmc_status bcmc_cache_reset(bcmc_vol* vol);

/* Debug views of the last query (device pointers owned by the volume), used by
 * the parity tests.  Lengths come from bcmc_stats_get / totalBlocks. */
typedef struct {
    const float* d_block_ranges;        /* vec2 per block                         */
    const uint32_t* d_block_active;     /* u32 per block                          */
    const uint32_t* d_active_block_ids; /* numActiveBlocks, ascending             */
    const uint32_t* d_blocks_with_vertices; /* numBlocksWithVertices, indices into active ids */
    const uint32_t* d_block_vertex_offsets; /* exclusive scan of per-block counts */
    const uint32_t* d_new_item_ids;     /* newDecompressed, ascending             */
    bcmc_lru* lru;                      /* the volume's cache                     */
} bcmc_vol_views;
bcmc_status bcmc_volume_views(bcmc_vol* vol, bcmc_vol_views* out);

/* ---- LRUCache (js/lru_cache.js) ----------------------------------------- */
/* new LRUCache(device, scan, compact, initialSize, elementSize, totalElements)
 * (js/lru_cache.js:4-305).  elementSize must be a multiple of 4 bytes. */
bcmc_status bcmc_lru_create(bcmc_ctx* ctx, uint32_t initial_size, uint32_t element_size,
                            uint32_t total_elements, bcmc_lru** out);
void bcmc_lru_destroy(bcmc_lru* lru);
/* update(itemNeeded) -> [numNewItems, newItemIDs] (js/lru_cache.js:312-843).
 * d_item_needed: u32 per element (1 = needed).  *d_new_item_ids stays valid
 * until the next update. */
bcmc_status bcmc_lru_update(bcmc_lru* lru, const uint32_t* d_item_needed, uint32_t* num_new,
                            const uint32_t** d_new_item_ids);
/* reset() (js/lru_cache.js:846-903). */
bcmc_status bcmc_lru_reset(bcmc_lru* lru);
typedef struct {
    uint32_t cacheSize, totalElements, elementSize, displayNumSlotsAvailable;
    const int32_t* d_cached_item_slots; /* per element: slot or -1             */
    const uint32_t* d_slot_age;         /* per slot                            */
    const uint32_t* d_slot_available;   /* per slot                            */
    const int32_t* d_slot_item;         /* per slot: element or -1             */
    void* d_cache;                      /* cacheSize * elementSize bytes       */
    const uint32_t* d_last_sorted_slots; /* available slots, oldest first      */
    uint32_t lastNumSlotsAvailable;
} bcmc_lru_view;
bcmc_status bcmc_lru_view_get(bcmc_lru* lru, bcmc_lru_view* out);

/* ---- ExclusiveScanPipeline / ExclusiveScanner (js/exclusive_scan.js) ----- */
/* getAlignedSize(n) = alignTo(n, 512) (js/exclusive_scan.js:95-97). */
uint32_t bcmc_scan_aligned_size(uint32_t n);
/* scanner.scan(dataSize) (js/exclusive_scan.js:178-295): in-place exclusive
 * scan of d_data[0..n) (uint32, wrapping); when n < aligned_size, d_data[n]
 * receives the total.  Returns the total through *total (synchronous). */
bcmc_status bcmc_scan_exclusive_u32(bcmc_ctx* ctx, uint32_t* d_data, uint32_t n,
                                    uint32_t aligned_size, uint32_t* total);
/* Asynchronous form: d_out may equal d_in; the total lands in *d_total. */
bcmc_status bcmc_scan_exclusive_u32_async(bcmc_ctx* ctx, const uint32_t* d_in, uint32_t* d_out,
                                          uint32_t n, uint32_t* d_total, void* stream);
/* No counterpart in the reference.  The asynchronous scan above without a
 * context and without any device allocation, for callers that may not
 * allocate on the call (a runtime that owns all device memory through its own
 * pool, or one that cannot take an allocation's implicit synchronisation) or
 * hold no context.  Scratch is a fixed static array of 137,480 bytes (about
 * 134 KiB) per device, so n > BCMC_SCAN_NOALLOC_MAX_N returns BCMC_E_LIMIT
 * with nothing launched.  Runs in the calling thread's current CUDA context
 * (the device's primary context when none is current); `stream` NULL is the
 * legacy default stream (there is no context stream).  The first call in a
 * context does its one-time set-up there (looks up the scratch array's device
 * address in that context and the SM count), so make it before any stream
 * capture in that context; a new context (after a device reset, or one the
 * caller creates) gets its own set-up.  Calls on one device share the
 * scratch: calls that may run concurrently (other streams or threads without
 * ordering) race, and their results are undefined.  A look-back wait that
 * runs out of spins is not reported here (its prefixes are wrong and the call
 * still returns BCMC_OK); the context-based scans report BCMC_E_TIMEOUT.
 * Failures: BCMC_E_ARG (null pointers with n > 0), BCMC_E_CUDA (set-up or
 * launch). */
#define BCMC_SCAN_NOALLOC_MAX_N (1u << 26)
bcmc_status bcmc_scan_exclusive_u32_noalloc(const uint32_t* d_in, uint32_t* d_out, uint32_t n,
                                            uint32_t* d_total, void* stream);

/* ---- StreamCompact (js/stream_compact.js) ------------------------------- */
/* compactActiveIDs(numElements, isActive, offsets, output)
 * (js/stream_compact.js:56-165, shaders/stream_compact.comp:26-32):
 * out[offsets[i]] = i for every i < n with flags[i] != 0. */
bcmc_status bcmc_compact_ids(bcmc_ctx* ctx, uint32_t n, const uint32_t* d_flags,
                             const uint32_t* d_offsets, uint32_t* d_out, void* stream);
/* Fused scan + compaction of the ids of nonzero flags (no offsets buffer). */
bcmc_status bcmc_select_ids(bcmc_ctx* ctx, uint32_t n, const uint32_t* d_flags, uint32_t* d_out,
                            uint32_t* d_count, void* stream);

/* ---- RadixSorter (js/radix_sort_by_key.js) ------------------------------ */
/* getAlignedSize(n) = nextPow2(ceil(n/64))*64 (js/radix_sort_by_key.js:155-158). */
uint32_t bcmc_sort_aligned_size(uint32_t n);
/* sort(keys, values, size, reverse) (js/radix_sort_by_key.js:161-400): sorts
 * the (key, value) pairs d_keys/d_values[0..n) in place, ascending by key, or
 * descending when reverse != 0, with the reference's order among equal keys
 * (ascending: later 64-element chunks first, index order within a chunk;
 * descending: earlier chunks first, reverse index order within a chunk).
 * Keys equal to 0xFFFFFFFF are ordered by that rule too (the reference pads
 * with that value). */
bcmc_status bcmc_sort_pairs_u32(bcmc_ctx* ctx, uint32_t* d_keys, uint32_t* d_values, uint32_t n,
                                int reverse, void* stream);

/* ---- ZFP fixed-rate float32 codec (shaders/zfp_decompress.comp) ---------- */
/* d_words in the calls below is a device buffer of at least
 * (blocks in the volume) * rate 64-bit words: block b occupies words
 * [b*rate, (b+1)*rate).  There is no length argument -- the kernels read every
 * block they are asked for -- so a shorter buffer is read out of bounds. */
/* zfp_compute_block_range.comp:19-61: vec2(min,max) of every block over the
 * voxels inside dims. */
bcmc_status bcmc_zfp_block_ranges(bcmc_ctx* ctx, const uint64_t* d_words, const uint32_t dims[3],
                                  uint32_t rate, float* d_ranges, void* stream);
/* zfp_decompress_block.comp:29-39: decode block d_block_ids[i] into
 * d_cache[64*d_item_slots[d_block_ids[i]] ...] for i < n. */
bcmc_status bcmc_zfp_decode_blocks(bcmc_ctx* ctx, const uint64_t* d_words, uint32_t rate,
                                   const uint32_t* d_block_ids, uint32_t n,
                                   const int32_t* d_item_slots, float* d_cache, void* stream);
/* Decode every block into d_out[64*b ...] (block order). */
bcmc_status bcmc_zfp_decode_volume(bcmc_ctx* ctx, const uint64_t* d_words, uint64_t nblocks,
                                   uint32_t rate, float* d_out, void* stream);
/* Fixed-rate encoder (no counterpart in the reference, which only decodes):
 * d_field is float32 x-fastest of dims; writes bcmc_zfp_stream_words() words. */
uint64_t bcmc_zfp_stream_words(const uint32_t dims[3], uint32_t rate);
bcmc_status bcmc_zfp_encode(bcmc_ctx* ctx, const float* d_field, const uint32_t dims[3],
                            uint32_t rate, uint64_t* d_words, void* stream);

/* The vertex stage's position math (mc_isosurface.vert:51-60,
 * block_vertex_position.comp:19-26) for n packed vertices of a volume of
 * `dims` and voxel `scale` (NULL = 1): d_world receives 3 floats per vertex,
 * scale * ((4 * block + q * 4 / 1023 + 0.5) / dims - 0.5).  When proj_view
 * (16 floats, column-major, host memory) and d_clip are given, d_clip receives
 * proj_view * (world, 1), 4 floats per vertex.  bcmc_render below is the
 * render pass that consumes them. */
bcmc_status bcmc_unpack_vertices(bcmc_ctx* ctx, const void* d_vertices, uint64_t n, const uint32_t dims[3],
                                 const float scale[3], float* d_world, const float* proj_view, float* d_clip,
                                 void* stream);

/* Headless render pass of the mesh (js/bcmc.js:174-190,237-265,377-391 with
 * shaders/mc_isosurface.vert/.frag): n packed vertices (n/3 triangles, in draw
 * order) into a width x height image.  The image is cleared to (1, 1, 1, 1)
 * and depth 1.0; a fragment is kept when its depth is in [0, 1) and less than
 * the stored depth ("less"), the earlier triangle winning ties as in an
 * in-order pipeline.  Pixel centres at (x + 0.5, y + 0.5), row 0 at the top
 * (NDC y = +1), depth = NDC z; edges follow the top-left rule.  Shading:
 * flat normal flipped toward the eye, Blinn-Phong with base colour
 * (0.3, 0.3, 0.9) and a head light, and with `fog` the depth-cueing fog toward
 * white from where the eye ray enters the volume's box.  A triangle with a
 * vertex at clip w <= 1e-6 is not drawn (no near-plane clipping).
 * d_rgba: width*height*4 floats, row-major, 16-byte aligned; d_depth (may be
 * NULL): width*height floats; d_triangle (may be NULL): per pixel the index
 * of the triangle drawn there, 0xFFFFFFFF for background.  The working
 * buffers (world and clip positions, one 64-bit depth/triangle key per pixel)
 * are the context's, grown on demand and kept; the call returns after the
 * stream has finished the pass, so calls on one context must not overlap. 
 * No counterpart as a function in the reference, whose render pass is a
 * WebGPU render pipeline. */
typedef struct bcmc_render_params {
    uint32_t width, height;
    float proj_view[16]; /* column-major, as ViewParams.proj_view */
    float eye_pos[3];    /* ViewParams.eye_pos */
    int32_t fog;         /* DRAW_FOG */
} bcmc_render_params;
bcmc_status bcmc_render(bcmc_ctx* ctx, const void* d_vertices, uint64_t n, const uint32_t dims[3],
                        const float scale[3], const bcmc_render_params* params, float* d_rgba, float* d_depth,
                        uint32_t* d_triangle, void* stream);

/* compute_block_active.comp:24-61: u32 active flag per block. */
bcmc_status bcmc_block_active(bcmc_ctx* ctx, const float* d_ranges, const uint32_t dims[3],
                              float isovalue, uint32_t* d_active, void* stream);

/* ---- Batched engine ------------------------------------------------------ */
/* No counterpart in the reference, which runs one computeSurface at a time per
 * volume.  An engine holds several compressed volumes resident on one device
 * and one pool of decoded-block slots shared by all of them, and answers a
 * batch of (volume, isovalue) queries with a fixed, device-driven launch
 * sequence: every query's active test and compaction in one persistent launch,
 * the decode of every block some query needs and no slot holds, every query's
 * marching cubes in one persistent launch.  Each query's vertices are the
 * vertices the plain path (bcmc_compute_surface on that volume) returns for it,
 * bit for bit and in the same order: the mesh depends only on the decoded
 * values of the active blocks, not on which slots hold them.  Slots are reused
 * across batches and evicted least-recently-used when the pool is full. */
typedef struct bcmc_engine bcmc_engine;
typedef struct {
    uint64_t pool_slots;       /* decoded-block slots (256 B each); 0 = every block of every volume */
    uint64_t vertex_capacity;  /* initial vertices per batch (grows on demand); 0 = 1<<24 */
    uint64_t vertex_budget;    /* admission: a launch sequence whose vertex count (known after its
                                  count pass) exceeds this runs as two halves; 0 = no limit */
    uint32_t max_batch;        /* queries per launch sequence; 0 = 1024 (larger batches are split) */
    uint32_t flags;            /* reserved, 0 */
} bcmc_engine_opts;
typedef struct {
    uint32_t volume;  /* id from bcmc_engine_add_volume */
    float isovalue;
} bcmc_query;
typedef struct {
    uint64_t vertex_offset;     /* first vertex of this query in the batch vertex buffer */
    uint32_t num_vertices;
    uint32_t num_active_blocks;
} bcmc_query_result;
typedef struct {
    uint64_t batches, launch_sequences, queries, decoded_blocks, evicted_blocks;
    uint64_t pool_slots, pool_used, vertex_capacity, device_bytes;
    double last_batch_ms;       /* device time of the last batch (CUDA events) */
    uint64_t overlapped_batches; /* server batches launched while another batch was on the device */
} bcmc_engine_stats;

bcmc_status bcmc_engine_create(bcmc_ctx* ctx, const bcmc_engine_opts* opts, bcmc_engine** out);
void bcmc_engine_destroy(bcmc_engine* eng);
/* Uploads a fixed-rate ZFP stream (host bytes, as bcmc_volume_create) and
 * computes its block ranges; *volume receives its id. */
bcmc_status bcmc_engine_add_volume(bcmc_engine* eng, const uint8_t* zfp, size_t len, uint32_t rate,
                                   const uint32_t dims[3], uint32_t* volume);
/* Runs n queries (split into launch sequences of at most max_batch) and blocks
 * until their vertex counts are known.  results[i] locates query i's vertices
 * in the batch vertex buffer (valid until the next run on this engine). */
bcmc_status bcmc_engine_run(bcmc_engine* eng, const bcmc_query* queries, uint32_t n,
                            bcmc_query_result* results);
/* Admission by memory: runs the longest prefix of queries[0..n) that the slot
 * pool and the vertex budget hold (at least queries[0], else
 * BCMC_E_ADMISSION) and sets *admitted to its length; the caller resubmits the
 * rest.  Vertex counts come from the count pass, before any vertex of a
 * refused query is kept. */
bcmc_status bcmc_engine_run_admit(bcmc_engine* eng, const bcmc_query* queries, uint32_t n,
                                  bcmc_query_result* results, uint32_t* admitted);
/* The batch vertex buffer of the last run: 8 bytes per vertex, laid out as the
 * plain path's (packed 10:10:10 position, block id). */
bcmc_status bcmc_engine_vertices(bcmc_engine* eng, const void** d_vertices, uint64_t* count);
bcmc_status bcmc_engine_copy_vertices(bcmc_engine* eng, uint64_t first, uint64_t count, void* host);
bcmc_status bcmc_engine_stats_get(bcmc_engine* eng, bcmc_engine_stats* out);
/* Autotuner: for the batch-size bucket of min(n, max_batch) queries, times the
 * launch sequence on these queries (device time, best of 3, CUDA events) over
 * the CTAs per SM of the active test and of the MC kernel (coordinate descent
 * from the defaults), and times a decode probe over up to 2^18 blocks of the
 * largest volume for the decode kernel's threads per CTA and CTAs per SM.  The
 * MC kernel's tile (active blocks per CTA tile: 8, 16 or 32, each a compiled
 * instance of the kernel) is tuned first, then its CTAs per SM.  The chosen
 * parameters are used (and captured into that bucket's graph) from then on.
 * The engine has no sort (its pool hands out free slots instead of the LRU's
 * age order), so no radix digit width is tuned here. */
typedef struct {
    uint32_t bucket;
    int32_t act_ctas_per_sm, decode_threads, decode_ctas_per_sm, mc_ctas_per_sm;
    double batch_ms_default, batch_ms_tuned, decode_ms_default, decode_ms_tuned;
    int32_t mc_blocks_per_tile;
} bcmc_tune_report;
bcmc_status bcmc_engine_autotune(bcmc_engine* eng, const bcmc_query* queries, uint32_t n,
                                 bcmc_tune_report* out);
/* Applies a tune report's launch parameters to its bucket (for instance one
 * saved from an earlier bcmc_engine_autotune), without timing anything.  The
 * timing fields are ignored.  BCMC_E_ARG for a bucket that is not a power of
 * two up to max_batch or a parameter outside the autotuner's choices. */
bcmc_status bcmc_engine_set_tuning(bcmc_engine* eng, const bcmc_tune_report* cfg);

/* ---- Isosurface server ----------------------------------------------------- */
/* No counterpart in the reference.  A request loop over an engine: a worker
 * thread takes every request that has arrived (up to max_batch) whenever the
 * device is free and runs them as one batch, so requests arriving while a
 * batch runs join the next one (continuous batching).  Each batch is admitted
 * by the engine's slot pool and vertex budget: a batch that does not fit runs
 * as smaller sequences.  Every request's vertices are those of the plain path.
 * While a server exists, only the server uses its engine. */
typedef struct bcmc_server bcmc_server;
typedef struct {
    uint32_t max_batch;    /* requests per batch; 0 = 256 */
    uint32_t max_wait_us;  /* an under-full batch waits this long for more arrivals; 0 = none */
} bcmc_server_opts;
bcmc_status bcmc_server_create(bcmc_engine* eng, const bcmc_server_opts* opts, bcmc_server** out);
/* Finishes the requests already submitted, then stops the worker. */
void bcmc_server_destroy(bcmc_server* srv);
/* Queues one request.  When host_vertices is not NULL the request's vertices
 * (8 bytes each, at most host_capacity of them) are copied there before the
 * request completes.  A volume id the engine does not hold returns
 * BCMC_E_ARG at once (nothing is queued). */
bcmc_status bcmc_server_submit(bcmc_server* srv, uint32_t volume, float isovalue, void* host_vertices,
                               uint64_t host_capacity, uint64_t* ticket);
/* Blocks until the request completes.  result->vertex_offset is 0 (batch
 * buffers are reused); latency_ms = completion - submission, wall clock.
 * Each ticket is waited for once: a ticket never issued or already waited
 * for returns BCMC_E_ARG at once. */
bcmc_status bcmc_server_wait(bcmc_server* srv, uint64_t ticket, bcmc_query_result* result,
                             double* latency_ms);
/* Open-loop load: `requests` arrivals with exponential inter-arrival times at
 * rate_qps (seeded), each on volume volumes[i] with probability weights[i] and
 * an isovalue uniform in [iso_lo[i], iso_hi[i]]; reports throughput and
 * latency percentiles of the completed requests. */
typedef struct {
    double rate_qps;
    uint32_t requests;
    uint32_t num_volumes;
    uint64_t seed;
    const uint32_t* volumes;
    const float* weights;
    const float* iso_lo;
    const float* iso_hi;
} bcmc_load_spec;
typedef struct {
    double offered_qps, achieved_qps, p50_ms, p95_ms, p99_ms, mean_ms, max_ms, mean_batch, duration_s;
    uint64_t completed, batches, vertices;
    uint64_t overlapped_batches; /* batches launched while the previous one was still on the device */
} bcmc_load_report;
bcmc_status bcmc_server_run_load(bcmc_server* srv, const bcmc_load_spec* spec, bcmc_load_report* out);

#ifdef __cplusplus
}
#endif
#endif
