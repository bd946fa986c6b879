// api.cu -- host objects and the C ABI of libbcmc_gb300 (include/bcmc.h).
//
// bcmc_vol mirrors CompressedMarchingCubes (js/compressed_marching_cubes.js),
// bcmc_lru mirrors LRUCache (js/lru_cache.js).  A query launches the fixed
// kernel sequence of pipeline.cu and reads the QueryState back once; the only
// host decisions left are physical growth of the cache buffers (the logical
// cache size follows the reference's rule on the device) and of the vertex
// buffer, each followed by a re-run of the affected launches.
#include <algorithm>
#include <utility>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>

#include "bcmc_pipeline.h"

using namespace bcmc;

namespace bcmc {

void* dev_alloc(bcmc_ctx* ctx, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw CudaError{e, "cudaMalloc"};
    }
    ctx->device_bytes += bytes;
    return p;
}

void dev_free(bcmc_ctx* ctx, void* p, size_t bytes)
{
    if (!p) return;
    cudaFree(p);
    if (bytes == 0) bytes = 16;
    ctx->device_bytes -= bytes;
}

void ensure_status(bcmc_ctx* ctx, size_t words)
{
    if (words <= ctx->status_words) return;
    BCMC_CUDA(cudaStreamSynchronize(ctx->stream));
    dev_free(ctx, ctx->d_status, ctx->status_words * 8);
    ctx->d_status = nullptr;
    ctx->status_words = 0;
    ctx->d_status = (uint64_t*)dev_alloc(ctx, words * 8);
    BCMC_CUDA(cudaMemsetAsync(ctx->d_status, 0, words * 8, ctx->stream));
    ctx->status_words = words;
}

void ensure_scratch(bcmc_ctx* ctx, size_t words)
{
    if (words <= ctx->scratch_words) return;
    BCMC_CUDA(cudaStreamSynchronize(ctx->stream));
    dev_free(ctx, ctx->d_scratch, ctx->scratch_words * 4);
    ctx->d_scratch = nullptr;
    ctx->scratch_words = 0;
    ctx->d_scratch = (uint32_t*)dev_alloc(ctx, words * 4);
    ctx->scratch_words = words;
}

}  // namespace bcmc

std::atomic<uint64_t> bcmc::g_kernel_launches{0};

// ---------------------------------------------------------------------------
// error plumbing
// ---------------------------------------------------------------------------
static bcmc_status fail(bcmc_ctx* ctx, bcmc_status st, const std::string& msg)
{
    if (ctx) ctx->last_error = msg;
    return st;
}

template <typename F>
static bcmc_status guarded(bcmc_ctx* ctx, F&& f)
{
    try {
        return f();
    } catch (const CudaError& e) {
        const bcmc_status st = (e.err == cudaErrorMemoryAllocation) ? BCMC_E_OOM : BCMC_E_CUDA;
        return fail(ctx, st, std::string(e.what) + ": " + cudaGetErrorString(e.err));
    } catch (const std::bad_alloc&) {
        return fail(ctx, BCMC_E_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(ctx, BCMC_E_CUDA, e.what());
    }
}

static cudaStream_t pick(bcmc_ctx* ctx, void* stream) { return stream ? (cudaStream_t)stream : ctx->stream; }

static void ctx_release(bcmc_ctx* ctx)
{
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, ctx->d_prim, sizeof(QueryState));
    dev_free(ctx, ctx->d_status, ctx->status_words * 8);
    dev_free(ctx, ctx->d_scratch, ctx->scratch_words * 4);
    dev_free(ctx, ctx->d_render, ctx->render_bytes);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

// A context outlives the volumes and caches made from it, whatever order the
// caller destroys them in (garbage collectors finalize in arbitrary order).
void bcmc::ctx_child_added(bcmc_ctx* ctx) { ++ctx->children; }
void bcmc::ctx_child_removed(bcmc_ctx* ctx)
{
    if (--ctx->children == 0 && ctx->destroy_pending) ctx_release(ctx);
}

// Keeps the look-back epochs of one QueryState away from wrap-around: every
// 2^26 calls the status words are cleared and the epoch restarts.
struct EpochGuard {
    uint64_t calls = 0;
};

// ---------------------------------------------------------------------------
// LRU cache object
// ---------------------------------------------------------------------------
struct bcmc_lru {
    bcmc_ctx* ctx = nullptr;
    uint32_t total = 0, aligned_total = 0, element_size = 0;
    uint32_t capacity = 0;  // physical slots
    uint32_t cache_size = 0, display_slots = 0;
    int32_t* item_slots = nullptr;  // aligned_total
    uint32_t* slot_age = nullptr;
    uint32_t* slot_avail = nullptr;
    int32_t* slot_item = nullptr;
    uint8_t* cache = nullptr;  // capacity * element_size
    uint32_t* new_ids = nullptr;  // total
    uint32_t* avail_ids = nullptr;
    uint32_t* avail_keys = nullptr;
    uint32_t* sort_bk = nullptr;
    uint32_t* sort_bv = nullptr;
    uint32_t* sort_ck = nullptr;
    uint32_t* sort_cv = nullptr;
    // age bins: joint histogram and dense ranks (k_slots' one-pass sort plan)
    uint32_t* age_hist = nullptr;
    uint8_t* age_rank = nullptr;
    uint64_t* status = nullptr;
    size_t status_words = 0;
    uint64_t* st_active_a = nullptr;
    uint64_t* st_active_n = nullptr;
    uint64_t* st_slots = nullptr;
    uint64_t* st_sort = nullptr;
    uint64_t* st_mc_v = nullptr;
    uint64_t* st_mc_b = nullptr;
    QueryState* q = nullptr;
    QueryState* h_q = nullptr;  // pinned
    uint64_t epoch_calls = 0;
    uint32_t last_num_new = 0, last_num_avail = 0;
};

static size_t slot_array_bytes(uint32_t cap) { return (size_t)cap * 4u; }

// k_slots leaves the age histogram zero after every update; it is cleared
// here when an update may not have finished (a wait gave up)
static void lru_clear_key16(bcmc_lru* c, cudaStream_t s)
{
    BCMC_CUDA(cudaMemsetAsync(c->age_hist, 0, (size_t)kAgeBins * 4, s));
}

static void lru_alloc_slots(bcmc_lru* c, uint32_t cap)
{
    bcmc_ctx* ctx = c->ctx;
    c->slot_age = (uint32_t*)dev_alloc(ctx, slot_array_bytes(cap));
    c->slot_avail = (uint32_t*)dev_alloc(ctx, slot_array_bytes(cap));
    c->slot_item = (int32_t*)dev_alloc(ctx, slot_array_bytes(cap));
    c->cache = (uint8_t*)dev_alloc(ctx, (size_t)cap * c->element_size);
    c->avail_ids = (uint32_t*)dev_alloc(ctx, slot_array_bytes(cap));
    c->avail_keys = (uint32_t*)dev_alloc(ctx, slot_array_bytes(cap));
    c->sort_bk = (uint32_t*)dev_alloc(ctx, slot_array_bytes(cap));
    c->sort_bv = (uint32_t*)dev_alloc(ctx, slot_array_bytes(cap));
    c->sort_ck = (uint32_t*)dev_alloc(ctx, slot_array_bytes(cap));
    c->sort_cv = (uint32_t*)dev_alloc(ctx, slot_array_bytes(cap));
    c->capacity = cap;
}

static void lru_free_slots(bcmc_lru* c)
{
    bcmc_ctx* ctx = c->ctx;
    const uint32_t cap = c->capacity;
    dev_free(ctx, c->slot_age, slot_array_bytes(cap));
    dev_free(ctx, c->slot_avail, slot_array_bytes(cap));
    dev_free(ctx, c->slot_item, slot_array_bytes(cap));
    dev_free(ctx, c->cache, (size_t)cap * c->element_size);
    dev_free(ctx, c->avail_ids, slot_array_bytes(cap));
    dev_free(ctx, c->avail_keys, slot_array_bytes(cap));
    dev_free(ctx, c->sort_bk, slot_array_bytes(cap));
    dev_free(ctx, c->sort_bv, slot_array_bytes(cap));
    dev_free(ctx, c->sort_ck, slot_array_bytes(cap));
    dev_free(ctx, c->sort_cv, slot_array_bytes(cap));
    c->slot_age = c->slot_avail = nullptr;
    c->slot_item = nullptr;
    c->cache = nullptr;
    c->avail_ids = c->avail_keys = c->sort_bk = c->sort_bv = c->sort_ck = c->sort_cv = nullptr;
    c->capacity = 0;
}

__global__ void k_lru_init_slots(uint32_t* age, uint32_t* avail, int32_t* item, uint32_t from, uint32_t to,
                                 int initial)
{
    for (uint32_t s = from + blockIdx.x * blockDim.x + threadIdx.x; s < to; s += gridDim.x * blockDim.x) {
        age[s] = initial ? 2u + s : 100000u;  // js/lru_cache.js:54-59 / lru_cache_init.comp:27-29
        avail[s] = 1u;
        item[s] = -1;
    }
}

__global__ void k_fill_i32(int32_t* p, uint32_t n, int32_t v)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

static int fill_grid(bcmc_ctx* ctx, uint32_t n)
{
    const uint32_t g = div_up(n ? n : 1, 256u), cap = (uint32_t)ctx->num_sms * 8u;
    return (int)(g < cap ? g : cap);
}

// Physical growth: copies the live slots and their cached data.
static void lru_grow_capacity(bcmc_lru* c, uint32_t needed)
{
    bcmc_ctx* ctx = c->ctx;
    uint64_t want = (uint64_t)c->capacity + c->capacity / 2u;
    if (want < needed) want = needed;
    if (want > c->aligned_total) want = c->aligned_total;
    const uint32_t new_cap = align_up((uint32_t)want, 32u);
    bcmc_lru old = *c;
    lru_alloc_slots(c, new_cap);
    const size_t live = c->cache_size;
    BCMC_CUDA(cudaMemcpyAsync(c->slot_age, old.slot_age, live * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    BCMC_CUDA(cudaMemcpyAsync(c->slot_avail, old.slot_avail, live * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    BCMC_CUDA(cudaMemcpyAsync(c->slot_item, old.slot_item, live * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    BCMC_CUDA(cudaMemcpyAsync(c->cache, old.cache, live * c->element_size, cudaMemcpyDeviceToDevice, ctx->stream));
    BCMC_CUDA(cudaStreamSynchronize(ctx->stream));
    bcmc_lru tmp = old;
    lru_free_slots(&tmp);
}

// Epoch rewind well before the 2^28 limit of the sort's status tags.
static void lru_epoch_tick(bcmc_lru* c, cudaStream_t s)
{
    if (++c->epoch_calls >= (1ull << 26)) {
        BCMC_CUDA(cudaMemsetAsync(c->status, 0, c->status_words * 8, s));
        BCMC_CUDA(cudaMemsetAsync(&c->q->epoch, 0, 4, s));
        c->epoch_calls = 1;
    }
}

static void lru_begin(bcmc_lru* c, cudaStream_t s, float iso, int mc_only, uint32_t vert_capacity)
{
    lru_epoch_tick(c, s);
    query_begin_launch(c->q, iso, mc_only, c->capacity, vert_capacity, s);
}

static bcmc_lru* lru_new(bcmc_ctx* ctx, uint32_t initial_size, uint32_t element_size, uint32_t total)
{
    bcmc_lru* c = new bcmc_lru();
    c->ctx = ctx;
    c->total = total;
    c->aligned_total = align_up(total, 32u);
    c->element_size = element_size;
    c->cache_size = align_up(initial_size, 32u);
    if (c->cache_size > c->aligned_total) c->cache_size = c->aligned_total;
    try {
        c->item_slots = (int32_t*)dev_alloc(ctx, (size_t)c->aligned_total * 4);
        c->new_ids = (uint32_t*)dev_alloc(ctx, (size_t)(total ? total : 1) * 4);
        lru_alloc_slots(c, c->cache_size ? c->cache_size : 32u);
        const size_t wa = active_tiles(total) + 1, ws = slot_tiles(c->aligned_total) + 1,
                     wsort = sort_status_words(c->aligned_total), wm = mc_grid(ctx, total) + 1;
        c->status_words = 2 * wa + ws + wsort + 2 * wm;
        c->status = (uint64_t*)dev_alloc(ctx, c->status_words * 8);
        c->st_active_a = c->status;
        c->st_active_n = c->st_active_a + wa;
        c->st_slots = c->st_active_n + wa;
        c->st_sort = c->st_slots + ws;
        c->st_mc_v = c->st_sort + wsort;
        c->st_mc_b = c->st_mc_v + wm;
        c->q = (QueryState*)dev_alloc(ctx, sizeof(QueryState));
        BCMC_CUDA(cudaMallocHost(&c->h_q, sizeof(QueryState)));
        c->age_hist = (uint32_t*)dev_alloc(ctx, (size_t)kAgeBins * 4);
        c->age_rank = (uint8_t*)dev_alloc(ctx, (size_t)kAgeBins);
        cudaStream_t s = ctx->stream;
        lru_clear_key16(c, s);
        BCMC_CUDA(cudaMemsetAsync(c->status, 0, c->status_words * 8, s));
        BCMC_CUDA(cudaMemsetAsync(c->q, 0, sizeof(QueryState), s));
        BCMC_CUDA(cudaMemcpyAsync(&c->q->cache_size, &c->cache_size, 4, cudaMemcpyHostToDevice, s));
        k_fill_i32<<<fill_grid(ctx, c->aligned_total), 256, 0, s>>>(c->item_slots, c->aligned_total, -1);
        count_launches(1);
        k_lru_init_slots<<<fill_grid(ctx, c->cache_size), 256, 0, s>>>(c->slot_age, c->slot_avail, c->slot_item,
                                                                       0, c->cache_size, 1);
        count_launches(1);
        BCMC_CUDA(cudaGetLastError());
        BCMC_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
        // release what was allocated, then report
        if (c->capacity) lru_free_slots(c);
        dev_free(ctx, c->item_slots, (size_t)c->aligned_total * 4);
        dev_free(ctx, c->new_ids, (size_t)(total ? total : 1) * 4);
        dev_free(ctx, c->status, c->status_words * 8);
        dev_free(ctx, c->q, sizeof(QueryState));
        if (c->h_q) cudaFreeHost(c->h_q);
        delete c;
        throw;
    }
    ctx_child_added(ctx);
    return c;
}

static void lru_delete(bcmc_lru* c)
{
    if (!c) return;
    bcmc_ctx* ctx = c->ctx;
    cudaStreamSynchronize(ctx->stream);
    lru_free_slots(c);
    dev_free(ctx, c->item_slots, (size_t)c->aligned_total * 4);
    dev_free(ctx, c->new_ids, (size_t)(c->total ? c->total : 1) * 4);
    dev_free(ctx, c->status, c->status_words * 8);
    dev_free(ctx, c->age_hist, (size_t)kAgeBins * 4);
    dev_free(ctx, c->age_rank, (size_t)kAgeBins);
    dev_free(ctx, c->q, sizeof(QueryState));
    if (c->h_q) cudaFreeHost(c->h_q);
    delete c;
    ctx_child_removed(ctx);
}

static SortBuffers lru_sort_buffers(bcmc_lru* c)
{
    SortBuffers b;
    b.in_keys = c->avail_keys;
    b.in_vals = c->avail_ids;
    b.b_keys = c->sort_bk;
    b.b_vals = c->sort_bv;
    b.c_keys = c->sort_ck;
    b.c_vals = c->sort_cv;
    b.status = c->st_sort;
    b.age_rank = c->age_rank;
    return b;
}

// update + LRU stages shared by the standalone cache and the volume query
static void lru_enqueue_update(bcmc_lru* c, cudaStream_t s, const uint32_t* needed, const uint64_t* words,
                               uint32_t max_bits)
{
    bcmc_ctx* ctx = c->ctx;
    SlotArgs sa{needed,    c->slot_age, c->slot_avail, c->slot_item, c->avail_ids, c->avail_keys, c->st_slots, 0u, 1u,
                c->age_hist, c->age_rank};
    slots_launch(ctx, c->q, sa, c->capacity, s);
    sort_launch(ctx, c->q, &c->q->num_avail, c->capacity, lru_sort_buffers(c), 1, s, /*plan_ready=*/1);
    AssignArgs aa{c->new_ids, c->sort_bv,   c->sort_cv, c->slot_age, c->slot_avail, c->slot_item,
                  c->item_slots, words, max_bits, reinterpret_cast<float*>(c->cache)};
    assign_launch(ctx, c->q, aa, c->total, s);
}

static void lru_read_state(bcmc_lru* c, cudaStream_t s)
{
    BCMC_CUDA(cudaMemcpyAsync(c->h_q, c->q, sizeof(QueryState), cudaMemcpyDeviceToHost, s));
    BCMC_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// volume
// ---------------------------------------------------------------------------
// device vertex buffers a query sequence into host memory cycles through
constexpr int kVertRing = 4;

struct bcmc_vol {
    bcmc_ctx* ctx = nullptr;
    uint32_t dims[3]{}, nb[3]{}, total = 0, rate = 0, max_bits = 0;
    float scale[3]{};
    uint64_t* words = nullptr;
    uint64_t nwords = 0;
    size_t compressed_bytes = 0;
    float* ranges = nullptr;
    uint32_t* active = nullptr;
    uint32_t* active_ids = nullptr;
    uint32_t* with_verts = nullptr;
    uint32_t* vert_offsets = nullptr;
    uint32_t* block_counts = nullptr;
    uint2* verts = nullptr;
    uint32_t vert_capacity = 0;
    uint32_t verts_storage = 0;  // the reference's numVerticesStorage
    // a ring of device vertex buffers for query sequences into host memory
    // (bcmc_compute_surfaces_host): a query computes into one while the
    // vertices of the queries before it are copied out of the others.
    // `verts` is ring[cur]; the other entries hold the rest of the ring.
    uint2* ring[kVertRing]{};
    uint32_t ring_cap[kVertRing]{};
    int cur = 0;
    cudaStream_t copy = nullptr;
    cudaEvent_t copy_ev[kVertRing]{};
    bcmc_lru* lru = nullptr;
    bcmc_stats stats{};
    cudaEvent_t ev[5]{};
    // the query as one CUDA graph: inputs copied from pinned memory, state
    // copied back to pinned memory; re-captured when a buffer is regrown
    QueryInputs* h_in = nullptr;  // pinned
    // [0]: without the stage-timing events, [1]: with them (a perf tracker),
    // [2]: vertices written straight into a page-locked host buffer, [2 + r]:
    // as [0] while ring buffer r (r >= 1) is the current vertex buffer
    cudaGraphExec_t graph[2 + kVertRing]{};
    uint64_t graph_key[2 + kVertRing][4]{};
    bool last_on_host = false;  // the last query's vertices went to host memory only
    uint64_t graph_kernels = 0;
    // the new blocks' decode runs on a branch of the query graph, beside the
    // LRU's slot selection, into `stage` (stage_blocks elements of 256 B)
    float* stage = nullptr;
    uint32_t stage_blocks = 0;
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
};

// new blocks a query stages at most (32 MiB); k_assign decodes any beyond
constexpr uint32_t kStageBlocksMax = 1u << 17;

static void vol_free(bcmc_vol* v)
{
    if (!v) return;
    bcmc_ctx* ctx = v->ctx;
    cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, v->words, v->nwords * 8);
    dev_free(ctx, v->ranges, (size_t)v->total * 8);
    dev_free(ctx, v->active, (size_t)v->total * 4);
    dev_free(ctx, v->active_ids, (size_t)v->total * 4);
    dev_free(ctx, v->with_verts, (size_t)v->total * 4);
    dev_free(ctx, v->vert_offsets, (size_t)v->total * 4);
    dev_free(ctx, v->block_counts, (size_t)v->total * 4);
    if (v->copy) cudaStreamSynchronize(v->copy);
    dev_free(ctx, v->verts, (size_t)v->vert_capacity * 8);
    for (int r = 0; r < kVertRing; ++r)
        if (r != v->cur) dev_free(ctx, v->ring[r], (size_t)v->ring_cap[r] * 8);
    dev_free(ctx, v->stage, (size_t)v->stage_blocks * 256u);
    lru_delete(v->lru);
    for (auto& e : v->ev)
        if (e) cudaEventDestroy(e);
    if (v->fork_ev) cudaEventDestroy(v->fork_ev);
    if (v->join_ev) cudaEventDestroy(v->join_ev);
    if (v->side) cudaStreamDestroy(v->side);
    for (auto& e : v->copy_ev)
        if (e) cudaEventDestroy(e);
    if (v->copy) cudaStreamDestroy(v->copy);
    for (auto& g : v->graph)
        if (g) cudaGraphExecDestroy(g);
    if (v->h_in) cudaFreeHost(v->h_in);
    delete v;
    ctx_child_removed(ctx);
}

static void vol_grow_verts(bcmc_vol* v, uint32_t needed)
{
    bcmc_ctx* ctx = v->ctx;
    // compressed_marching_cubes.js:774-786: storage = max(needed, 1.5 * storage)
    uint64_t st = (uint64_t)v->verts_storage * 3u / 2u;
    if (st < needed) st = needed;
    if (st > 0xffffffffull) st = 0xffffffffull;
    BCMC_CUDA(cudaStreamSynchronize(ctx->stream));
    if (v->copy) BCMC_CUDA(cudaStreamSynchronize(v->copy));  // a transfer may still read it
    dev_free(ctx, v->verts, (size_t)v->vert_capacity * 8);
    v->verts = nullptr;
    v->vert_capacity = 0;
    v->verts = (uint2*)dev_alloc(ctx, (size_t)st * 8);
    v->vert_capacity = (uint32_t)st;
    v->verts_storage = (uint32_t)st;
}

static bcmc_status vol_create_common(bcmc_ctx* ctx, const void* src, bool src_device, size_t len, uint32_t rate,
                                     const uint32_t dims[3], const float scale[3], bcmc_vol** out)
{
    if (!ctx || !src || !dims || !out) return fail(ctx, BCMC_E_ARG, "null argument");
    if (rate == 0 || rate > 32) return fail(ctx, BCMC_E_ARG, "rate must be in [1, 32] bits per value");
    if (dims[0] == 0 || dims[1] == 0 || dims[2] == 0) return fail(ctx, BCMC_E_ARG, "empty volume");
    uint32_t nb[3];
    for (int i = 0; i < 3; ++i) nb[i] = div_up(dims[i], 4u);
    const uint64_t total = (uint64_t)nb[0] * nb[1] * nb[2];
    if (total > 0x7fffffffull) return fail(ctx, BCMC_E_ARG, "volume has more than 2^31 blocks");
    const uint32_t max_bits = 64u * rate;
    const uint64_t need_bytes = (total * max_bits + 7u) / 8u;
    if (len < need_bytes) return fail(ctx, BCMC_E_ARG, "compressed stream shorter than blocks * 64 * rate bits");
    return guarded(ctx, [&]() -> bcmc_status {
        bcmc_vol* v = new bcmc_vol();
        v->ctx = ctx;
        ctx_child_added(ctx);  // vol_free removes it, also on the error path below
        for (int i = 0; i < 3; ++i) {
            v->dims[i] = dims[i];
            v->nb[i] = nb[i];
            v->scale[i] = scale ? scale[i] : 1.0f;
        }
        v->total = (uint32_t)total;
        v->rate = rate;
        v->max_bits = max_bits;
        v->compressed_bytes = len;
        try {
            cudaStream_t s = ctx->stream;
            // one zero word past the last block: the reader may prefetch it
            v->nwords = (len + 7u) / 8u + 2u;
            v->words = (uint64_t*)dev_alloc(ctx, v->nwords * 8);
            BCMC_CUDA(cudaMemsetAsync(v->words, 0, v->nwords * 8, s));
            BCMC_CUDA(cudaMemcpyAsync(v->words, src, len, src_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
            v->ranges = (float*)dev_alloc(ctx, (size_t)total * 8);
            v->active = (uint32_t*)dev_alloc(ctx, (size_t)total * 4);
            v->active_ids = (uint32_t*)dev_alloc(ctx, (size_t)total * 4);
            v->with_verts = (uint32_t*)dev_alloc(ctx, (size_t)total * 4);
            v->vert_offsets = (uint32_t*)dev_alloc(ctx, (size_t)total * 4);
            v->block_counts = (uint32_t*)dev_alloc(ctx, (size_t)total * 4);
            const uint32_t init_slots =
                (uint32_t)std::min<double>((double)total, std::ceil((double)total * ctx->opts.initial_cache_fraction));
            v->lru = lru_new(ctx, init_slots, 256u, (uint32_t)total);
            const uint32_t init_verts = 1u << 20;
            v->verts = (uint2*)dev_alloc(ctx, (size_t)init_verts * 8);
            v->vert_capacity = init_verts;
            v->verts_storage = 0;
            for (auto& e : v->ev) BCMC_CUDA(cudaEventCreate(&e));
            BCMC_CUDA(cudaMallocHost(&v->h_in, sizeof(QueryInputs)));
            v->stage_blocks = (uint32_t)std::min<uint64_t>(total, kStageBlocksMax);
            v->stage = (float*)dev_alloc(ctx, (size_t)v->stage_blocks * 256u);
            BCMC_CUDA(cudaStreamCreateWithFlags(&v->side, cudaStreamNonBlocking));
            BCMC_CUDA(cudaEventCreateWithFlags(&v->fork_ev, cudaEventDisableTiming));
            BCMC_CUDA(cudaEventCreateWithFlags(&v->join_ev, cudaEventDisableTiming));
            zfp_ranges_launch(ctx, v->words, v->dims, max_bits, v->ranges, s);
            BCMC_CUDA(cudaStreamSynchronize(s));
            v->stats.totalBlocks = v->total;
            v->stats.cacheSize = v->lru->cache_size;
        } catch (...) {
            vol_free(v);
            throw;
        }
        *out = v;
        return BCMC_OK;
    });
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

uint64_t bcmc_kernel_launches(void) { return g_kernel_launches.load(std::memory_order_relaxed); }

void bcmc_opts_default(bcmc_opts* o)
{
    if (!o) return;
    o->device = 0;
    o->initial_cache_fraction = 0.05;
    o->flags = 0;
}

bcmc_status bcmc_ctx_create(const bcmc_opts* opts, bcmc_ctx** out)
{
    if (!out) return BCMC_E_ARG;
    *out = nullptr;
    bcmc_ctx* ctx = new (std::nothrow) bcmc_ctx();
    if (!ctx) return BCMC_E_OOM;
    if (opts) ctx->opts = *opts;
    else bcmc_opts_default(&ctx->opts);
    if (!(ctx->opts.initial_cache_fraction > 0.0) || ctx->opts.initial_cache_fraction > 1.0 ||
        (ctx->opts.flags & ~BCMC_FLAG_FULL_RANGES) != 0) {
        delete ctx;
        return BCMC_E_ARG;
    }
    const bcmc_status st = guarded(ctx, [&]() -> bcmc_status {
        int n = 0;
        BCMC_CUDA(cudaGetDeviceCount(&n));
        if (ctx->opts.device < 0 || ctx->opts.device >= n) return fail(ctx, BCMC_E_ARG, "no such CUDA device");
        ctx->device = ctx->opts.device;
        BCMC_CUDA(cudaSetDevice(ctx->device));
        BCMC_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device));
        BCMC_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->d_prim = (QueryState*)dev_alloc(ctx, sizeof(QueryState));
        BCMC_CUDA(cudaMemset(ctx->d_prim, 0, sizeof(QueryState)));
        BCMC_CUDA(cudaMallocHost(&ctx->h_pinned, 4096));
        return BCMC_OK;
    });
    if (st != BCMC_OK) {
        bcmc_ctx_destroy(ctx);
        return st;
    }
    *out = ctx;
    return BCMC_OK;
}

void bcmc_ctx_destroy(bcmc_ctx* ctx)
{
    if (!ctx) return;
    if (ctx->children > 0) {
        ctx->destroy_pending = true;  // released with its last volume / cache
        return;
    }
    ctx_release(ctx);
}

const char* bcmc_last_error(const bcmc_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

bcmc_status bcmc_debug_drop_tile(bcmc_ctx* ctx, uint32_t tile_plus_one)
{
    if (!ctx) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        ctx->debug_drop_tile = tile_plus_one;
        BCMC_CUDA(cudaMemcpyAsync(&ctx->d_prim->debug_drop_tile, &ctx->debug_drop_tile, 4, cudaMemcpyHostToDevice,
                                  ctx->stream));
        BCMC_CUDA(cudaStreamSynchronize(ctx->stream));
        return BCMC_OK;
    });
}

void* bcmc_ctx_stream(bcmc_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

bcmc_status bcmc_ctx_synchronize(bcmc_ctx* ctx)
{
    if (!ctx) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        BCMC_CUDA(cudaStreamSynchronize(ctx->stream));
        return BCMC_OK;
    });
}

bcmc_status bcmc_volume_create(bcmc_ctx* ctx, const uint8_t* zfp, size_t len, uint32_t rate, const uint32_t dims[3],
                               const float scale[3], bcmc_vol** out)
{
    return vol_create_common(ctx, zfp, false, len, rate, dims, scale, out);
}

bcmc_status bcmc_volume_create_device(bcmc_ctx* ctx, const void* d_zfp, size_t len, uint32_t rate,
                                      const uint32_t dims[3], const float scale[3], bcmc_vol** out)
{
    return vol_create_common(ctx, d_zfp, true, len, rate, dims, scale, out);
}

void bcmc_volume_destroy(bcmc_vol* v) { vol_free(v); }

// The kernels of one query, in order, on stream s (captured into the graph).
static void vol_enqueue_query(bcmc_vol* v, cudaStream_t s, float iso, int from_state, bool events, uint2* out)
{
    bcmc_ctx* ctx = v->ctx;
    bcmc_lru* c = v->lru;
    const uint3 nb = make_uint3(v->nb[0], v->nb[1], v->nb[2]);
    const BlockGrid grid = make_block_grid(nb);
    ActiveArgs aa{reinterpret_cast<const float2*>(v->ranges), nb, grid, nullptr, v->active, c->item_slots,
                  v->total, v->active_ids, c->new_ids, c->st_active_a, c->st_active_n};
    McArgs ma{v->active, v->active_ids, c->item_slots, reinterpret_cast<const float*>(c->cache), nb, grid,
              v->with_verts, v->vert_offsets, v->block_counts, out, c->st_mc_v, c->st_mc_b, out != v->verts ? 1u : 0u};
    SlotArgs sa{v->active,  c->slot_age, c->slot_avail, c->slot_item, c->avail_ids, c->avail_keys, c->st_slots, 1u, 1u,
                c->age_hist, c->age_rank};
    AssignArgs as{c->new_ids, c->sort_bv, c->sort_cv, c->slot_age, c->slot_avail, c->slot_item,
                  c->item_slots, v->words, v->max_bits, reinterpret_cast<float*>(c->cache), v->stage, v->stage_blocks};
    DecodeArgs da{c->new_ids, v->words, v->max_bits, v->stage, v->stage_blocks};
    if (events) BCMC_CUDA(cudaEventRecordWithFlags(v->ev[0], s, cudaEventRecordExternal));
    query_begin_launch(c->q, iso, 0, c->capacity, v->vert_capacity, s, from_state ? v->h_in : nullptr);
    active_launch(ctx, c->q, aa, s);
    if (events) BCMC_CUDA(cudaEventRecordWithFlags(v->ev[1], s, cudaEventRecordExternal));
    // branch: the new blocks' decode into the staging buffer needs only the
    // active test's new ids, so it overlaps the slot selection below
    BCMC_CUDA(cudaEventRecord(v->fork_ev, s));
    slots_launch(ctx, c->q, sa, c->capacity, s);
    BCMC_CUDA(cudaStreamWaitEvent(v->side, v->fork_ev, 0));
    decode_new_launch(ctx, c->q, da, v->side);
    BCMC_CUDA(cudaEventRecord(v->join_ev, v->side));
    sort_launch(ctx, c->q, &c->q->num_avail, c->capacity, lru_sort_buffers(c), 1, s, /*plan_ready=*/1);
    if (events) BCMC_CUDA(cudaEventRecordWithFlags(v->ev[2], s, cudaEventRecordExternal));
    BCMC_CUDA(cudaStreamWaitEvent(s, v->join_ev, 0));
    assign_launch(ctx, c->q, as, v->total, s);
    if (events) BCMC_CUDA(cudaEventRecordWithFlags(v->ev[3], s, cudaEventRecordExternal));
    mc_launch(ctx, c->q, ma, v->total, s);
    if (events) BCMC_CUDA(cudaEventRecordWithFlags(v->ev[4], s, cudaEventRecordExternal));
    query_end_launch(c->q, c->h_q, s);
}

// Captures the query into a CUDA graph if the buffers it refers to changed.
// mode 0/1: the volume's vertex buffer without/with stage events; mode 2: the
// vertices go to `out` (the device address of a page-locked host buffer).
static int graph_slot(const bcmc_vol* v, int mode) { return mode == 0 && v->cur != 0 ? 2 + v->cur : mode; }

static void vol_ensure_graph(bcmc_vol* v, int mode, uint2* out = nullptr)
{
    bcmc_lru* c = v->lru;
    if (mode != 2) out = v->verts;
    const uint64_t key[4] = {c->capacity, mode == 2 ? 0u : v->vert_capacity, (uint64_t)(uintptr_t)out,
                             (uint64_t)(uintptr_t)c->cache};
    const int slot = graph_slot(v, mode);
    cudaGraphExec_t& graph = v->graph[slot];
    if (graph && std::memcmp(key, v->graph_key[slot], sizeof(key)) == 0) return;
    if (graph) {
        cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
    cudaStream_t s = v->ctx->stream;
    const uint64_t before = g_kernel_launches.load();
    BCMC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaGraph_t g = nullptr;
    try {
        vol_enqueue_query(v, s, 0.0f, 1, mode == 1, out);
    } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    BCMC_CUDA(cudaStreamEndCapture(s, &g));
    const cudaError_t e = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    BCMC_CUDA(e);
    // captured launches did not run: count them per replay instead
    v->graph_kernels = g_kernel_launches.load() - before;
    g_kernel_launches.fetch_sub(v->graph_kernels);
    std::memcpy(v->graph_key[slot], key, sizeof(key));
}

// One query: into the volume's vertex buffer (host_out null), or straight
// into a page-locked host buffer of host_cap vertices (host_out = its device
// address).
static bcmc_status lru_reset_impl(bcmc_lru* c);

static bcmc_status vol_query(bcmc_vol* v, float iso, bcmc_perf* perf, uint32_t* num_vertices, uint2* host_out,
                             uint64_t host_cap)
{
    bcmc_ctx* ctx = v->ctx;
    return guarded(ctx, [&]() -> bcmc_status {
        bcmc_lru* c = v->lru;
        cudaStream_t s = ctx->stream;
        const int mode = host_out ? 2 : (perf ? 1 : 0);
        const uint32_t out_cap = host_out ? (uint32_t)std::min<uint64_t>(host_cap, 0xffffffffull) : v->vert_capacity;
        for (int attempt = 0;; ++attempt) {
            vol_ensure_graph(v, mode, host_out);
            lru_epoch_tick(c, s);
            *v->h_in = QueryInputs{iso, c->capacity, out_cap, 0u, ctx->debug_drop_tile};
            BCMC_CUDA(cudaGraphLaunch(v->graph[graph_slot(v, mode)], s));
            count_launches(v->graph_kernels);
            BCMC_CUDA(cudaStreamSynchronize(s));
            if (c->h_q->error) {
                // the cache's slot arrays are not trusted after a wait gave up: reset them
                // over the logical size the query reached
                const uint32_t site = c->h_q->error;
                c->cache_size = std::min(std::max(c->cache_size, c->h_q->cache_size), c->capacity);
                lru_clear_key16(c, s);
                lru_reset_impl(c);
                return fail(ctx, BCMC_E_TIMEOUT, "device wait timed out (site " + std::to_string(site) + ")");
            }
            if (c->h_q->grow_needed) {
                if (attempt > 2) return fail(ctx, BCMC_E_STATE, "cache growth did not converge");
                lru_grow_capacity(c, c->h_q->grow_needed);
                continue;
            }
            break;
        }
        const uint3 nb = make_uint3(v->nb[0], v->nb[1], v->nb[2]);
        McArgs ma{v->active, v->active_ids, c->item_slots, reinterpret_cast<const float*>(c->cache), nb,
                  make_block_grid(nb), v->with_verts, v->vert_offsets, v->block_counts, v->verts, c->st_mc_v,
                  c->st_mc_b};
        QueryState& h = *c->h_q;
        v->last_on_host = host_out != nullptr;
        if (host_out && h.num_active > 0 && h.num_verts > 0 && h.vert_overflow) {
            // the host buffer is the caller's: report the size it needs
            if (num_vertices) *num_vertices = h.num_verts;
            c->cache_size = h.cache_size;
            return fail(ctx, BCMC_E_LIMIT, "the host buffer holds " + std::to_string(host_cap) + " vertices; the query has " +
                                               std::to_string(h.num_verts));
        }
        if (h.num_active > 0 && h.num_verts > 0 && h.vert_overflow) {
            vol_grow_verts(v, h.num_verts);
            lru_begin(c, s, iso, 1, v->vert_capacity);
            ma.verts = v->verts;
            mc_launch(ctx, c->q, ma, v->total, s);
            if (perf) BCMC_CUDA(cudaEventRecord(v->ev[4], s));
            lru_read_state(c, s);
            if (c->h_q->error) return fail(ctx, BCMC_E_TIMEOUT, "device wait timed out");
            // a query of 2^32 or more vertices lands here too: vertex counts
            // are 32-bit (as the reference's), so the CTA whose range crosses
            // 2^32 fails its fit check again after any growth
            if (c->h_q->vert_overflow)
                return fail(ctx, BCMC_E_STATE,
                            "vertex buffer growth failed (or the query has 2^32 or more vertices, past the 32-bit "
                            "vertex count)");
        } else if (h.num_verts > v->verts_storage) {
            v->verts_storage = h.num_verts;  // the reference's storage bookkeeping
        }
        c->cache_size = h.cache_size;
        if (perf) {
            float t[4];
            BCMC_CUDA(cudaEventElapsedTime(&t[0], v->ev[0], v->ev[1]));
            BCMC_CUDA(cudaEventElapsedTime(&t[1], v->ev[1], v->ev[2]));
            BCMC_CUDA(cudaEventElapsedTime(&t[2], v->ev[2], v->ev[3]));
            BCMC_CUDA(cudaEventElapsedTime(&t[3], v->ev[3], v->ev[4]));
            perf->computeActiveBlocks = t[0];
            perf->cacheUpdate = t[1];
            perf->decompression = t[2];
            perf->computeVertices = t[3];
            perf->total = t[0] + t[1] + t[2] + t[3];
        }
        // field updates at the reference's points (compressed_marching_cubes.js:630-808)
        uint32_t result = 0;
        if (h.num_active > 0) {
            v->stats.newDecompressed = h.num_new;
            v->stats.numActiveBlocks = h.num_active;
            v->stats.numBlocksWithVertices = h.num_with_verts;
            if (h.num_new > 0) {
                c->display_slots = h.display_slots_available;
                c->last_num_new = h.num_new;
                c->last_num_avail = h.num_avail;
            }
            if (h.num_verts > 0) {
                v->stats.numVertices = h.num_verts;
                result = h.num_verts;
            }
        }
        v->stats.cacheSize = c->cache_size;
        v->stats.displayNumSlotsAvailable = c->display_slots;
        v->stats.lastNumVertices = result;
        if (num_vertices) *num_vertices = result;
        return BCMC_OK;
    });
}

bcmc_status bcmc_compute_surface(bcmc_vol* v, float iso, bcmc_perf* perf, uint32_t* num_vertices)
{
    if (!v) return BCMC_E_ARG;
    return vol_query(v, iso, perf, num_vertices, nullptr, 0);
}

bcmc_status bcmc_compute_surface_host(bcmc_vol* v, float iso, void* host_vertices, uint64_t capacity,
                                      uint32_t* num_vertices)
{
    if (!v || !host_vertices || capacity == 0 || reinterpret_cast<uintptr_t>(host_vertices) % 8 != 0)
        return BCMC_E_ARG;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host_vertices) != cudaSuccess || at.type != cudaMemoryTypeHost ||
        !at.devicePointer) {
        cudaGetLastError();
        return fail(v->ctx, BCMC_E_ARG, "the host buffer must be page-locked (cudaMallocHost or cudaHostRegister)");
    }
    return vol_query(v, iso, nullptr, num_vertices, static_cast<uint2*>(at.devicePointer), capacity);
}

// Makes ring buffer r the volume's vertex buffer.
static void vol_select_verts(bcmc_vol* v, int r)
{
    if (r == v->cur) return;
    v->ring[v->cur] = v->verts;
    v->ring_cap[v->cur] = v->vert_capacity;
    v->verts = v->ring[r];
    v->vert_capacity = v->ring_cap[r];
    v->cur = r;
}

bcmc_status bcmc_compute_surfaces_host(bcmc_vol* v, const float* isovalues, uint32_t n, void* host_vertices,
                                       uint64_t capacity, uint32_t* num_vertices)
{
    if (!v || (n && (!isovalues || !host_vertices || !num_vertices || capacity == 0)) ||
        reinterpret_cast<uintptr_t>(host_vertices) % 8 != 0)
        return BCMC_E_ARG;
    if (n == 0) return BCMC_OK;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host_vertices) != cudaSuccess || at.type != cudaMemoryTypeHost) {
        cudaGetLastError();
        return fail(v->ctx, BCMC_E_ARG, "the host buffer must be page-locked (cudaMallocHost or cudaHostRegister)");
    }
    for (uint32_t i = 0; i < n; ++i) num_vertices[i] = 0;
    bcmc_ctx* ctx = v->ctx;
    uint2* const host = static_cast<uint2*>(host_vertices);
    bool pending[kVertRing] = {};
    const bcmc_status st = guarded(ctx, [&]() -> bcmc_status {
        if (!v->copy) {
            BCMC_CUDA(cudaStreamCreateWithFlags(&v->copy, cudaStreamNonBlocking));
            for (auto& e : v->copy_ev) BCMC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        uint64_t used = 0;
        for (uint32_t i = 0; i < n; ++i) {
            const int b = (int)(i % kVertRing);  // ring buffer 0 is the volume's vertex buffer
            vol_select_verts(v, b);
            uint32_t largest = 0;
            for (int r = 0; r < kVertRing; ++r)
                if (r != b) largest = std::max(largest, v->ring_cap[r]);
            if (v->vert_capacity < largest) {
                // every buffer at the largest size; the transfer from this one ends first
                if (pending[b]) BCMC_CUDA(cudaEventSynchronize(v->copy_ev[b]));
                pending[b] = false;
                dev_free(ctx, v->verts, (size_t)v->vert_capacity * 8);
                v->verts = nullptr;
                v->vert_capacity = 0;
                v->verts = (uint2*)dev_alloc(ctx, (size_t)largest * 8);
                v->vert_capacity = largest;
            }
            // the query writes this buffer only after its previous transfer
            if (pending[b]) BCMC_CUDA(cudaStreamWaitEvent(ctx->stream, v->copy_ev[b], 0));
            uint32_t nv = 0;
            const bcmc_status q = vol_query(v, isovalues[i], nullptr, &nv, nullptr, 0);
            if (q != BCMC_OK) return q;
            num_vertices[i] = nv;
            if (nv > capacity - used)
                return fail(ctx, BCMC_E_LIMIT, "the host buffer holds " + std::to_string(capacity) +
                                                    " vertices; query " + std::to_string(i) + " needs " +
                                                    std::to_string(used + nv));
            if (nv) {
                // the query has completed on the library's stream (vol_query waits for it)
                BCMC_CUDA(cudaMemcpyAsync(host + used, v->verts, (size_t)nv * 8, cudaMemcpyDeviceToHost, v->copy));
                BCMC_CUDA(cudaEventRecord(v->copy_ev[b], v->copy));
                pending[b] = true;
            }
            used += nv;
        }
        return BCMC_OK;
    });
    // every transfer has ended when the call returns, also on failure
    if (v->copy && cudaStreamSynchronize(v->copy) != cudaSuccess && st == BCMC_OK)
        return fail(ctx, BCMC_E_CUDA, "vertex transfer failed");
    return st;
}

bcmc_status bcmc_vertices(bcmc_vol* v, const void** d_vertices, uint64_t* bytes)
{
    if (!v || !d_vertices || !bytes) return BCMC_E_ARG;
    if (v->last_on_host) return fail(v->ctx, BCMC_E_STATE, "the last query wrote its vertices to host memory");
    *d_vertices = v->verts;
    *bytes = (uint64_t)v->stats.lastNumVertices * 8u;
    return BCMC_OK;
}

bcmc_status bcmc_copy_vertices(bcmc_vol* v, void* host, uint64_t bytes)
{
    if (!v || (!host && bytes)) return BCMC_E_ARG;
    if (bytes > (uint64_t)v->stats.lastNumVertices * 8u) return fail(v->ctx, BCMC_E_ARG, "more bytes than vertices");
    if (v->last_on_host && bytes) return fail(v->ctx, BCMC_E_STATE, "the last query wrote its vertices to host memory");
    if (bytes == 0) return BCMC_OK;
    return guarded(v->ctx, [&]() -> bcmc_status {
        BCMC_CUDA(cudaMemcpyAsync(host, v->verts, bytes, cudaMemcpyDeviceToHost, v->ctx->stream));
        BCMC_CUDA(cudaStreamSynchronize(v->ctx->stream));
        return BCMC_OK;
    });
}

bcmc_status bcmc_stats_get(bcmc_vol* v, bcmc_stats* out)
{
    if (!v || !out) return BCMC_E_ARG;
    *out = v->stats;
    return BCMC_OK;
}

bcmc_status bcmc_memory_report(bcmc_vol* v, bcmc_memory* m)
{
    if (!v || !m) return BCMC_E_ARG;
    const bcmc_lru* c = v->lru;
    std::memset(m, 0, sizeof(*m));
    m->compressedData = v->nwords * 8;
    m->vertexBuffer = (uint64_t)v->vert_capacity * 8;
    m->blockActive = (uint64_t)v->total * 4;
    m->blockRanges = (uint64_t)v->total * 8;
    m->activeBlockIDs = (uint64_t)v->total * 4;
    m->blocksWithVertices = (uint64_t)v->total * 4;
    m->blockVertexOffsets = (uint64_t)v->total * 4;
    m->cache = (uint64_t)c->capacity * c->element_size;
    m->cachedItemSlots = (uint64_t)c->aligned_total * 4;
    m->slotData = (uint64_t)c->capacity * 12;
    m->scratch = (uint64_t)c->capacity * 4 * 6 + c->status_words * 8 + (uint64_t)c->total * 4 + sizeof(QueryState) +
                 (uint64_t)v->stage_blocks * 256u;
    m->deviceTotal = m->compressedData + m->vertexBuffer + m->blockActive + m->blockRanges + m->activeBlockIDs +
                     m->blocksWithVertices + m->blockVertexOffsets + m->cache + m->cachedItemSlots + m->slotData +
                     m->scratch;
    return BCMC_OK;
}

static bcmc_status lru_reset_impl(bcmc_lru* c)
{
    bcmc_ctx* ctx = c->ctx;
    return guarded(ctx, [&]() -> bcmc_status {
        cudaStream_t s = ctx->stream;
        k_lru_init_slots<<<fill_grid(ctx, c->cache_size), 256, 0, s>>>(c->slot_age, c->slot_avail, c->slot_item, 0,
                                                                       c->cache_size, 0);
        count_launches(1);
        k_fill_i32<<<fill_grid(ctx, c->total), 256, 0, s>>>(c->item_slots, c->total, -1);
        count_launches(1);
        BCMC_CUDA(cudaGetLastError());
        BCMC_CUDA(cudaStreamSynchronize(s));
        return BCMC_OK;
    });
}

bcmc_status bcmc_cache_reset(bcmc_vol* v)
{
    if (!v) return BCMC_E_ARG;
    return lru_reset_impl(v->lru);
}

bcmc_status bcmc_volume_views(bcmc_vol* v, bcmc_vol_views* out)
{
    if (!v || !out) return BCMC_E_ARG;
    out->d_block_ranges = v->ranges;
    out->d_block_active = v->active;
    out->d_active_block_ids = v->active_ids;
    out->d_blocks_with_vertices = v->with_verts;
    out->d_block_vertex_offsets = v->vert_offsets;
    out->d_new_item_ids = v->lru->new_ids;
    out->lru = v->lru;
    return BCMC_OK;
}

// ---- LRUCache --------------------------------------------------------------
bcmc_status bcmc_lru_create(bcmc_ctx* ctx, uint32_t initial_size, uint32_t element_size, uint32_t total,
                            bcmc_lru** out)
{
    if (!ctx || !out) return BCMC_E_ARG;
    if (total == 0 || element_size == 0 || element_size % 4 != 0)
        return fail(ctx, BCMC_E_ARG, "totalElements > 0 and elementSize a multiple of 4 required");
    return guarded(ctx, [&]() -> bcmc_status {
        *out = lru_new(ctx, initial_size, element_size, total);
        return BCMC_OK;
    });
}

void bcmc_lru_destroy(bcmc_lru* c) { lru_delete(c); }

bcmc_status bcmc_lru_update(bcmc_lru* c, const uint32_t* d_item_needed, uint32_t* num_new,
                            const uint32_t** d_new_item_ids)
{
    if (!c || !d_item_needed) return BCMC_E_ARG;
    bcmc_ctx* ctx = c->ctx;
    return guarded(ctx, [&]() -> bcmc_status {
        cudaStream_t s = ctx->stream;
        for (int attempt = 0;; ++attempt) {
            lru_begin(c, s, 0.0f, 0, 0);
            ActiveArgs aa{nullptr, make_uint3(0, 0, 0), make_block_grid(make_uint3(1, 1, 1)), d_item_needed, nullptr,
                          c->item_slots, c->total, nullptr, c->new_ids, c->st_active_a, c->st_active_n};
            active_launch(ctx, c->q, aa, s);
            lru_enqueue_update(c, s, d_item_needed, nullptr, 0);
            lru_read_state(c, s);
            if (c->h_q->error) {
                lru_clear_key16(c, s);
                return fail(ctx, BCMC_E_TIMEOUT, "device wait timed out");
            }
            if (c->h_q->grow_needed) {
                if (attempt > 2) return fail(ctx, BCMC_E_STATE, "cache growth did not converge");
                lru_grow_capacity(c, c->h_q->grow_needed);
                continue;
            }
            break;
        }
        c->cache_size = c->h_q->cache_size;
        if (c->h_q->num_new > 0) {
            c->display_slots = c->h_q->display_slots_available;
            c->last_num_new = c->h_q->num_new;
            c->last_num_avail = c->h_q->num_avail;
        }
        if (num_new) *num_new = c->h_q->num_new;
        if (d_new_item_ids) *d_new_item_ids = c->new_ids;
        return BCMC_OK;
    });
}

bcmc_status bcmc_lru_reset(bcmc_lru* c)
{
    if (!c) return BCMC_E_ARG;
    return lru_reset_impl(c);
}

bcmc_status bcmc_lru_view_get(bcmc_lru* c, bcmc_lru_view* o)
{
    if (!c || !o) return BCMC_E_ARG;
    o->cacheSize = c->cache_size;
    o->totalElements = c->total;
    o->elementSize = c->element_size;
    o->displayNumSlotsAvailable = c->display_slots;
    o->d_cached_item_slots = c->item_slots;
    o->d_slot_age = c->slot_age;
    o->d_slot_available = c->slot_avail;
    o->d_slot_item = c->slot_item;
    o->d_cache = c->cache;
    o->d_last_sorted_slots = c->h_q->sort_final == 2 ? c->sort_cv : c->sort_bv;
    o->lastNumSlotsAvailable = c->last_num_avail;
    return BCMC_OK;
}

// ---- scan / compact / sort -------------------------------------------------
uint32_t bcmc_scan_aligned_size(uint32_t n) { return align_up(n, 512u); }

bcmc_status bcmc_scan_exclusive_u32_async(bcmc_ctx* ctx, const uint32_t* d_in, uint32_t* d_out, uint32_t n,
                                          uint32_t* d_total, void* stream)
{
    if (!ctx || (n && (!d_in || !d_out))) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        cudaStream_t s = pick(ctx, stream);
        if (n == 0) {
            if (d_total) BCMC_CUDA(cudaMemsetAsync(d_total, 0, 4, s));
            return BCMC_OK;
        }
        ensure_status(ctx, div_up(n, kScanTile) + 1);
        prim_begin(ctx->d_prim, s);
        scan_launch(ctx, ctx->d_prim, d_in, d_out, n, d_total, ctx->d_status, s);
        return BCMC_OK;
    });
}

bcmc_status bcmc_scan_exclusive_u32(bcmc_ctx* ctx, uint32_t* d_data, uint32_t n, uint32_t aligned_size,
                                    uint32_t* total)
{
    if (!ctx || (n && !d_data) || aligned_size < n) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        cudaStream_t s = ctx->stream;
        uint32_t* d_tot = &ctx->d_prim->pad[0];
        if (n == 0) {
            BCMC_CUDA(cudaMemsetAsync(d_tot, 0, 4, s));
        } else {
            ensure_status(ctx, div_up(n, kScanTile) + 1);
            prim_begin(ctx->d_prim, s);
            scan_launch(ctx, ctx->d_prim, d_data, d_data, n, d_tot, ctx->d_status, s);
        }
        if (n < aligned_size) BCMC_CUDA(cudaMemcpyAsync(d_data + n, d_tot, 4, cudaMemcpyDeviceToDevice, s));
        BCMC_CUDA(cudaMemcpyAsync(ctx->h_pinned, d_tot, 4, cudaMemcpyDeviceToHost, s));
        BCMC_CUDA(cudaMemcpyAsync(ctx->h_pinned + 1, &ctx->d_prim->error, 4, cudaMemcpyDeviceToHost, s));
        BCMC_CUDA(cudaStreamSynchronize(s));
        if (n && ctx->h_pinned[1]) return fail(ctx, BCMC_E_TIMEOUT, "device wait timed out");
        if (total) *total = ctx->h_pinned[0];
        return BCMC_OK;
    });
}

bcmc_status bcmc_compact_ids(bcmc_ctx* ctx, uint32_t n, const uint32_t* d_flags, const uint32_t* d_offsets,
                             uint32_t* d_out, void* stream)
{
    if (!ctx || (n && (!d_flags || !d_offsets || !d_out))) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        compact_launch(ctx, n, d_flags, d_offsets, d_out, pick(ctx, stream));
        return BCMC_OK;
    });
}

bcmc_status bcmc_select_ids(bcmc_ctx* ctx, uint32_t n, const uint32_t* d_flags, uint32_t* d_out, uint32_t* d_count,
                            void* stream)
{
    if (!ctx || (n && (!d_flags || !d_out))) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        cudaStream_t s = pick(ctx, stream);
        if (n == 0) {
            if (d_count) BCMC_CUDA(cudaMemsetAsync(d_count, 0, 4, s));
            return BCMC_OK;
        }
        ensure_status(ctx, div_up(n, kScanTile) + 1);
        prim_begin(ctx->d_prim, s);
        select_launch(ctx, ctx->d_prim, d_flags, d_out, n, d_count, ctx->d_status, s);
        return BCMC_OK;
    });
}

uint32_t bcmc_sort_aligned_size(uint32_t n)
{
    // nextPow2(ceil(n/64)) * 64, with nextPow2(0) = 0 as in the reference
    const uint32_t c = div_up(n, 64u);
    if (c == 0) return 0;
    uint32_t p = 1;
    while (p < c) p <<= 1;
    return p * 64u;
}

bcmc_status bcmc_sort_pairs_u32(bcmc_ctx* ctx, uint32_t* d_keys, uint32_t* d_values, uint32_t n, int reverse,
                                void* stream)
{
    if (!ctx || (n && (!d_keys || !d_values))) return BCMC_E_ARG;
    if (n == 0) return BCMC_OK;
    return guarded(ctx, [&]() -> bcmc_status {
        cudaStream_t s = pick(ctx, stream);
        ensure_status(ctx, sort_status_words(n));
        ensure_scratch(ctx, (size_t)n * 4);
        SortBuffers b;
        b.in_keys = d_keys;
        b.in_vals = d_values;
        b.b_keys = ctx->d_scratch;
        b.b_vals = ctx->d_scratch + n;
        b.c_keys = ctx->d_scratch + 2 * (size_t)n;
        b.c_vals = ctx->d_scratch + 3 * (size_t)n;
        b.status = ctx->d_status;
        prim_begin(ctx->d_prim, s);
        sort_launch(ctx, ctx->d_prim, nullptr, n, b, reverse ? 1 : 0, s);
        sort_writeback(ctx, ctx->d_prim, nullptr, n, b, d_keys, d_values, reverse ? 1 : 0, s);
        return BCMC_OK;
    });
}

// ---- ZFP -------------------------------------------------------------------
uint64_t bcmc_zfp_stream_words(const uint32_t dims[3], uint32_t rate)
{
    if (!dims) return 0;
    const uint64_t nb = (uint64_t)div_up(dims[0], 4) * div_up(dims[1], 4) * div_up(dims[2], 4);
    return (nb * 64u * rate + 63u) / 64u + 1u;
}

bcmc_status bcmc_zfp_block_ranges(bcmc_ctx* ctx, const uint64_t* d_words, const uint32_t dims[3], uint32_t rate,
                                  float* d_ranges, void* stream)
{
    if (!ctx || !d_words || !dims || !d_ranges || rate == 0 || rate > 32) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        zfp_ranges_launch(ctx, d_words, dims, 64u * rate, d_ranges, pick(ctx, stream));
        return BCMC_OK;
    });
}

bcmc_status bcmc_zfp_decode_blocks(bcmc_ctx* ctx, const uint64_t* d_words, uint32_t rate, const uint32_t* d_block_ids,
                                   uint32_t n, const int32_t* d_item_slots, float* d_cache, void* stream)
{
    if (!ctx || rate == 0 || rate > 32 || (n && (!d_words || !d_block_ids || !d_item_slots || !d_cache)))
        return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        zfp_decode_blocks_launch(ctx, d_words, 64u * rate, d_block_ids, n, d_item_slots, d_cache, pick(ctx, stream));
        return BCMC_OK;
    });
}

bcmc_status bcmc_unpack_vertices(bcmc_ctx* ctx, const void* d_vertices, uint64_t n, const uint32_t dims[3],
                                 const float scale[3], float* d_world, const float* proj_view, float* d_clip,
                                 void* stream)
{
    if (!ctx || !dims || !dims[0] || !dims[1] || !dims[2] || (n && (!d_vertices || !d_world)) ||
        (proj_view && !d_clip))
        return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        unpack_launch(ctx, static_cast<const uint2*>(d_vertices), n, dims, scale, proj_view, d_world, d_clip,
                      pick(ctx, stream));
        return BCMC_OK;
    });
}

bcmc_status bcmc_render(bcmc_ctx* ctx, const void* d_vertices, uint64_t n, const uint32_t dims[3],
                        const float scale[3], const bcmc_render_params* params, float* d_rgba, float* d_depth,
                        uint32_t* d_triangle, void* stream)
{
    if (!ctx || !dims || !dims[0] || !dims[1] || !dims[2] || !params || !d_rgba || (n && !d_vertices))
        return BCMC_E_ARG;
    if (params->width == 0 || params->height == 0 || params->width > 16384 || params->height > 16384)
        return fail(ctx, BCMC_E_ARG, "render: width and height must be in [1, 16384]");
    if (n / 3 > 0xffffffffull) return fail(ctx, BCMC_E_LIMIT, "render: more than 2^32-1 triangles");
    if (reinterpret_cast<uintptr_t>(d_rgba) % 16 != 0 || (n && reinterpret_cast<uintptr_t>(d_vertices) % 8 != 0))
        return fail(ctx, BCMC_E_ARG, "render: d_rgba must be 16-byte and d_vertices 8-byte aligned");
    return guarded(ctx, [&]() -> bcmc_status {
        render_launch(ctx, static_cast<const uint2*>(d_vertices), n, dims, scale, *params, d_rgba, d_depth, d_triangle,
                      pick(ctx, stream));
        return BCMC_OK;
    });
}

bcmc_status bcmc_zfp_decode_volume(bcmc_ctx* ctx, const uint64_t* d_words, uint64_t nblocks, uint32_t rate,
                                   float* d_out, void* stream)
{
    if (!ctx || rate == 0 || rate > 32 || (nblocks && (!d_words || !d_out))) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        zfp_decode_volume_launch(ctx, d_words, nblocks, 64u * rate, d_out, pick(ctx, stream));
        return BCMC_OK;
    });
}

bcmc_status bcmc_zfp_encode(bcmc_ctx* ctx, const float* d_field, const uint32_t dims[3], uint32_t rate,
                            uint64_t* d_words, void* stream)
{
    if (!ctx || !d_field || !dims || !d_words || rate == 0 || rate > 32) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        cudaStream_t s = pick(ctx, stream);
        BCMC_CUDA(cudaMemsetAsync(d_words, 0, bcmc_zfp_stream_words(dims, rate) * 8, s));
        zfp_encode_launch(ctx, d_field, dims, 64u * rate, d_words, s);
        return BCMC_OK;
    });
}

bcmc_status bcmc_block_active(bcmc_ctx* ctx, const float* d_ranges, const uint32_t dims[3], float iso,
                              uint32_t* d_active, void* stream)
{
    if (!ctx || !d_ranges || !dims || !d_active) return BCMC_E_ARG;
    return guarded(ctx, [&]() -> bcmc_status {
        cudaStream_t s = pick(ctx, stream);
        const uint3 nb = make_uint3(div_up(dims[0], 4), div_up(dims[1], 4), div_up(dims[2], 4));
        const uint64_t total = (uint64_t)nb.x * nb.y * nb.z;
        ensure_status(ctx, 2 * (active_tiles((uint32_t)total) + 1));
        query_begin_launch(ctx->d_prim, iso, 0, 0, 0, s);
        ActiveArgs aa{reinterpret_cast<const float2*>(d_ranges), nb, make_block_grid(nb), nullptr, d_active, nullptr,
                      (uint32_t)total, nullptr, nullptr, ctx->d_status, ctx->d_status + active_tiles((uint32_t)total) + 1};
        active_launch(ctx, ctx->d_prim, aa, s);
        return BCMC_OK;
    });
}

}  // extern "C"
