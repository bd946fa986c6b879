// bcmc_node.cc -- N-API addon: the reference's CompressedMarchingCubes object
// (js/compressed_marching_cubes.js) over the C ABI of libbcmc_gb300.so.
//
// Exposes class CompressedMarchingCubes with the reference's method names:
//   new CompressedMarchingCubes(device)            js/compressed_marching_cubes.js:1
//   setCompressedVolume(bytes, rate, dims, scale)  :432 -> Promise<void>
//   computeSurface(isovalue, perfTracker)          :580 -> Promise<numVertices>
//   reportMemoryUse()                              :366 -> [sizes, names, total]
//   lruCacheReset()                                js/lru_cache.js:846 (the JS
//                                                  wrapper maps lruCache.reset())
//   copyVertices() -> Uint32Array [numVertices*2]  the vertex buffer's contents
//   vertexBufferAddress() -> BigInt                its device address (:781-784)
//   stats() -> {totalBlocks, numActiveBlocks, ...} the fields js/bcmc.js:77-100 reads
// `device` is the CUDA device ordinal (the reference passes its GPUDevice).
// GPU work runs on a napi_async_work worker and settles the Promise the
// reference's async methods return.  As in the reference, each call on one
// object is awaited before the next is made; a call made while another is in
// flight on the same object is rejected.
//
// Build (where Node.js headers exist): node-gyp rebuild, with
// BCMC_LIB_DIR pointing at webgpu-bcmc_gb300/_build (see binding.gyp).
#include <node_api.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "bcmc.h"

namespace {

struct Surface {
    bcmc_ctx* ctx = nullptr;
    bcmc_vol* vol = nullptr;
    bool busy = false;
    napi_ref self = nullptr;
};

#define NAPI_CHECK(env, call)                                                 \
    do {                                                                      \
        if ((call) != napi_ok) {                                              \
            napi_throw_error((env), nullptr, "N-API call failed: " #call);    \
            return nullptr;                                                   \
        }                                                                     \
    } while (0)

std::string status_message(bcmc_ctx* ctx, bcmc_status st, const char* what)
{
    std::string m = std::string(what) + " failed (status " + std::to_string((int)st) + ")";
    if (ctx) m += ": " + std::string(bcmc_last_error(ctx));
    return m;
}

napi_value reject_now(napi_env env, const std::string& msg)
{
    napi_deferred d;
    napi_value promise, err, text;
    napi_create_promise(env, &d, &promise);
    napi_create_string_utf8(env, msg.c_str(), NAPI_AUTO_LENGTH, &text);
    napi_create_error(env, nullptr, text, &err);
    napi_reject_deferred(env, d, err);
    return promise;
}

Surface* unwrap(napi_env env, napi_callback_info info, size_t* argc, napi_value* argv)
{
    napi_value self;
    if (napi_get_cb_info(env, info, argc, argv, &self, nullptr) != napi_ok) return nullptr;
    Surface* s = nullptr;
    if (napi_unwrap(env, self, reinterpret_cast<void**>(&s)) != napi_ok) return nullptr;
    return s;
}

// ---- async jobs -------------------------------------------------------------
struct Job {
    Surface* s = nullptr;
    napi_deferred deferred = nullptr;
    napi_async_work work = nullptr;
    bcmc_status st = BCMC_OK;
    std::string what;
    // setCompressedVolume
    std::vector<uint8_t> bytes;
    uint32_t rate = 0, dims[3] = {0, 0, 0};
    float scale[3] = {1.f, 1.f, 1.f};
    bcmc_vol* new_vol = nullptr;
    // computeSurface
    float iso = 0.f;
    bool want_perf = false;
    bcmc_perf perf{};
    uint32_t n = 0;
    bcmc_stats stats{};
    napi_ref perf_ref = nullptr;
};

void finish(napi_env env, Job* j, napi_value ok_value)
{
    j->s->busy = false;
    if (j->st == BCMC_OK) {
        napi_resolve_deferred(env, j->deferred, ok_value);
    } else {
        napi_value err, text;
        napi_create_string_utf8(env, status_message(j->s->ctx, j->st, j->what.c_str()).c_str(), NAPI_AUTO_LENGTH,
                                &text);
        napi_create_error(env, nullptr, text, &err);
        napi_reject_deferred(env, j->deferred, err);
    }
    if (j->perf_ref) napi_delete_reference(env, j->perf_ref);
    napi_delete_async_work(env, j->work);
    delete j;
}

void volume_exec(napi_env, void* p)
{
    auto* j = static_cast<Job*>(p);
    j->st = bcmc_volume_create(j->s->ctx, j->bytes.data(), j->bytes.size(), j->rate, j->dims, j->scale, &j->new_vol);
}

void volume_done(napi_env env, napi_status, void* p)
{
    auto* j = static_cast<Job*>(p);
    if (j->st == BCMC_OK) {
        if (j->s->vol) bcmc_volume_destroy(j->s->vol);
        j->s->vol = j->new_vol;
    }
    napi_value undef;
    napi_get_undefined(env, &undef);
    finish(env, j, undef);
}

void surface_exec(napi_env, void* p)
{
    auto* j = static_cast<Job*>(p);
    j->st = bcmc_compute_surface(j->s->vol, j->iso, j->want_perf ? &j->perf : nullptr, &j->n);
    if (j->st == BCMC_OK) j->st = bcmc_stats_get(j->s->vol, &j->stats);
}

// perfTracker[key].push(value), creating the array on first use
// (js/compressed_marching_cubes.js:593-610 initialises the same keys)
void push_perf(napi_env env, napi_value tracker, const char* key, double value)
{
    bool has = false;
    napi_value arr, v, push, ret;
    napi_has_named_property(env, tracker, key, &has);
    if (!has) {
        napi_create_array(env, &arr);
        napi_set_named_property(env, tracker, key, arr);
    } else {
        napi_get_named_property(env, tracker, key, &arr);
    }
    napi_create_double(env, value, &v);
    napi_get_named_property(env, arr, "push", &push);
    napi_call_function(env, arr, push, 1, &v, &ret);
}

void surface_done(napi_env env, napi_status, void* p)
{
    auto* j = static_cast<Job*>(p);
    napi_value n;
    napi_create_uint32(env, j->n, &n);
    if (j->st == BCMC_OK && j->perf_ref) {
        napi_value t;
        napi_get_reference_value(env, j->perf_ref, &t);
        napi_value tb;
        napi_create_uint32(env, j->stats.totalBlocks, &tb);
        napi_set_named_property(env, t, "totalBlocks", tb);
        push_perf(env, t, "computeActiveBlocks", j->perf.computeActiveBlocks);
        push_perf(env, t, "numActiveBlocks", j->stats.numActiveBlocks);
        push_perf(env, t, "cacheUpdate", j->perf.cacheUpdate);
        push_perf(env, t, "numBlocksDecompressed", j->stats.newDecompressed);
        push_perf(env, t, "decompression", j->perf.decompression);
        push_perf(env, t, "compactActiveIDs", 0.0);         // fused into computeActiveBlocks
        push_perf(env, t, "computeBlockHasVertices", 0.0);  // fused into computeVertices
        push_perf(env, t, "numBlocksWithVertices", j->stats.numBlocksWithVertices);
        push_perf(env, t, "compactBlocksWithVertices", 0.0);
        push_perf(env, t, "numVertices", j->n);
        push_perf(env, t, "computeVertices", j->perf.computeVertices);
    }
    finish(env, j, n);
}

bool get_u32_triple(napi_env env, napi_value arr, uint32_t out[3])
{
    for (uint32_t i = 0; i < 3; ++i) {
        napi_value e;
        if (napi_get_element(env, arr, i, &e) != napi_ok || napi_get_value_uint32(env, e, &out[i]) != napi_ok)
            return false;
    }
    return true;
}

bool get_f32_triple(napi_env env, napi_value arr, float out[3])
{
    for (uint32_t i = 0; i < 3; ++i) {
        napi_value e;
        double d;
        if (napi_get_element(env, arr, i, &e) != napi_ok || napi_get_value_double(env, e, &d) != napi_ok)
            return false;
        out[i] = (float)d;
    }
    return true;
}

napi_value queue(napi_env env, Job* j, napi_async_execute_callback exec, napi_async_complete_callback done)
{
    napi_value promise, name;
    napi_create_promise(env, &j->deferred, &promise);
    napi_create_string_utf8(env, j->what.c_str(), NAPI_AUTO_LENGTH, &name);
    napi_create_async_work(env, nullptr, name, exec, done, j, &j->work);
    j->s->busy = true;
    napi_queue_async_work(env, j->work);
    return promise;
}

// ---- methods ------------------------------------------------------------------
napi_value SetCompressedVolume(napi_env env, napi_callback_info info)
{
    size_t argc = 4;
    napi_value argv[4];
    Surface* s = unwrap(env, info, &argc, argv);
    if (!s) return reject_now(env, "setCompressedVolume: not a CompressedMarchingCubes");
    if (s->busy) return reject_now(env, "setCompressedVolume: a call is in flight on this object");
    auto* j = new Job;
    j->s = s;
    j->what = "setCompressedVolume";
    bool is_ta = false;
    napi_is_typedarray(env, argv[0], &is_ta);
    napi_typedarray_type type;
    size_t length = 0, offset = 0;
    void* data = nullptr;
    napi_value ab;
    if (argc < 3 || !is_ta ||
        napi_get_typedarray_info(env, argv[0], &type, &length, &data, &ab, &offset) != napi_ok ||
        type != napi_uint8_array || napi_get_value_uint32(env, argv[1], &j->rate) != napi_ok ||
        !get_u32_triple(env, argv[2], j->dims) || (argc > 3 && !get_f32_triple(env, argv[3], j->scale))) {
        delete j;
        return reject_now(env, "setCompressedVolume(Uint8Array, rate, [x, y, z], [sx, sy, sz]): bad arguments");
    }
    j->bytes.assign(static_cast<uint8_t*>(data), static_cast<uint8_t*>(data) + length);  // the worker owns a copy
    return queue(env, j, volume_exec, volume_done);
}

napi_value ComputeSurface(napi_env env, napi_callback_info info)
{
    size_t argc = 2;
    napi_value argv[2];
    Surface* s = unwrap(env, info, &argc, argv);
    if (!s || !s->vol) return reject_now(env, "computeSurface: no volume set");
    if (s->busy) return reject_now(env, "computeSurface: a call is in flight on this object");
    auto* j = new Job;
    j->s = s;
    j->what = "computeSurface";
    double iso = 0.0;
    if (argc < 1 || napi_get_value_double(env, argv[0], &iso) != napi_ok) {
        delete j;
        return reject_now(env, "computeSurface(isovalue, perfTracker): bad isovalue");
    }
    j->iso = (float)iso;
    napi_valuetype t = napi_undefined;
    if (argc > 1) napi_typeof(env, argv[1], &t);
    if (t == napi_object) {
        j->want_perf = true;
        napi_create_reference(env, argv[1], 1, &j->perf_ref);
    }
    return queue(env, j, surface_exec, surface_done);
}

napi_value CopyVertices(napi_env env, napi_callback_info info)
{
    size_t argc = 0;
    Surface* s = unwrap(env, info, &argc, nullptr);
    bcmc_stats st{};
    if (!s || !s->vol || s->busy || bcmc_stats_get(s->vol, &st) != BCMC_OK) {
        napi_throw_error(env, nullptr, "copyVertices: no finished query on this object");
        return nullptr;
    }
    void* data = nullptr;
    napi_value ab, out;
    const size_t bytes = (size_t)st.lastNumVertices * 8u;
    NAPI_CHECK(env, napi_create_arraybuffer(env, bytes, &data, &ab));
    if (bytes && bcmc_copy_vertices(s->vol, data, bytes) != BCMC_OK) {
        napi_throw_error(env, nullptr, status_message(s->ctx, BCMC_E_CUDA, "copyVertices").c_str());
        return nullptr;
    }
    NAPI_CHECK(env, napi_create_typedarray(env, napi_uint32_array, bytes / 4u, ab, 0, &out));
    return out;
}

napi_value VertexBufferAddress(napi_env env, napi_callback_info info)
{
    size_t argc = 0;
    Surface* s = unwrap(env, info, &argc, nullptr);
    const void* d = nullptr;
    uint64_t bytes = 0;
    if (!s || !s->vol || bcmc_vertices(s->vol, &d, &bytes) != BCMC_OK) {
        napi_throw_error(env, nullptr, "vertexBufferAddress: no vertex buffer");
        return nullptr;
    }
    napi_value v;
    NAPI_CHECK(env, napi_create_bigint_uint64(env, (uint64_t)(uintptr_t)d, &v));
    return v;
}

napi_value Stats(napi_env env, napi_callback_info info)
{
    size_t argc = 0;
    Surface* s = unwrap(env, info, &argc, nullptr);
    bcmc_stats st{};
    if (!s || !s->vol || bcmc_stats_get(s->vol, &st) != BCMC_OK) {
        napi_throw_error(env, nullptr, "stats: no volume set");
        return nullptr;
    }
    napi_value o;
    NAPI_CHECK(env, napi_create_object(env, &o));
    const struct {
        const char* k;
        uint32_t v;
    } f[] = {{"totalBlocks", st.totalBlocks},
             {"numActiveBlocks", st.numActiveBlocks},
             {"newDecompressed", st.newDecompressed},
             {"numBlocksWithVertices", st.numBlocksWithVertices},
             {"numVertices", st.numVertices},
             {"cacheSize", st.cacheSize},
             {"displayNumSlotsAvailable", st.displayNumSlotsAvailable}};
    for (const auto& e : f) {
        napi_value v;
        napi_create_uint32(env, e.v, &v);
        napi_set_named_property(env, o, e.k, v);
    }
    return o;
}

napi_value ReportMemoryUse(napi_env env, napi_callback_info info)
{
    size_t argc = 0;
    Surface* s = unwrap(env, info, &argc, nullptr);
    bcmc_memory m{};
    if (!s || !s->vol || bcmc_memory_report(s->vol, &m) != BCMC_OK) {
        napi_throw_error(env, nullptr, "reportMemoryUse: no volume set");
        return nullptr;
    }
    // [per-buffer sizes, their names, the total], as the reference returns
    const struct {
        const char* k;
        uint64_t v;
    } f[] = {{"compressedData", m.compressedData},   {"vertexBuffer", m.vertexBuffer},
             {"blockActive", m.blockActive},         {"blockRanges", m.blockRanges},
             {"activeBlockIDs", m.activeBlockIDs},   {"blocksWithVertices", m.blocksWithVertices},
             {"blockVertexOffsets", m.blockVertexOffsets}, {"cache", m.cache},
             {"cachedItemSlots", m.cachedItemSlots}, {"slotData", m.slotData},
             {"scratch", m.scratch}};
    napi_value sizes, names, ret, total;
    NAPI_CHECK(env, napi_create_object(env, &sizes));
    NAPI_CHECK(env, napi_create_array(env, &names));
    uint32_t i = 0;
    for (const auto& e : f) {
        napi_value v, k;
        napi_create_double(env, (double)e.v, &v);
        napi_set_named_property(env, sizes, e.k, v);
        napi_create_string_utf8(env, e.k, NAPI_AUTO_LENGTH, &k);
        napi_set_element(env, names, i++, k);
    }
    napi_create_double(env, (double)m.deviceTotal, &total);
    NAPI_CHECK(env, napi_create_array_with_length(env, 3, &ret));
    napi_set_element(env, ret, 0, sizes);
    napi_set_element(env, ret, 1, names);
    napi_set_element(env, ret, 2, total);
    return ret;
}

napi_value LruCacheReset(napi_env env, napi_callback_info info)
{
    size_t argc = 0;
    Surface* s = unwrap(env, info, &argc, nullptr);
    if (!s || !s->vol || s->busy) return reject_now(env, "lruCache.reset: no idle volume on this object");
    napi_deferred d;
    napi_value promise, undef;
    napi_create_promise(env, &d, &promise);
    napi_get_undefined(env, &undef);
    const bcmc_status st = bcmc_cache_reset(s->vol);  // short: two fill kernels
    if (st == BCMC_OK) {
        napi_resolve_deferred(env, d, undef);
    } else {
        napi_value err, text;
        napi_create_string_utf8(env, status_message(s->ctx, st, "lruCache.reset").c_str(), NAPI_AUTO_LENGTH, &text);
        napi_create_error(env, nullptr, text, &err);
        napi_reject_deferred(env, d, err);
    }
    return promise;
}

void Finalize(napi_env, void* data, void*)
{
    auto* s = static_cast<Surface*>(data);
    if (s->vol) bcmc_volume_destroy(s->vol);
    if (s->ctx) bcmc_ctx_destroy(s->ctx);
    delete s;
}

napi_value Construct(napi_env env, napi_callback_info info)
{
    size_t argc = 1;
    napi_value argv[1], self;
    NAPI_CHECK(env, napi_get_cb_info(env, info, &argc, argv, &self, nullptr));
    bcmc_opts o;
    bcmc_opts_default(&o);
    if (argc > 0) {
        int32_t dev = 0;
        if (napi_get_value_int32(env, argv[0], &dev) == napi_ok) o.device = dev;  // else: a device object, use 0
    }
    auto* s = new Surface;
    const bcmc_status st = bcmc_ctx_create(&o, &s->ctx);
    if (st != BCMC_OK) {
        const std::string m = status_message(s->ctx, st, "new CompressedMarchingCubes");
        if (s->ctx) bcmc_ctx_destroy(s->ctx);
        delete s;
        napi_throw_error(env, nullptr, m.c_str());
        return nullptr;
    }
    NAPI_CHECK(env, napi_wrap(env, self, s, Finalize, nullptr, &s->self));
    return self;
}

napi_value Init(napi_env env, napi_value exports)
{
    const napi_property_descriptor methods[] = {
        {"setCompressedVolume", nullptr, SetCompressedVolume, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"computeSurface", nullptr, ComputeSurface, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"copyVertices", nullptr, CopyVertices, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"vertexBufferAddress", nullptr, VertexBufferAddress, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"stats", nullptr, Stats, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"reportMemoryUse", nullptr, ReportMemoryUse, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"lruCacheReset", nullptr, LruCacheReset, nullptr, nullptr, nullptr, napi_default, nullptr},
    };
    napi_value cls;
    NAPI_CHECK(env, napi_define_class(env, "CompressedMarchingCubes", NAPI_AUTO_LENGTH, Construct, nullptr,
                                      sizeof(methods) / sizeof(methods[0]), methods, &cls));
    NAPI_CHECK(env, napi_set_named_property(env, exports, "CompressedMarchingCubes", cls));
    return exports;
}

}  // namespace

NAPI_MODULE(NODE_GYP_MODULE_NAME, Init)
