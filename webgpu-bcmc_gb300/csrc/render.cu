// render.cu -- headless rendering of an isosurface mesh into a device image:
// the reference's render pass (js/bcmc.js:174-190,237-265,377-391) with the
// shading of shaders/mc_isosurface.vert/.frag, as CUDA kernels instead of a
// graphics pipeline (no window, swapchain or graphics API).
//
//   vertex stage  unpack_launch (unpack.cu): world and clip positions, plus
//                 the fog entry distance of mc_isosurface.vert:35-49
//   k_raster      one thread per triangle: clip -> NDC -> pixels (WebGPU
//                 conventions: y up in NDC, depth in [0, 1]), edge functions
//                 with a top-left rule at pixel centres, depth "less" against a
//                 buffer cleared to 1.0 -- each covered pixel takes the 64-bit
//                 atomicMin of (depth bits, triangle id), so the result does not
//                 depend on thread order
//   k_resolve     one thread per pixel: the winning triangle's fragment shading
//                 (mc_isosurface.frag:15-40: flat normal, Blinn-Phong, optional
//                 fog), background (1, 1, 1, 1) where no triangle won
// Triangles with a vertex at w <= 1e-6 (behind the eye) or more than 2^21
// pixels off the image are not drawn: there is no clipping.  Every float
// operation is an explicitly rounded IEEE operation (no contraction), so the
// CPU restatement in the oracle reproduces the depth/triangle buffers bit for
// bit.
#include "bcmc_impl.h"

namespace bcmc {
namespace {

struct RenderArgs {
    const float* world;  // 3 per vertex
    const float* clip;   // 4 per vertex
    const float* tenter; // 1 per vertex (fog), or null
    uint64_t ntri;
    uint32_t w, h;
    float eye[3];
    int fog;
    unsigned long long* keys;  // per pixel
    float* rgba;               // 4 per pixel
    float* depth;              // 1 per pixel, or null
    uint32_t* triangle;        // 1 per pixel, or null
    uint32_t* big;             // triangles left to k_raster_big
    unsigned int* nbig;
};

// a triangle whose pixel box holds more than this many pixels is rasterised by
// a whole CTA (k_raster_big) instead of one thread
constexpr long long kBigBox = 256;

// Screen positions are snapped to 1/256 pixel (the sub-pixel precision
// WebGPU's rasterisers use) and the edge functions are evaluated in 64-bit
// integers, exactly: the shared edge of two triangles gives opposite values
// in the two, so with the top-left rule every pixel centre on it is covered
// by exactly one of them (no cracks, no double coverage).
constexpr float kSub = 256.0f;          // sub-pixel steps per pixel
constexpr float kGuard = 2097152.0f;    // |screen coordinate| limit in pixels (2^21)

struct Tri {
    int x[3], y[3];   // fixed-point screen positions, positive winding
    float z[3];       // NDC depth
    int idx[3];       // which input vertex each of the three is
    long long area;   // twice the area in fixed-point units, > 0
};

__device__ __forceinline__ long long edge_fn(int ax, int ay, int bx, int by, int px, int py)
{
    return (long long)(bx - ax) * (long long)(py - ay) - (long long)(by - ay) * (long long)(px - ax);
}

// top-left rule (screen y down, positive winding): a pixel centre exactly on
// an edge belongs to the triangle when the edge is a top edge (horizontal,
// running in +x) or a left edge (running in -y)
__device__ __forceinline__ bool top_left(int ax, int ay, int bx, int by) { return (ay == by && bx > ax) || (by < ay); }

// false when the triangle is not drawn: a vertex at w <= 1e-6, a vertex
// beyond the guard band (or not finite), or zero area
__device__ __forceinline__ bool tri_setup(const float* c, uint32_t w, uint32_t h, Tri& t)
{
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float cw = c[4 * k + 3];
        if (!(cw > 1e-6f)) return false;
        const float nx = __fdiv_rn(c[4 * k], cw), ny = __fdiv_rn(c[4 * k + 1], cw);
        const float sx = __fmul_rn(__fadd_rn(__fmul_rn(nx, 0.5f), 0.5f), (float)w);
        const float sy = __fmul_rn(__fsub_rn(0.5f, __fmul_rn(ny, 0.5f)), (float)h);
        if (!(fabsf(sx) <= kGuard && fabsf(sy) <= kGuard)) return false;
        t.x[k] = (int)rintf(__fmul_rn(sx, kSub));
        t.y[k] = (int)rintf(__fmul_rn(sy, kSub));
        t.z[k] = __fdiv_rn(c[4 * k + 2], cw);
        t.idx[k] = k;
    }
    t.area = edge_fn(t.x[0], t.y[0], t.x[1], t.y[1], t.x[2], t.y[2]);
    if (t.area == 0) return false;
    if (t.area < 0) {  // make the winding positive
        int tmp = t.x[1]; t.x[1] = t.x[2]; t.x[2] = tmp;
        tmp = t.y[1]; t.y[1] = t.y[2]; t.y[2] = tmp;
        const float tz = t.z[1]; t.z[1] = t.z[2]; t.z[2] = tz;
        t.idx[1] = 2;
        t.idx[2] = 1;
        t.area = -t.area;
    }
    return true;
}

// floor(v / 256) for any sign
__device__ __forceinline__ int floor_div256(int v) { return v >= 0 ? v / 256 : -((255 - v) / 256); }

__device__ __forceinline__ void edges_at(const Tri& t, int px, int py, long long e[3])
{
    const int cx = px * 256 + 128, cy = py * 256 + 128;  // pixel centre
    e[0] = edge_fn(t.x[1], t.y[1], t.x[2], t.y[2], cx, cy);
    e[1] = edge_fn(t.x[2], t.y[2], t.x[0], t.y[0], cx, cy);
    e[2] = edge_fn(t.x[0], t.y[0], t.x[1], t.y[1], cx, cy);
}

// coverage and depth test of one pixel centre: the 64-bit atomicMin of
// (depth bits, triangle index) keeps the nearest fragment, the earlier
// triangle on ties (depth >= 0, so its bits order as the values do)
__device__ __forceinline__ void shade_sample(const RenderArgs& a, const Tri& t, uint32_t ti, int px, int py)
{
    long long e[3];
    edges_at(t, px, py, e);
    const bool in0 = e[0] > 0 || (e[0] == 0 && top_left(t.x[1], t.y[1], t.x[2], t.y[2]));
    const bool in1 = e[1] > 0 || (e[1] == 0 && top_left(t.x[2], t.y[2], t.x[0], t.y[0]));
    const bool in2 = e[2] > 0 || (e[2] == 0 && top_left(t.x[0], t.y[0], t.x[1], t.y[1]));
    if (!(in0 && in1 && in2)) return;
    // depth: NDC z interpolated linearly in screen space
    const float z = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(__ll2float_rn(e[0]), t.z[0]),
                                                  __fmul_rn(__ll2float_rn(e[1]), t.z[1])),
                                        __fmul_rn(__ll2float_rn(e[2]), t.z[2])),
                              __ll2float_rn(t.area));
    if (!(z >= 0.0f && z < 1.0f)) return;  // outside the depth range, or not less than the clear value
    const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | ti;
    atomicMin(a.keys + (uint64_t)py * a.w + px, key);
}

__global__ void __launch_bounds__(256) k_raster(RenderArgs a)
{
    for (uint64_t ti = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; ti < a.ntri;
         ti += (uint64_t)gridDim.x * blockDim.x) {
        Tri t;
        if (!tri_setup(a.clip + 12 * ti, a.w, a.h, t)) continue;
        const int xmin = min(t.x[0], min(t.x[1], t.x[2])), xmax = max(t.x[0], max(t.x[1], t.x[2]));
        const int ymin = min(t.y[0], min(t.y[1], t.y[2])), ymax = max(t.y[0], max(t.y[1], t.y[2]));
        // pixels whose centre (256 p + 128) lies in the box, clamped to the image
        const int x0 = max(0, floor_div256(xmin - 128 + 255)), x1 = min((int)a.w - 1, floor_div256(xmax - 128));
        const int y0 = max(0, floor_div256(ymin - 128 + 255)), y1 = min((int)a.h - 1, floor_div256(ymax - 128));
        if (x0 > x1 || y0 > y1) continue;
        if ((long long)(x1 - x0 + 1) * (y1 - y0 + 1) > kBigBox) {
            a.big[atomicAdd(a.nbig, 1u)] = (uint32_t)ti;
            continue;
        }
        for (int py = y0; py <= y1; ++py)
            for (int px = x0; px <= x1; ++px) shade_sample(a, t, (uint32_t)ti, px, py);
    }
}

// the triangles k_raster set aside, one CTA each, its threads striding over
// the pixel box
__global__ void __launch_bounds__(256) k_raster_big(RenderArgs a)
{
    const unsigned int nbig = *a.nbig;
    for (unsigned int b = blockIdx.x; b < nbig; b += gridDim.x) {
        const uint32_t ti = a.big[b];
        Tri t;
        tri_setup(a.clip + 12 * (uint64_t)ti, a.w, a.h, t);
        const int xmin = min(t.x[0], min(t.x[1], t.x[2])), xmax = max(t.x[0], max(t.x[1], t.x[2]));
        const int ymin = min(t.y[0], min(t.y[1], t.y[2])), ymax = max(t.y[0], max(t.y[1], t.y[2]));
        const int x0 = max(0, floor_div256(xmin - 128 + 255)), x1 = min((int)a.w - 1, floor_div256(xmax - 128));
        const int y0 = max(0, floor_div256(ymin - 128 + 255)), y1 = min((int)a.h - 1, floor_div256(ymax - 128));
        const long long bw = x1 - x0 + 1, npix = bw * (y1 - y0 + 1);
        for (long long p = threadIdx.x; p < npix; p += blockDim.x)
            shade_sample(a, t, ti, x0 + (int)(p % bw), y0 + (int)(p / bw));
    }
}

__device__ __forceinline__ float3 f3(const float* p) { return make_float3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b)
{
    return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float dot3(float3 a, float3 b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float3 scale3(float3 a, float s)
{
    return make_float3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s));
}
// GLSL's definitions: normalize(x) = x / length(x), min(x, y) = y < x ? y : x,
// max(x, y) = x < y ? y : x, clamp(x, a, b) = min(max(x, a), b)
__device__ __forceinline__ float3 norm3(float3 a)
{
    const float len = __fsqrt_rn(dot3(a, a));
    return make_float3(__fdiv_rn(a.x, len), __fdiv_rn(a.y, len), __fdiv_rn(a.z, len));
}
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return make_float3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
                       __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
                       __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float clamp01(float x) { return gmin(gmax(x, 0.0f), 1.0f); }

__global__ void __launch_bounds__(256) k_resolve(RenderArgs a)
{
    const uint64_t npix = (uint64_t)a.w * a.h;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < npix; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long key = a.keys[i];
        float4 out = make_float4(1.0f, 1.0f, 1.0f, 1.0f);  // clearValue (js/bcmc.js:179)
        float depth = 1.0f;
        uint32_t tri = 0xffffffffu;
        if (key != ~0ull) {
            const uint64_t t = key & 0xffffffffull;
            tri = (uint32_t)t;
            depth = __uint_as_float((uint32_t)(key >> 32));
            Tri tr;
            tri_setup(a.clip + 12 * t, a.w, a.h, tr);  // drawn, so set up as in k_raster
            long long ee[3];
            edges_at(tr, (int)(i % a.w), (int)(i / a.w), ee);
            const float e[3] = {__ll2float_rn(ee[0]), __ll2float_rn(ee[1]), __ll2float_rn(ee[2])};
            const int* idx = tr.idx;
            // perspective-correct weights of the varyings: (e_k / w_k) / sum
            float pw[3], psum = 0.0f;
            for (int k = 0; k < 3; ++k) {
                pw[k] = __fdiv_rn(e[k], a.clip[12 * t + 4 * idx[k] + 3]);
                psum = __fadd_rn(psum, pw[k]);
            }
            float3 wp = make_float3(0.0f, 0.0f, 0.0f);
            float te = 0.0f;
            for (int k = 0; k < 3; ++k) {
                const float b = __fdiv_rn(pw[k], psum);
                const float* wk = a.world + 3 * (3 * t + idx[k]);
                wp = make_float3(__fadd_rn(wp.x, __fmul_rn(b, wk[0])), __fadd_rn(wp.y, __fmul_rn(b, wk[1])),
                                 __fadd_rn(wp.z, __fmul_rn(b, wk[2])));
                if (a.fog) te = __fadd_rn(te, __fmul_rn(b, a.tenter[3 * t + idx[k]]));
            }
            // mc_isosurface.frag:15-40
            const float3 eye = make_float3(a.eye[0], a.eye[1], a.eye[2]);
            float3 v = sub3(wp, eye);
            const float dist = __fsqrt_rn(dot3(v, v));
            v = scale3(norm3(v), -1.0f);
            const float3 light = v;
            const float* w0 = a.world + 9 * t;
            float3 n = norm3(cross3(sub3(f3(w0 + 3), f3(w0)), sub3(f3(w0 + 6), f3(w0))));
            if (dot3(n, light) < 0.0f) n = scale3(n, -1.0f);
            const float3 base = make_float3(0.3f, 0.3f, 0.9f);
            const float3 hv = norm3(make_float3(__fadd_rn(v.x, light.x), __fadd_rn(v.y, light.y), __fadd_rn(v.z, light.z)));
            const float diff = __fmul_rn(0.6f, clamp01(dot3(light, n)));
            const float sp = clamp01(dot3(n, hv));
            const float sp2 = __fmul_rn(sp, sp);
            const float spec = __fmul_rn(0.1f, powf(sp, 5.0f));
            float3 col = make_float3(__fadd_rn(__fadd_rn(__fmul_rn(base.x, 0.2f), __fmul_rn(diff, base.x)), spec),
                                     __fadd_rn(__fadd_rn(__fmul_rn(base.y, 0.2f), __fmul_rn(diff, base.y)), spec),
                                     __fadd_rn(__fadd_rn(__fmul_rn(base.z, 0.2f), __fmul_rn(diff, base.z)), spec));
            if (a.fog) {
                const float fog = expf(__fmul_rn(-1.0f, gmax(__fsub_rn(dist, __fadd_rn(te, 0.1f)), 0.0f)));
                const float rest = __fsub_rn(1.0f, fog);
                col = make_float3(__fadd_rn(__fmul_rn(fog, col.x), rest), __fadd_rn(__fmul_rn(fog, col.y), rest),
                                  __fadd_rn(__fmul_rn(fog, col.z), rest));
            }
            out = make_float4(col.x, col.y, col.z, 1.0f);
        }
        reinterpret_cast<float4*>(a.rgba)[i] = out;
        if (a.depth) a.depth[i] = depth;
        if (a.triangle) a.triangle[i] = tri;
    }
}

// mc_isosurface.vert:35-49: distance along the eye ray where it enters the
// volume's box [-scale/2, scale/2], clamped at 0
__global__ void __launch_bounds__(256) k_fog_enter(const float* world, uint64_t n, float3 eye, float3 half,
                                                   float* tenter)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float3 d = norm3(sub3(f3(world + 3 * i), eye));
        const float o[3] = {eye.x, eye.y, eye.z}, dd[3] = {d.x, d.y, d.z}, hh[3] = {half.x, half.y, half.z};
        float tmin[3];
        for (int k = 0; k < 3; ++k) {
            const float inv = __fdiv_rn(1.0f, dd[k]);
            const float ta = __fmul_rn(__fsub_rn(-hh[k], o[k]), inv), tb = __fmul_rn(__fsub_rn(hh[k], o[k]), inv);
            tmin[k] = gmin(ta, tb);
        }
        tenter[i] = gmax(gmax(tmin[0], gmax(tmin[1], tmin[2])), 0.0f);
    }
}

int grid_of(bcmc_ctx* ctx, uint64_t n)
{
    const uint64_t want = (n + 255) / 256, cap = (uint64_t)ctx->num_sms * 16;
    return (int)(want == 0 ? 1 : (want < cap ? want : cap));
}

}  // namespace

void render_launch(bcmc_ctx* ctx, const uint2* verts, uint64_t n, const uint32_t dims[3], const float scale[3],
                   const bcmc_render_params& p, float* rgba, float* depth, uint32_t* triangle, cudaStream_t s)
{
    const uint64_t ntri = n / 3, nv = ntri * 3, npix = (uint64_t)p.width * p.height;
    // working buffers, carved from one grow-only context allocation: world and
    // clip positions, fog entry distances, the per-pixel keys, the list of
    // large triangles and its counter
    auto up = [](uint64_t b) { return (b + 255) & ~uint64_t(255); };
    const uint64_t b_world = up(nv * 12), b_clip = up(nv * 16), b_tenter = p.fog ? up(nv * 4) : 0,
                   b_keys = up(npix * 8), b_big = up((ntri + 1) * 4);
    const uint64_t need = b_world + b_clip + b_tenter + b_keys + b_big;
    if (need > ctx->render_bytes) {
        dev_free(ctx, ctx->d_render, ctx->render_bytes);
        ctx->d_render = nullptr;
        ctx->render_bytes = 0;
        ctx->d_render = dev_alloc(ctx, need);
        ctx->render_bytes = need;
    }
    char* base = static_cast<char*>(ctx->d_render);
    float* world = reinterpret_cast<float*>(base);
    float* clip = reinterpret_cast<float*>(base + b_world);
    float* tenter = p.fog ? reinterpret_cast<float*>(base + b_world + b_clip) : nullptr;
    unsigned long long* keys = reinterpret_cast<unsigned long long*>(base + b_world + b_clip + b_tenter);
    uint32_t* big = reinterpret_cast<uint32_t*>(base + b_world + b_clip + b_tenter + b_keys);
    try {
        BCMC_CUDA(cudaMemsetAsync(keys, 0xff, npix * 8, s));
        if (nv) {
            BCMC_CUDA(cudaMemsetAsync(big + ntri, 0, 4, s));
            unpack_launch(ctx, verts, nv, dims, scale, p.proj_view, world, clip, s);
            if (p.fog) {
                const float3 half = make_float3((scale ? scale[0] : 1.0f) * 0.5f, (scale ? scale[1] : 1.0f) * 0.5f,
                                                (scale ? scale[2] : 1.0f) * 0.5f);
                k_fog_enter<<<grid_of(ctx, nv), 256, 0, s>>>(world, nv, make_float3(p.eye_pos[0], p.eye_pos[1],
                                                                                    p.eye_pos[2]), half, tenter);
                count_launches(1);
            }
        }
        RenderArgs a{};
        a.world = world;
        a.clip = clip;
        a.tenter = tenter;
        a.ntri = ntri;
        a.w = p.width;
        a.h = p.height;
        for (int k = 0; k < 3; ++k) a.eye[k] = p.eye_pos[k];
        a.fog = p.fog ? 1 : 0;
        a.keys = keys;
        a.rgba = rgba;
        a.depth = depth;
        a.triangle = triangle;
        a.big = big;
        a.nbig = reinterpret_cast<unsigned int*>(big + ntri);
        if (ntri) {
            k_raster<<<grid_of(ctx, ntri), 256, 0, s>>>(a);
            k_raster_big<<<ctx->num_sms * 4, 256, 0, s>>>(a);
            count_launches(2);
        }
        k_resolve<<<grid_of(ctx, npix), 256, 0, s>>>(a);
        count_launches(1);
        BCMC_CUDA(cudaGetLastError());
        BCMC_CUDA(cudaStreamSynchronize(s));  // the working buffers are free again when this returns
    } catch (...) {
        cudaStreamSynchronize(s);
        throw;
    }
}

}  // namespace bcmc
