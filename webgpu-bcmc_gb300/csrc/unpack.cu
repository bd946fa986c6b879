// unpack.cu -- world-space positions of packed vertices: the position math of
// the reference's vertex stage (shaders/mc_isosurface.vert:51-60 with
// block_vertex_position.comp:19-26), as a CUDA kernel for consumers of the
// mesh that do not decode the packed form themselves.
#include "bcmc_impl.h"

namespace bcmc {
namespace {

struct UnpackArgs {
    const uint2* verts;
    uint64_t n;
    BlockGrid grid;
    float dims[3], scale[3];
    float m[16];  // column-major view-projection
    int has_clip;
    float* world;  // 3 floats per vertex
    float* clip;   // 4 floats per vertex
};

__global__ void __launch_bounds__(256) k_unpack(UnpackArgs a)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 v = __ldg(a.verts + i);
        const uint3 b = block_coords(v.y, a.grid);
        const float q[3] = {(float)((v.x & 0x3ff00000u) >> 20), (float)((v.x & 0x000ffc00u) >> 10),
                            (float)(v.x & 0x000003ffu)};
        const float bp[3] = {__fmul_rn(4.0f, (float)b.x), __fmul_rn(4.0f, (float)b.y), __fmul_rn(4.0f, (float)b.z)};
        float w[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            // decompress_position: (quantized * 4.0) / 1023 + 0.5
            const float d = __fadd_rn(__fdiv_rn(__fmul_rn(q[k], 4.0f), 1023.0f), 0.5f);
            // world = scale * ((block_pos + d) / dims - 0.5)
            w[k] = __fmul_rn(a.scale[k], __fsub_rn(__fdiv_rn(__fadd_rn(bp[k], d), a.dims[k]), 0.5f));
            a.world[3 * i + k] = w[k];
        }
        if (a.has_clip) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                float acc = __fmul_rn(a.m[r], w[0]);
                acc = __fadd_rn(acc, __fmul_rn(a.m[4 + r], w[1]));
                acc = __fadd_rn(acc, __fmul_rn(a.m[8 + r], w[2]));
                acc = __fadd_rn(acc, a.m[12 + r]);  // * 1.0
                a.clip[4 * i + r] = acc;
            }
        }
    }
}

}  // namespace

void unpack_launch(bcmc_ctx* ctx, const uint2* verts, uint64_t n, const uint32_t dims[3], const float scale[3],
                   const float* proj_view, float* world, float* clip, cudaStream_t s)
{
    if (n == 0) return;
    UnpackArgs a{};
    a.verts = verts;
    a.n = n;
    a.grid = make_block_grid(make_uint3(div_up(dims[0], 4u), div_up(dims[1], 4u), div_up(dims[2], 4u)));
    for (int k = 0; k < 3; ++k) {
        a.dims[k] = (float)dims[k];
        a.scale[k] = scale ? scale[k] : 1.0f;
    }
    a.has_clip = proj_view && clip ? 1 : 0;
    for (int k = 0; k < 16; ++k) a.m[k] = proj_view ? proj_view[k] : (k % 5 == 0 ? 1.0f : 0.0f);
    a.world = world;
    a.clip = clip;
    const uint64_t want = (n + 255) / 256, cap = (uint64_t)ctx->num_sms * 16;
    k_unpack<<<(int)(want < cap ? want : cap), 256, 0, s>>>(a);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

}  // namespace bcmc
