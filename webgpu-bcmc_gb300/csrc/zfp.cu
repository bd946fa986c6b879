// zfp.cu -- ZFP fixed-rate float32 kernels: block ranges, decode into cache
// slots, full-volume decode, and the encoder used to produce streams.
#include "bcmc_impl.h"
#include "zfp_device.cuh"

namespace bcmc {

// Decode kernels: the CTA stages its blocks' compressed words in shared
// memory (zfp_stage_run / zfp_stage_block), each thread decodes one block
// from there (zfp_decode_staged).  Loop bounds are uniform across the CTA
// (the staging is followed by a barrier).
constexpr int kDecThreads = 128;
constexpr int kDecPerSm = 5;  // 96 registers: measured faster than 4 CTAs per SM at 128

__device__ __forceinline__ uint32_t* stage_words() { extern __shared__ __align__(16) uint32_t s_dyn[]; return s_dyn; }

__device__ __forceinline__ void store_block(float* __restrict__ dst, const float* v)
{
    float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
    for (int i = 0; i < 16; ++i) d4[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
}

// zfp_compute_block_range.comp:19-61: min/max over the voxels of each block
// that lie inside the volume (partial blocks at the +x/+y/+z faces are
// clipped), starting from (1e20, -1e20).
__global__ void __launch_bounds__(kDecThreads, kDecPerSm) k_block_ranges(const uint64_t* __restrict__ words, uint3 dims, uint3 nb,
                                                              uint32_t rate, uint64_t ranged,
                                                              float2* __restrict__ ranges)
{
    uint32_t* s_words = stage_words();
    uint32_t* pl = zfp_stage_planes(s_words, kDecThreads, rate);
    const uint64_t nblocks = (uint64_t)nb.x * nb.y * nb.z;
    for (uint64_t b0 = (uint64_t)blockIdx.x * kDecThreads; b0 < nblocks; b0 += (uint64_t)gridDim.x * kDecThreads) {
        const uint32_t n = (uint32_t)(nblocks - b0 < (uint64_t)kDecThreads ? nblocks - b0 : (uint64_t)kDecThreads);
        __syncthreads();
        zfp_stage_run(words, b0, n, rate, s_words);
        __syncthreads();
        if (threadIdx.x >= n) continue;
        const uint64_t b = b0 + threadIdx.x;
        if (b >= ranged) {  // beyond the reference's block count: the buffer's zero
            ranges[b] = make_float2(0.0f, 0.0f);
            continue;
        }
        float v[64];
        zfp_decode_staged(s_words + threadIdx.x * 2u * rate, 64u * rate, pl, v);
        const uint32_t bx = (uint32_t)(b % nb.x), by = (uint32_t)((b / nb.x) % nb.y),
                       bz = (uint32_t)(b / ((uint64_t)nb.x * nb.y));
        const uint32_t px = min(dims.x - 4u * bx, 4u), py = min(dims.y - 4u * by, 4u),
                       pz = min(dims.z - 4u * bz, 4u);
        float lo = 1e20f, hi = -1e20f;
#pragma unroll
        for (int z = 0; z < 4; ++z)
#pragma unroll
            for (int y = 0; y < 4; ++y)
#pragma unroll
                for (int x = 0; x < 4; ++x) {
                    if ((uint32_t)x < px && (uint32_t)y < py && (uint32_t)z < pz) {
                        const float f = v[16 * z + 4 * y + x];
                        lo = f < lo ? f : lo;
                        hi = hi < f ? f : hi;
                    }
                }
        ranges[b] = make_float2(lo, hi);
    }
}

// zfp_decompress_block.comp:29-39: decode ids[i] into its cache slot.
__global__ void __launch_bounds__(kDecThreads, kDecPerSm) k_decode_blocks(const uint64_t* __restrict__ words, uint32_t rate,
                                                               const uint32_t* __restrict__ ids, uint32_t n,
                                                               const int32_t* __restrict__ item_slots,
                                                               float* __restrict__ cache)
{
    uint32_t* s_words = stage_words();
    uint32_t* pl = zfp_stage_planes(s_words, kDecThreads, rate);
    if (threadIdx.x < 4) s_words[kDecThreads * 2u * rate + threadIdx.x] = 0u;
    for (uint32_t i0 = blockIdx.x * kDecThreads; i0 < n; i0 += gridDim.x * kDecThreads) {
        const uint32_t i = i0 + threadIdx.x;
        uint32_t b = 0;
        int32_t slot = -1;
        __syncthreads();
        if (i < n) {
            b = ids[i];
            slot = item_slots[b];
            if (slot >= 0) zfp_stage_block(words, b, rate, s_words);
        }
        __syncthreads();
        if (slot < 0) continue;  // not cached: nothing to decode into
        float v[64];
        zfp_decode_staged(s_words + threadIdx.x * 2u * rate, 64u * rate, pl, v);
        store_block(cache + (uint64_t)slot * 64u, v);
    }
}

__global__ void __launch_bounds__(kDecThreads, kDecPerSm) k_decode_volume(const uint64_t* __restrict__ words, uint64_t nblocks,
                                                               uint32_t rate, float* __restrict__ out)
{
    uint32_t* s_words = stage_words();
    uint32_t* pl = zfp_stage_planes(s_words, kDecThreads, rate);
    const uint32_t wb = threadIdx.x & ~31u;  // the warp's first block in the run
    for (uint64_t b0 = (uint64_t)blockIdx.x * kDecThreads; b0 < nblocks; b0 += (uint64_t)gridDim.x * kDecThreads) {
        const uint32_t n = (uint32_t)(nblocks - b0 < (uint64_t)kDecThreads ? nblocks - b0 : (uint64_t)kDecThreads);
        __syncthreads();
        zfp_stage_run(words, b0, n, rate, s_words);
        __syncthreads();
        if (wb >= n) continue;  // the whole warp
        const bool mine = threadIdx.x < n;
        float v[64];
        if (mine) zfp_decode_staged(s_words + threadIdx.x * 2u * rate, 64u * rate, pl, v);
        zfp_store_warp(pl, v, mine, out + (b0 + wb) * 64u, n - wb);
    }
}

// Encoder: gathers the block (zfp's padding of partial blocks) and codes it.
__device__ __forceinline__ void pad_row(float* p, uint32_t n, uint32_t s)
{
    switch (n) {
    case 0: p[0] = 0.0f; [[fallthrough]];
    case 1: p[1 * s] = p[0]; [[fallthrough]];
    case 2: p[2 * s] = p[1 * s]; [[fallthrough]];
    case 3: p[3 * s] = p[0]; [[fallthrough]];
    default: break;
    }
}

__global__ void __launch_bounds__(128) k_encode(const float* __restrict__ field, uint3 dims, uint3 nb,
                                                uint32_t max_bits, unsigned long long* words)
{
    const uint64_t nblocks = (uint64_t)nb.x * nb.y * nb.z;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblocks;
         b += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x0 = 4u * (uint32_t)(b % nb.x), y0 = 4u * (uint32_t)((b / nb.x) % nb.y),
                       z0 = 4u * (uint32_t)(b / ((uint64_t)nb.x * nb.y));
        const uint32_t nx = min(dims.x - x0, 4u), ny = min(dims.y - y0, 4u), nz = min(dims.z - z0, 4u);
        float blk[64];
        for (uint32_t z = 0; z < nz; ++z) {
            for (uint32_t y = 0; y < ny; ++y) {
                const float* row = field + (uint64_t)x0 + (uint64_t)dims.x * ((uint64_t)(y0 + y) + (uint64_t)dims.y * (z0 + z));
                for (uint32_t x = 0; x < nx; ++x) blk[16 * z + 4 * y + x] = row[x];
                pad_row(blk + 16 * z + 4 * y, nx, 1);
            }
            for (uint32_t x = 0; x < 4; ++x) pad_row(blk + 16 * z + x, ny, 4);
        }
        for (uint32_t y = 0; y < 4; ++y)
            for (uint32_t x = 0; x < 4; ++x) pad_row(blk + 4 * y + x, nz, 16);
        BitWriter bw;
        bw.init(words, b * max_bits);
        zfp_encode_block(blk, max_bits, bw);
        bw.finish();
    }
}

static int grid_for(bcmc_ctx* ctx, uint64_t n, int threads, int per_sm)
{
    const uint64_t want = (n + threads - 1) / threads;
    const uint64_t cap = (uint64_t)ctx->num_sms * per_sm;
    return (int)(want < cap ? (want ? want : 1) : cap);
}

// One thread per block (grid-stride only beyond 2^31 - 1 CTAs).
static int grid_all(uint64_t n, int threads)
{
    const uint64_t want = (n + threads - 1) / threads;
    return (int)(want == 0 ? 1 : (want < 0x7fffffffull ? want : 0x7fffffffull));
}

void zfp_ranges_launch(bcmc_ctx* ctx, const uint64_t* words, const uint32_t dims[3], uint32_t max_bits,
                       float* ranges, cudaStream_t s)
{
    const uint3 d = make_uint3(dims[0], dims[1], dims[2]);
    const uint3 nb = make_uint3(div_up(dims[0], 4), div_up(dims[1], 4), div_up(dims[2], 4));
    const uint64_t n = (uint64_t)nb.x * nb.y * nb.z;
    // zfp_compute_block_range.comp:22 counts (padded x * padded y) / 64 * padded z
    // blocks in u32, which truncates when nb.x * nb.y is not a multiple of 4;
    // the blocks past that count keep the zero of the new range buffer
    // (compressed_marching_cubes.js:526-529).  BCMC_FLAG_FULL_RANGES ranges all.
    const uint32_t ref_count = (4u * nb.x * 4u * nb.y) / 64u * (4u * nb.z);
    const uint64_t ranged = (ctx->opts.flags & BCMC_FLAG_FULL_RANGES) ? n : (ref_count < n ? ref_count : n);
    const uint32_t rate = max_bits / 64u;
    const size_t smem = zfp_stage_smem(kDecThreads, rate);
    allow_smem(k_block_ranges, smem);
    k_block_ranges<<<grid_all(n, kDecThreads), kDecThreads, smem, s>>>(words, d, nb, rate, ranged,
                                                                      reinterpret_cast<float2*>(ranges));
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void zfp_decode_blocks_launch(bcmc_ctx* ctx, const uint64_t* words, uint32_t max_bits, const uint32_t* ids,
                              uint32_t n, const int32_t* item_slots, float* cache, cudaStream_t s)
{
    if (n == 0) return;
    const uint32_t rate = max_bits / 64u;
    const size_t smem = zfp_stage_smem(kDecThreads, rate);
    allow_smem(k_decode_blocks, smem);
    k_decode_blocks<<<grid_for(ctx, n, kDecThreads, 16), kDecThreads, smem, s>>>(words, rate, ids, n, item_slots,
                                                                                 cache);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void zfp_decode_volume_launch(bcmc_ctx* ctx, const uint64_t* words, uint64_t nblocks, uint32_t max_bits,
                              float* out, cudaStream_t s)
{
    if (nblocks == 0) return;
    const uint32_t rate = max_bits / 64u;
    const size_t smem = zfp_stage_smem(kDecThreads, rate);
    allow_smem(k_decode_volume, smem);
    k_decode_volume<<<grid_all(nblocks, kDecThreads), kDecThreads, smem, s>>>(words, nblocks, rate, out);
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

void zfp_encode_launch(bcmc_ctx* ctx, const float* field, const uint32_t dims[3], uint32_t max_bits,
                       uint64_t* words, cudaStream_t s)
{
    const uint3 d = make_uint3(dims[0], dims[1], dims[2]);
    const uint3 nb = make_uint3(div_up(dims[0], 4), div_up(dims[1], 4), div_up(dims[2], 4));
    const uint64_t n = (uint64_t)nb.x * nb.y * nb.z;
    k_encode<<<grid_for(ctx, n, 128, 16), 128, 0, s>>>(field, d, nb, max_bits,
                                                       reinterpret_cast<unsigned long long*>(words));
    count_launches(1);
    BCMC_CUDA(cudaGetLastError());
}

}  // namespace bcmc
