// active_test.cuh -- the active-block test of compute_block_active.comp,
// shared by the per-query pipeline (pipeline.cu) and the batched engine
// (engine.cu).
#pragma once

#include "bcmc_internal.cuh"

namespace bcmc {

// compute_block_active.comp:24-61.  The reference tests, for each of the 26
// neighbours n, iso in [min(lo_b, lo_n), max(hi_b, hi_n)].  With A = (iso >=
// lo), B = (iso <= hi) that is (A_b || A_n) && (B_b || B_n), so over all
// neighbours (and b itself, which adds nothing new):
//   active = (A_b && anyB) || (B_b && anyA) || any(A_n && B_n)
// -- the same booleans, evaluated without branches or early exits.
__device__ __forceinline__ uint32_t block_is_active(const float2* __restrict__ ranges, const BlockGrid& g,
                                                    uint32_t b, float iso)
{
    const uint3 nb = g.nb;
    const float2 r = __ldg(ranges + b);
    const bool A = iso >= r.x, B = iso <= r.y;
    const uint3 c = block_coords(b, g);
    const int bx = (int)c.x, by = (int)c.y, bz = (int)c.z;
    bool anyA = false, anyB = false, anyC = false;
#pragma unroll
    for (int k = -1; k < 2; ++k)
#pragma unroll
        for (int j = -1; j < 2; ++j)
#pragma unroll
            for (int i = -1; i < 2; ++i) {
                const int cx = bx + i, cy = by + j, cz = bz + k;
                if (cx < 0 || cy < 0 || cz < 0 || cx >= (int)nb.x || cy >= (int)nb.y || cz >= (int)nb.z) continue;
                const float2 n = __ldg(ranges + ((uint32_t)cx + nb.x * ((uint32_t)cy + nb.y * (uint32_t)cz)));
                const bool an = iso >= n.x, bn = iso <= n.y;
                anyA |= an;
                anyB |= bn;
                anyC |= an && bn;
            }
    return ((A && anyB) || (B && anyA) || anyC) ? 1u : 0u;
}

__device__ __forceinline__ void range_bits(const float2 r, float iso, uint32_t& a, uint32_t& b)
{
    a = iso >= r.x ? 1u : 0u;
    b = iso <= r.y ? 1u : 0u;
}

// Active flags of the 4 consecutive blocks b0..b0+3 of one x-row: the 9
// neighbour rows (y-1..y+1, z-1..z+1) are read once for the 4 blocks (6 ranges
// per row), 13.5 loads per block instead of 27.
__device__ __forceinline__ uint32_t row4_active(const float2* __restrict__ ranges, const BlockGrid& g, uint3 c,
                                                uint32_t b0, float iso)
{
    const uint3 nb = g.nb;
    uint32_t anyA = 0, anyB = 0, anyC = 0, selfA = 0, selfB = 0;  // bit i = block b0+i
#pragma unroll
    for (int dz = -1; dz < 2; ++dz)
#pragma unroll
        for (int dy = -1; dy < 2; ++dy) {
            const int yy = (int)c.y + dy, zz = (int)c.z + dz;
            if (yy < 0 || zz < 0 || yy >= (int)nb.y || zz >= (int)nb.z) continue;
            const int64_t shift = (int64_t)dy * nb.x + (int64_t)dz * nb.x * nb.y;
            const float2* row = ranges + (int64_t)b0 + shift;  // position x0 of the neighbour row
            uint32_t A = 0, B = 0;  // bit p = position x0 - 1 + p, p = 0..5
#pragma unroll
            for (int p = 0; p < 6; ++p) {
                const int xx = (int)c.x - 1 + p;
                if (xx < 0 || xx >= (int)nb.x) continue;
                uint32_t a, b;
                range_bits(__ldg(row + (p - 1)), iso, a, b);
                A |= a << p;
                B |= b << p;
            }
            const uint32_t C = A & B;
            // window of block i covers positions i..i+2
            anyA |= (A | (A >> 1) | (A >> 2)) & 15u;
            anyB |= (B | (B >> 1) | (B >> 2)) & 15u;
            anyC |= (C | (C >> 1) | (C >> 2)) & 15u;
            if (dy == 0 && dz == 0) {
                selfA = (A >> 1) & 15u;
                selfB = (B >> 1) & 15u;
            }
        }
    return ((selfA & anyB) | (selfB & anyA) | anyC) & 15u;
}

}  // namespace bcmc
