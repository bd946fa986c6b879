// mc_vertex.cuh -- the marching-cubes case tables as the kernels use them
// (built at compile time from the reference's tri table) and the position of
// one vertex.  Free of the CUDA runtime, so that a host build of it can be
// checked against the oracle; mc_common.cuh places the tables in device memory.
#pragma once

#include <math.h>
#include <stdint.h>

namespace bcmc {

namespace mc_detail {
#define BCMC_TABLE_QUALIFIER constexpr
#include "mc_tables.inc"
#undef BCMC_TABLE_QUALIFIER
// corner i of a cell (compute_vertex_values.comp:48-57), packed x|y<<1|z<<2
constexpr uint8_t kCorner[8] = {0, 1, 3, 2, 4, 5, 7, 6};
// cube edge -> its two corners (compute_block_vertices.comp:10-23)
constexpr uint8_t kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {6, 5},
                                  {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

// The case table as the kernels use it: each entry's edge as the packed
// corner pair o0 | o1 << 3 (0xff past the case's last entry), and each
// case's vertex count -- derived at compile time from the table above.
struct TriCorners {
    uint8_t corners[256][16];
    uint8_t count[256];
};
constexpr TriCorners make_tri_corners()
{
    TriCorners t{};
    for (int c = 0; c < 256; ++c) {
        int n = 0;
        for (int k = 0; k < 16; ++k) {
            const int e = kTriEdges[c][k];
            t.corners[c][k] = e < 0 ? (uint8_t)0xff : (uint8_t)(kCorner[kEdge[e][0]] | (kCorner[kEdge[e][1]] << 3));
            if (e >= 0 && n == k) ++n;
        }
        t.count[c] = (uint8_t)n;
    }
    return t;
}
// The emit's view of the same table: per (case, k) the k-th vertex's edge as
// bits 0-4 its first corner's offset in the block's 5^3 grid relative to the
// cell (x + 5y + 25z), bits 5-9 its second corner's, bits 10-11 the edge's
// axis (0, 1, 2 = x, y, z) and bits 12-14 the first corner (x|y<<1|z<<2).
constexpr uint32_t grid_off(uint32_t o) { return (o & 1u) + 5u * ((o >> 1) & 1u) + 25u * (o >> 2); }
struct TriEdges {
    uint16_t e[256][16];
};
constexpr TriEdges make_tri_edges()
{
    TriEdges t{};
    for (int c = 0; c < 256; ++c)
        for (int k = 0; k < 16; ++k) {
            const int e = kTriEdges[c][k];
            if (e < 0) {
                t.e[c][k] = 0xffff;
                continue;
            }
            const uint32_t o0 = kCorner[kEdge[e][0]], o1 = kCorner[kEdge[e][1]];
            t.e[c][k] = (uint16_t)(grid_off(o0) | (grid_off(o1) << 5) | (((o0 ^ o1) >> 1) << 10) | (o0 << 12));
        }
    return t;
}
// Per cell (x + 4y + 16z of a block) and corner: the corner's packed 10-bit
// quantized position (block_vertex_position.comp:9-17) on all three axes,
// floor(c * 255.75) for coordinate c in 0..4; a vertex keeps two of these
// axes, since its edge varies only along the third.
struct CornerPack {
    uint32_t p[64][8];
};
constexpr uint32_t q10(uint32_t c) { return (c * 1023u) >> 2; }
constexpr CornerPack make_corner_pack()
{
    CornerPack t{};
    for (uint32_t cc = 0; cc < 64; ++cc)
        for (uint32_t o = 0; o < 8; ++o)
            t.p[cc][o] = (q10((cc & 3u) + (o & 1u)) << 20) | (q10(((cc >> 2) & 3u) + ((o >> 1) & 1u)) << 10) |
                         q10((cc >> 4) + (o >> 2));
    return t;
}
// every edge is axis aligned (its corners differ on one axis), which the emit's
// exact treatment of the two fixed axes relies on
constexpr bool edges_axis_aligned()
{
    for (int e = 0; e < 12; ++e) {
        const uint32_t x = (uint32_t)(kCorner[kEdge[e][0]] ^ kCorner[kEdge[e][1]]);
        if (x != 1u && x != 2u && x != 4u) return false;
    }
    return true;
}
static_assert(edges_axis_aligned(), "cube edges vary along one axis");
static_assert(make_corner_pack().p[63][7] == ((1023u << 20) | (1023u << 10) | 1023u), "last cell's far corner");
}  // namespace mc_detail

// block_vertex_position.comp:9-17 with the f32 operations of
// compute_block_vertices.comp:62-74,161-162 in the reference's order, each
// rounded on its own (no contraction).
__device__ __forceinline__ uint32_t quantize(float p)
{
    const float f = __fmul_rn(__fmul_rn(__fsub_rn(p, 0.5f), 0.25f), 1023.0f);
    return __float2uint_rz(f) & 0x3ffu;  // saturating float->uint, as WGSL u32()
}

// A vertex's packed position (compute_block_vertices.comp:62-74,161-162,
// block_vertex_position.comp:9-17): `e` its entry of the emit table
// (TriEdges), `cc` its cell in the block, `vol` the block's 5^3 grid, `cp`
// the corner pack table (CornerPack), both in shared memory.  The
// interpolation is the reference's f32 expression, each operation rounded on
// its own; the two axes the edge does not vary along are exact (a + v + 0.5
// quantizes to floor((a + v) * 255.75)) and come from the table.
__device__ __forceinline__ uint32_t mc_vertex(uint32_t e, uint32_t cc, const float* vol, const uint32_t* cp, float iso)
{
    const uint32_t g = cc + ((cc >> 2) & 3u) + 9u * (cc >> 4);  // the cell's corner 0 in the grid
    const float fa = vol[g + (e & 31u)], fb = vol[g + ((e >> 5) & 31u)];
    float tt = 0.0f;
    if (!(fabsf(__fsub_rn(fa, fb)) < 0.001f)) tt = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
    const uint32_t d = (e >> 10) & 3u, oa = (e >> 12) & 7u;
    if (isfinite(tt)) {
        const uint32_t ad = (oa >> d) & 1u, vd = (cc >> (2u * d)) & 3u;
        const float pd = __fadd_rn(__fadd_rn(ad ? __fsub_rn(1.0f, tt) : tt, (float)vd), 0.5f);
        const uint32_t sh = 20u - 10u * d;
        return (cp[8u * cc + oa] & ~(1023u << sh)) | (quantize(pd) << sh);
    }
    // tt infinite or NaN: the general expression on every axis
    const uint32_t ob = oa ^ (1u << d);
    uint32_t q = 0;
#pragma unroll
    for (uint32_t ax = 0; ax < 3; ++ax) {
        const uint32_t a = (oa >> ax) & 1u, b = (ob >> ax) & 1u, v = (cc >> (2u * ax)) & 3u;
        const float p = __fadd_rn(__fadd_rn(__fadd_rn((float)a, __fmul_rn(tt, (float)((int)b - (int)a))), (float)v), 0.5f);
        q |= quantize(p) << (20u - 10u * ax);
    }
    return q;
}

}  // namespace bcmc
