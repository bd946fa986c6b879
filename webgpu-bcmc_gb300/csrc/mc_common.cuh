// mc_common.cuh -- tables and helpers of the marching-cubes kernels, shared
// by the per-query MC kernel (pipeline.cu) and the batched one (engine.cu).
// The __constant__ tables are static: each translation unit has its own copy.
#pragma once

#include "bcmc_internal.cuh"

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

static __constant__ __align__(16) mc_detail::TriCorners c_tri = mc_detail::make_tri_corners();
// in global memory: the kernels copy them into shared memory with coalesced
// 16-byte loads at launch (each thread a different address, which the
// constant cache would serialise)
static __device__ const __align__(16) mc_detail::TriEdges c_tri_edges = mc_detail::make_tri_edges();
static __device__ const __align__(16) mc_detail::CornerPack c_corner_pack = mc_detail::make_corner_pack();

// Ghost voxels of a block's 5^3 grid (some coordinate == 4): x|y<<4|z<<8 and,
// in bits 12-14, which +x/+y/+z neighbour holds them (kNb* order below).
static __constant__ uint16_t c_ghost[61] = {
#define G(x, y, z, k) (uint16_t)((x) | ((y) << 4) | ((z) << 8) | ((k) << 12))
    G(4, 0, 0, 0), G(4, 1, 0, 0), G(4, 2, 0, 0), G(4, 3, 0, 0), G(0, 4, 0, 1), G(1, 4, 0, 1), G(2, 4, 0, 1),
    G(3, 4, 0, 1), G(4, 4, 0, 3), G(4, 0, 1, 0), G(4, 1, 1, 0), G(4, 2, 1, 0), G(4, 3, 1, 0), G(0, 4, 1, 1),
    G(1, 4, 1, 1), G(2, 4, 1, 1), G(3, 4, 1, 1), G(4, 4, 1, 3), G(4, 0, 2, 0), G(4, 1, 2, 0), G(4, 2, 2, 0),
    G(4, 3, 2, 0), G(0, 4, 2, 1), G(1, 4, 2, 1), G(2, 4, 2, 1), G(3, 4, 2, 1), G(4, 4, 2, 3), G(4, 0, 3, 0),
    G(4, 1, 3, 0), G(4, 2, 3, 0), G(4, 3, 3, 0), G(0, 4, 3, 1), G(1, 4, 3, 1), G(2, 4, 3, 1), G(3, 4, 3, 1),
    G(4, 4, 3, 3), G(0, 0, 4, 2), G(1, 0, 4, 2), G(2, 0, 4, 2), G(3, 0, 4, 2), G(4, 0, 4, 4), G(0, 1, 4, 2),
    G(1, 1, 4, 2), G(2, 1, 4, 2), G(3, 1, 4, 2), G(4, 1, 4, 4), G(0, 2, 4, 2), G(1, 2, 4, 2), G(2, 2, 4, 2),
    G(3, 2, 4, 2), G(4, 2, 4, 4), G(0, 3, 4, 2), G(1, 3, 4, 2), G(2, 3, 4, 2), G(3, 3, 4, 2), G(4, 3, 4, 4),
    G(0, 4, 4, 5), G(1, 4, 4, 5), G(2, 4, 4, 5), G(3, 4, 4, 5), G(4, 4, 4, 6)
#undef G
};
// neighbour k of a block: +x, +y, +z, +xy, +xz, +yz, +xyz (packed x|y<<1|z<<2)
static __constant__ uint8_t c_nb_off[7] = {1, 2, 4, 3, 5, 6, 7};
enum { kNbX = 0, kNbY, kNbZ, kNbXY, kNbXZ, kNbYZ, kNbXYZ, kNbSelf };

// Ghost voxel c_ghost[gi] decoded for the loads: bits 0-2 the axes on which
// it lies in a neighbour (its coordinate 4 there), bits 3-8 its voxel in that
// neighbour's block, bits 9-15 its index in the 5^3 grid, bits 16+ which
// neighbour (kNb*).  MC kernels decode the table once per CTA.
__device__ __forceinline__ uint32_t ghost_desc(uint32_t g)
{
    const uint32_t gx = g & 15u, gy = (g >> 4) & 15u, gz = (g >> 8) & 15u;
    const uint32_t need = (gx == 4u ? 1u : 0u) | (gy == 4u ? 2u : 0u) | (gz == 4u ? 4u : 0u);
    const uint32_t src = (gx & 3u) + 4u * ((gy & 3u) + 4u * (gz & 3u));
    return need | (src << 3) | ((gx + 5u * (gy + 5u * gz)) << 9) | ((g >> 12) << 16);
}

// The axes on which a grid of `dims` (block_dims_with_ghost) takes the
// neighbour's layer: ghost voxel d is in the grid when (d & 7 & ~axes) == 0.
__device__ __forceinline__ uint32_t ghost_axes(uint32_t dims)
{
    return ((dims & 15u) == 5u ? 1u : 0u) | (((dims >> 4) & 15u) == 5u ? 2u : 0u) | ((dims >> 8) == 5u ? 4u : 0u);
}

// compute_vertex_values.comp:96-156: grid extent of the block plus the ghost
// layer taken from active +x/+y/+z neighbours, tested corner, edges, faces.
// `act` has bit k set when neighbour k exists and is active.
__device__ __forceinline__ uint32_t block_dims_with_ghost(uint32_t act, bool hx, bool hy, bool hz)
{
    uint32_t dx = hx ? 5 : 4, dy = hy ? 5 : 4, dz = hz ? 5 : 4;
    if (dx == 5 && dy == 5 && dz == 5 && !(act >> kNbXYZ & 1u)) dx = dy = dz = 4;
    if (dx == 5 && dy == 5 && !(act >> kNbXY & 1u)) dx = dy = 4;
    if (dx == 5 && dz == 5 && !(act >> kNbXZ & 1u)) dx = dz = 4;
    if (dy == 5 && dz == 5 && !(act >> kNbYZ & 1u)) dy = dz = 4;
    if (dx == 5 && !(act >> kNbX & 1u)) dx = 4;
    if (dy == 5 && !(act >> kNbY & 1u)) dy = 4;
    if (dz == 5 && !(act >> kNbZ & 1u)) dz = 4;
    return dx | (dy << 4) | (dz << 8);
}

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
