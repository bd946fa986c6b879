// mc_common.cuh -- tables and helpers of the marching-cubes kernels, shared
// by the per-query MC kernel (pipeline.cu) and the batched one (engine.cu):
// the case tables of mc_vertex.cuh in device memory, the ghost-voxel table and
// the grid helpers.  The tables are static: each translation unit has its own
// copy.
#pragma once

#include "bcmc_internal.cuh"
#include "mc_vertex.cuh"

namespace bcmc {

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

}  // namespace bcmc
