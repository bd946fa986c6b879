// The marching-cubes vertex code of the MC kernels (mc_vertex.cuh: the emit
// table, the corner pack table and mc_vertex) built as host code, one vertex
// at a time, for the CPU test against a restatement of the oracle's emit.
#include "cuda_host_shim.h"
#include "mc_vertex.cuh"

namespace {
const bcmc::mc_detail::TriEdges kEdges = bcmc::mc_detail::make_tri_edges();
const bcmc::mc_detail::CornerPack kPack = bcmc::mc_detail::make_corner_pack();
const bcmc::mc_detail::TriCorners kTri = bcmc::mc_detail::make_tri_corners();
}  // namespace

extern "C" uint32_t mc_case_count(uint32_t c) { return kTri.count[c & 255u]; }

// Vertex k of case c in cell cc (x + 4y + 16z) of a block, the cell's 8
// corner values given in the reference's corner order; the rest of the 5^3
// grid is NaN, so a read outside the cell would show.
extern "C" uint32_t mc_vertex_host(uint32_t c, uint32_t k, uint32_t cc, const float* corners, float iso)
{
    float vol[128];
    for (float& v : vol) v = NAN;
    const uint32_t x = cc & 3u, y = (cc >> 2) & 3u, z = cc >> 4;
    for (int i = 0; i < 8; ++i) {
        const uint32_t o = bcmc::mc_detail::kCorner[i];
        vol[(x + (o & 1u)) + 5u * ((y + ((o >> 1) & 1u)) + 5u * (z + (o >> 2)))] = corners[i];
    }
    return bcmc::mc_vertex(kEdges.e[c & 255u][k & 15u], cc & 63u, vol, &kPack.p[0][0], iso);
}
