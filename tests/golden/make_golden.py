"""Generates the golden fixtures in this folder from the reference's own compute
shaders, compiled as host C++ (oracle/_ref, built by oracle/ref_build.py from
a checkout of Twinklebear/webgpu-bcmc).

Inputs are seeded synthetic fields (bcmc.datasets) encoded with the oracle's
fixed-rate ZFP encoder (the reference has no encoder: its streams come from
zfp), plus random bit streams for the decoder.  Outputs are what the
reference's shaders produce for them:

  mc_<case>.npz      words, rate, dims, isos; block ranges; per iso: active
                     flags, active ids, blocks with vertices, vertex offsets,
                     the packed vertex buffer
  decode_rate<r>.npz random words and the reference decoder's output, bits
  unpack_ct44.npz    the vertex stage's world and clip positions of a mesh, bits
  sort.npz           RadixSorter.sort results (values, ascending and descending)
  render_ct44.npz    the render shaders on the ct44 mesh: the fog vertex
                     stage's t_enter per vertex, and the fragment shader's
                     colour (with and without fog) at sampled fragments

Run from the repository root:  python tests/golden/make_golden.py [name ...]
(names: mc decode unpack sort render; default all)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "webgpu-bcmc_gb300")]

import oracle as O  # noqa: E402
import ref as R  # noqa: E402
from bcmc import datasets as D  # noqa: E402

MC_CASES = {
    # name: (field kind, dims (x, y, z), seed, rate, isovalues)
    "blobs32_r8": ("blobs", (32, 32, 32), 1, 8, [0.5, 0.3]),
    "blobs_partial_r4": ("blobs", (30, 21, 17), 4, 4, [0.6, 1.5]),
    "ct44_r4": ("ct_like", (44, 40, 36), 2, 4, [60.0, 150.0]),
    "turb24_r2": ("turbulence", (24, 24, 24), 3, 2, [0.0, 0.3]),
    "ct16bit_r4": ("ct_uint16", (36, 32, 28), 5, 4, [800.0, 2500.0]),
}
DECODE_RATES = (1, 2, 3, 8, 16, 32)
DECODE_BLOCKS = 96


def make_mc(name, kind, dims, seed, rate, isos):
    f = D.make_field(kind, dims, seed)
    words = O.zfp_encode(f, rate)
    ranges = R.block_ranges(words, rate, dims)
    out = {"words": words, "rate": np.int32(rate), "dims": np.asarray(dims, np.uint32),
           "isos": np.asarray(isos, np.float32), "ranges": ranges}
    for i, iso in enumerate(isos):
        s = R.surface(words, rate, dims, float(iso))
        assert np.array_equal(s["ranges"].view(np.uint32), ranges.view(np.uint32))
        out[f"active_{i}"] = s["active"]
        out[f"active_ids_{i}"] = s["active_ids"]
        out[f"with_verts_{i}"] = s["with_verts"]
        out[f"vert_offsets_{i}"] = s["vert_offsets"]
        out[f"vertices_{i}"] = s["vertices"]
        print(f"{name} iso {iso}: {len(s['active_ids'])} active, {len(s['with_verts'])} with vertices, "
              f"{s['num_vertices']} vertices")
    np.savez_compressed(os.path.join(HERE, f"mc_{name}.npz"), **out)


def make_decode(rate):
    rng = np.random.default_rng(1000 + rate)
    nwords = DECODE_BLOCKS * rate + 2
    words = rng.integers(0, 1 << 63, size=nwords, dtype=np.int64).view(np.uint64)
    words[0] |= np.uint64(1)  # first block nonzero
    words[-2:] = 0
    ids = np.arange(DECODE_BLOCKS, dtype=np.uint32)
    dec = R.decode_blocks(words, rate, ids, ids.astype(np.int32), DECODE_BLOCKS)
    np.savez_compressed(os.path.join(HERE, f"decode_rate{rate}.npz"), words=words, rate=np.int32(rate),
                        decoded_bits=dec.view(np.uint32))


UNPACK_PROJ = (np.arange(16, dtype=np.float32).reshape(4, 4) * np.float32(0.37) - np.float32(1.1))


def make_unpack():
    """mc_isosurface.vert's position math on the ct44 mesh (scale != 1, a
    view-projection matrix)."""
    g = np.load(os.path.join(HERE, "mc_ct44_r4.npz"))
    verts = g["vertices_0"]
    dims = tuple(int(d) for d in g["dims"])
    scale = (1.0, 0.5, 2.0)
    world, clip = R.unpack_vertices(verts, dims, scale, UNPACK_PROJ)
    np.savez_compressed(os.path.join(HERE, "unpack_ct44.npz"), dims=np.asarray(dims, np.uint32),
                        scale=np.asarray(scale, np.float32), proj=UNPACK_PROJ, vertices=verts,
                        world_bits=world.view(np.uint32), clip_bits=clip.view(np.uint32))


SORT_CASES = [(65, 5), (100, 3), (1000, 50), (4097, 7), (20000, 1000), (3000, 1 << 31)]


def make_sort():
    """RadixSorter.sort over the reference's chunk-sort, merge and reverse
    shaders (n > 64: below that the reference's reverse pass races)."""
    out = {}
    for i, (n, kmax) in enumerate(SORT_CASES):
        rng = np.random.default_rng(500 + i)
        keys = rng.integers(0, kmax, size=n, dtype=np.uint64).astype(np.uint32)
        vals = rng.permutation(n).astype(np.uint32)
        out[f"keys_{i}"] = keys
        out[f"values_{i}"] = vals
        out[f"asc_{i}"] = R.sort_by_key(keys, vals, False)
        out[f"desc_{i}"] = R.sort_by_key(keys, vals, True)
    np.savez_compressed(os.path.join(HERE, "sort.npz"), cases=np.int32(len(SORT_CASES)), **out)


RENDER_SCALE = (1.0, 0.9, 0.8)
RENDER_EYE = (0.3, 0.4, 1.2)
RENDER_FRAGMENTS = 400


def make_render():
    """mc_isosurface.vert (DRAW_FOG) per vertex of the ct44 mesh, and
    mc_isosurface.frag at fragments inside its triangles (random barycentric
    points; t_enter interpolated the same way; the world-position derivatives
    are the triangle's edges, which span its plane as the screen derivatives
    do)."""
    g = np.load(os.path.join(HERE, "mc_ct44_r4.npz"))
    verts = g["vertices_0"]
    dims = tuple(int(d) for d in g["dims"])
    world, te = R.vert_fog(verts, dims, RENDER_SCALE, RENDER_EYE)
    rng = np.random.default_rng(77)
    tri = rng.integers(0, len(verts) // 3, RENDER_FRAGMENTS)
    bary = rng.dirichlet((1.0, 1.0, 1.0), RENDER_FRAGMENTS).astype(np.float32)
    tw = world.reshape(-1, 3, 3)[tri]
    wp = (bary[:, :, None] * tw).sum(1).astype(np.float32)
    fte = (bary * te.reshape(-1, 3)[tri]).sum(1).astype(np.float32)
    dx, dy = tw[:, 1] - tw[:, 0], tw[:, 2] - tw[:, 0]
    rgba = R.frag(wp, fte, RENDER_EYE, dx, dy, False)
    rgba_fog = R.frag(wp, fte, RENDER_EYE, dx, dy, True)
    np.savez_compressed(os.path.join(HERE, "render_ct44.npz"), dims=np.asarray(dims, np.uint32),
                        scale=np.asarray(RENDER_SCALE, np.float32), eye=np.asarray(RENDER_EYE, np.float32),
                        t_enter_bits=te.view(np.uint32), frag_tri=tri.astype(np.uint32), frag_world=wp,
                        frag_t_enter=fte, frag_rgba_bits=rgba.view(np.uint32),
                        frag_rgba_fog_bits=rgba_fog.view(np.uint32))


def main(names=None):
    O.build()
    if not R.available():
        sys.exit("oracle/_ref is not built (no reference checkout): cannot generate fixtures")
    names = set(names or ["mc", "decode", "unpack", "sort", "render"])
    if "mc" in names:
        for name, spec in MC_CASES.items():
            make_mc(name, *spec)
    if "decode" in names:
        for rate in DECODE_RATES:
            make_decode(rate)
    if "unpack" in names:
        make_unpack()
    if "sort" in names:
        make_sort()
    if "render" in names:
        make_render()


if __name__ == "__main__":
    main(sys.argv[1:])
