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
  scan_compact.npz   ExclusiveScanner.scan and StreamCompact.compactActiveIDs
                     over the scan and compaction shaders: inputs, totals, and
                     the outputs (in full when small, else their SHA-256)
  lru_seq.npz        LRUCache.update sequences over the LRU, scan, compaction
                     and sort shaders (growth, resets, empty updates): per
                     update the needed items, the new item ids, the cache
                     size, the slot arrays and cachedItemSlots (their SHA-256
                     for the 70000-item sequence)
  lru_pipeline.npz   computeSurface sequences with the LRU in the loop, on the
                     mc_* volumes: per query the counts, the mesh's SHA-256
                     and the LRU state

Run from the repository root:  python tests/golden/make_golden.py [name ...]
(names: mc decode unpack sort render scan lru; default all)
"""
from __future__ import annotations

import hashlib
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


# (n, kind, seed): "flags" are 0/1 at a density drawn per case, "counts" 0..15
SCAN_CASES = [(1, "flags", 1), (7, "flags", 2), (511, "counts", 3), (512, "flags", 4), (513, "flags", 5),
              (5000, "counts", 6), (262144, "flags", 7), (262145, "flags", 8), (700001, "flags", 9),
              (100000, "counts", 10)]
FULL_OUTPUT_MAX = 6000


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()


def make_scan():
    """ExclusiveScanner.scan (js/exclusive_scan.js:178-295) of each input as
    prepareInput uploads it (zero-padded to 512), then compactActiveIDs
    (js/stream_compact.js:56-165) of its nonzero elements."""
    out = {"cases": np.int32(len(SCAN_CASES))}
    for i, (n, kind, seed) in enumerate(SCAN_CASES):
        rng = np.random.default_rng(900 + seed)
        if kind == "flags":
            v = (rng.random(n) < rng.uniform(0.05, 0.9)).astype(np.uint8)
            out[f"in_{i}"] = np.packbits(v)
        else:
            v = rng.integers(0, 16, n).astype(np.uint8)
            out[f"in_{i}"] = v
        out[f"n_{i}"] = np.int64(n)
        out[f"kind_{i}"] = np.array(kind)
        buf = np.zeros(R._align(n, 512), np.uint32)
        buf[:n] = v
        total = R.ExclusiveScanner(buf, len(buf)).scan(n)
        flags = np.zeros(len(buf), np.uint32)
        flags[:n] = v != 0
        offs = np.zeros(len(buf), np.uint32)
        offs[:n] = flags[:n]
        m = R.ExclusiveScanner(offs, len(offs)).scan(n)
        ids = np.zeros(max(m, 1), np.uint32)
        R.compact_active_ids(n, flags, offs, ids)
        ids = ids[:m]
        out[f"total_{i}"] = np.int64(total)
        out[f"compact_count_{i}"] = np.int64(m)
        out[f"scan_sha_{i}"] = np.array(sha(buf[:n]))
        out[f"compact_sha_{i}"] = np.array(sha(ids))
        if n <= FULL_OUTPUT_MAX:
            out[f"scan_{i}"] = buf[:n].copy()
            out[f"compact_{i}"] = ids
        print(f"scan n={n} {kind}: total {total}, {m} compacted")
    np.savez_compressed(os.path.join(HERE, "scan_compact.npz"), **out)


# (total items, initial size, updates, seed, update before which the cache is reset)
LRU_SEQS = [(300, 20, 40, 1, 37), (5000, 64, 18, 2, 15), (70000, 3500, 8, 3, 6)]
LRU_FULL_STATE_MAX = 10000  # larger sequences keep the SHA-256 of each state array


def lru_needed(rng, total, step):
    """Spatially coherent runs of needed items, as active blocks are; every
    7th update (from the 4th) needs nothing."""
    p = rng.uniform(0.01, 0.4)
    needed = (np.convolve(rng.random(total) < p / 8, np.ones(8), mode="same") > 0).astype(np.uint32)
    if step % 7 == 3:
        needed[:] = 0
    return needed


def make_lru():
    """LRUCache.update sequences (js/lru_cache.js:312-843) and computeSurface
    sequences with the cache in the loop (js/compressed_marching_cubes.js:580-809)."""
    out = {"seqs": np.int32(len(LRU_SEQS))}
    for s, (total, initial, steps, seed, reset_at) in enumerate(LRU_SEQS):
        rng = np.random.default_rng(seed)
        c = R.LRUCache(initial, total)
        out[f"s{s}_spec"] = np.array([total, initial, steps, reset_at], np.int64)
        for step in range(steps):
            if step == reset_at:
                c.reset()
            needed = lru_needed(rng, total, step)
            ids = c.update(needed)
            st = c.state()
            p = f"s{s}_{step}_"
            out[p + "needed"] = np.packbits(needed.astype(np.uint8))
            out[p + "new"] = ids
            out[p + "display"] = np.int64(c.display_num_slots_available if len(ids) else -1)
            out[p + "cache_size"] = np.int64(c.cache_size)
            for k in ("item_slots", "age", "avail", "item"):
                if total <= LRU_FULL_STATE_MAX:
                    out[p + k] = st[k]
                else:
                    out[p + k + "_sha"] = np.array(sha(st[k].view(np.uint32)))
        print(f"lru seq {s}: total {total}, final cache size {c.cache_size}")
    np.savez_compressed(os.path.join(HERE, "lru_seq.npz"), **out)

    pipe = {"cases": np.int32(len(LRU_PIPE_CASES))}
    for ci, (name, frac, isos, reset_at) in enumerate(LRU_PIPE_CASES):
        g = np.load(os.path.join(HERE, f"mc_{name}.npz"))
        rate, dims = int(g["rate"]), tuple(int(d) for d in g["dims"])
        m = R.CompressedMarchingCubes(g["words"], rate, dims, frac)
        p = f"c{ci}_"
        pipe[p + "name"] = np.array(name)
        pipe[p + "frac"] = np.float64(frac)
        pipe[p + "isos"] = np.asarray(isos, np.float32)
        pipe[p + "reset_at"] = np.int64(reset_at)
        for qi, iso in enumerate(np.asarray(isos, np.float32)):
            if qi == reset_at:
                m.cache_reset()
            n = m.compute_surface(float(iso))
            q = f"{p}{qi}_"
            last = m.last
            pipe[q + "counts"] = np.array([n, last["numActiveBlocks"], last["newDecompressed"],
                                          last["numBlocksWithVertices"]], np.int64)
            pipe[q + "mesh_sha"] = np.array(sha(last["vertices"].reshape(-1)))
            st = m.lru.state()
            for k in ("item_slots", "age", "avail", "item"):
                pipe[q + k] = st[k]
        print(f"lru pipeline {name}: cache size {m.lru.cache_size}")
    np.savez_compressed(os.path.join(HERE, "lru_pipeline.npz"), **pipe)


def _walk(lo, hi, n, seed):
    rng = np.random.default_rng(seed)
    x = [rng.uniform(lo, hi)]
    for _ in range(n - 1):
        x.append(float(np.clip(x[-1] + rng.normal(0, 0.12 * (hi - lo)), lo, hi)))
    return x


# (mc fixture, initial cache fraction, isovalues, query before which the cache is reset)
LRU_PIPE_CASES = [
    ("ct44_r4", 0.05, _walk(20.0, 240.0, 12, 21) + [1000.0] + _walk(20.0, 240.0, 5, 22), 14),
    ("turb24_r2", 0.25, _walk(-0.8, 0.8, 14, 23), 9),
    ("blobs_partial_r4", 0.05, _walk(0.05, 1.9, 10, 24), 6),
]


def main(names=None):
    O.build()
    if not R.available():
        sys.exit("oracle/_ref is not built (no reference checkout): cannot generate fixtures")
    names = set(names or ["mc", "decode", "unpack", "sort", "render", "scan", "lru"])
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
    if "scan" in names:
        make_scan()
    if "lru" in names:
        make_lru()


if __name__ == "__main__":
    main(sys.argv[1:])
