"""ctypes front end of oracle/_ref/libbcmc_ref.so: the reference's own compute
shaders compiled as host C++ by oracle/ref_build.py (TEST INFRASTRUCTURE ONLY).

`available()` is False when the reference checkout is absent (for example on a
machine that only has this repository); callers then fall back to the golden
fixtures under tests/golden/, which were generated from this module.

`surface(words, rate, dims, iso)` composes the shader programs the way
js/compressed_marching_cubes.js does for one query with every active block
cached (computeBlockRanges :522-578, computeActiveBlocks :811-829, stream
compaction, decompressBlocks :831-913, computeBlockHasVertices :915-991,
computeBlockVertexCounts :993-1042, computeVertices :1044-1122).  The host
steps between dispatches (compaction to ascending ids, exclusive scan of the
per-block counts) are restated in numpy.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

P = C.c_void_p
U32 = C.c_uint32
F32 = C.c_float
_SIGS = {
    "ref_zfp_decompress_blocks": [P, U32, P, U32, P, P],
    "ref_zfp_block_ranges": [P, P, U32, P],
    "ref_block_active": [P, P, F32, P],
    "ref_block_has_vertices": [P, F32, P, P, P, P, U32, P],
    "ref_block_num_verts": [P, F32, P, P, P, P, P, U32, P],
    "ref_block_vertices": [P, F32, P, P, P, P, P, U32, P],
    "ref_unpack_vertices": [P, C.c_uint64, P, P, P, P, P],
    "ref_vert_fog": [P, C.c_uint64, P, P, P, P, P],
    "ref_frag": [P, P, P, P, P, C.c_uint64, P],
    "ref_frag_fog": [P, P, P, P, P, C.c_uint64, P],
    "ref_radix_sort_chunk": [P, P, U32, U32],
    "ref_merge_sorted_chunks": [P, P, P, P, U32, U32],
    "ref_reverse_buffer": [P, U32, U32],
}


def build(reference: str | None = None):
    import ref_build

    return ref_build.build(reference)


def available() -> bool:
    try:
        return load() is not None
    except OSError:
        return False


def load():
    global _LIB
    if _LIB is None:
        path = build()
        if path is None:
            return None
        lib = C.CDLL(path)
        for name, args in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = None
        _LIB = lib
    return _LIB


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _dims(dims):
    return np.ascontiguousarray(np.asarray(dims, dtype=np.uint32))


def _words(words: np.ndarray) -> np.ndarray:
    w = np.ascontiguousarray(words).view(np.uint64)
    return np.concatenate([w, np.zeros(2, np.uint64)])  # the reader may fetch one word past the end


def block_ranges(words, rate: int, dims) -> np.ndarray:
    d = _dims(dims)
    nb = int(np.prod([(int(x) + 3) // 4 for x in dims]))
    out = np.zeros((nb, 2), np.float32)
    w = _words(words)
    load().ref_zfp_block_ranges(_p(w), _p(d), 64 * rate, _p(out))
    return out


def decode_blocks(words, rate: int, ids: np.ndarray, slots: np.ndarray, cache_slots: int) -> np.ndarray:
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    slots = np.ascontiguousarray(slots).astype(np.int32).view(np.uint32)
    cache = np.zeros((cache_slots, 64), np.float32)
    w = _words(words)
    load().ref_zfp_decompress_blocks(_p(w), 64 * rate, _p(ids), len(ids), _p(slots), _p(cache))
    return cache


def block_active(ranges: np.ndarray, dims, iso: float) -> np.ndarray:
    d = _dims(dims)
    r = np.ascontiguousarray(ranges, dtype=np.float32)
    out = np.zeros(len(r), np.uint32)
    load().ref_block_active(_p(r), _p(d), F32(iso), _p(out))
    return out


def surface(words, rate: int, dims, iso: float) -> dict:
    """One query with every active block cached (slot = rank among active blocks)."""
    L = load()
    d = _dims(dims)
    ranges = block_ranges(words, rate, dims)
    active = block_active(ranges, dims, iso)
    ids = np.nonzero(active)[0].astype(np.uint32)
    n = len(ids)
    total = len(active)
    slots = np.full(total, -1, np.int32)
    slots[ids] = np.arange(n, dtype=np.int32)
    cache = decode_blocks(words, rate, ids, slots, max(n, 1))
    uslots = slots.view(np.uint32)
    has = np.zeros(max(n, 1), np.uint32)
    if n:
        L.ref_block_has_vertices(_p(d), F32(iso), _p(cache), _p(active), _p(uslots), _p(ids), n, _p(has))
    with_verts = np.nonzero(has[:n])[0].astype(np.uint32)
    m = len(with_verts)
    counts = np.zeros(max(m, 1), np.uint32)
    if m:
        L.ref_block_num_verts(_p(d), F32(iso), _p(cache), _p(active), _p(uslots), _p(ids), _p(with_verts), m,
                              _p(counts))
    counts = counts[:m]
    offsets = (np.cumsum(counts.astype(np.uint64)) - counts).astype(np.uint32)
    nverts = int(counts.astype(np.uint64).sum())
    verts = np.zeros((max(nverts, 1), 2), np.uint32)
    if m:
        info = np.ascontiguousarray(np.stack([with_verts, offsets], axis=1).astype(np.uint32))
        L.ref_block_vertices(_p(d), F32(iso), _p(cache), _p(active), _p(uslots), _p(ids), _p(info), m, _p(verts))
    return {"ranges": ranges, "active": active, "active_ids": ids, "with_verts": with_verts,
            "block_counts": counts, "vert_offsets": offsets, "num_vertices": nverts, "vertices": verts[:nverts],
            "decoded": cache[:n]}


def unpack_vertices(verts: np.ndarray, dims, scale=(1.0, 1.0, 1.0), proj_view=None):
    """mc_isosurface.vert's position math per vertex: world [n, 3] (and clip [n, 4])."""
    v = np.ascontiguousarray(verts, dtype=np.uint32).reshape(-1, 2)
    n = len(v)
    world = np.zeros((n, 3), np.float32)
    sc = np.ascontiguousarray(np.asarray(scale, np.float32))
    clip = np.zeros((n, 4), np.float32) if proj_view is not None else None
    pv = np.ascontiguousarray(np.asarray(proj_view, np.float32).reshape(16)) if proj_view is not None else None
    load().ref_unpack_vertices(_p(v), n, _p(_dims(dims)), _p(sc), _p(pv) if pv is not None else None, _p(world),
                               _p(clip) if clip is not None else None)
    return (world, clip) if clip is not None else world


def vert_fog(verts: np.ndarray, dims, scale, eye):
    """mc_isosurface.vert with DRAW_FOG per vertex: (world [n, 3], t_enter [n])."""
    v = np.ascontiguousarray(verts, dtype=np.uint32).reshape(-1, 2)
    n = len(v)
    world = np.zeros((n, 3), np.float32)
    te = np.zeros(n, np.float32)
    sc = np.ascontiguousarray(np.asarray(scale, np.float32))
    e = np.ascontiguousarray(np.asarray(eye, np.float32))
    load().ref_vert_fog(_p(v), n, _p(_dims(dims)), _p(sc), _p(e), _p(world), _p(te))
    return world, te


def frag(world_pos, t_enter, eye, dfdx, dfdy, fog: bool) -> np.ndarray:
    """mc_isosurface.frag per fragment (with DRAW_FOG when `fog`): rgba [n, 4]."""
    wp = np.ascontiguousarray(world_pos, dtype=np.float32).reshape(-1, 3)
    n = len(wp)
    te = np.ascontiguousarray(np.asarray(t_enter, np.float32).reshape(n))
    e = np.ascontiguousarray(np.asarray(eye, np.float32))
    dx = np.ascontiguousarray(dfdx, dtype=np.float32).reshape(n, 3)
    dy = np.ascontiguousarray(dfdy, dtype=np.float32).reshape(n, 3)
    out = np.zeros((n, 4), np.float32)
    (load().ref_frag_fog if fog else load().ref_frag)(_p(wp), _p(te), _p(e), _p(dx), _p(dy), n, _p(out))
    return out


def _next_pow2(a: int) -> int:
    a -= 1
    for sh in (1, 2, 4, 8, 16):
        a |= a >> sh
    return a + 1


def sort_by_key(keys: np.ndarray, values: np.ndarray, reverse: bool) -> np.ndarray:
    """RadixSorter.sort (js/radix_sort_by_key.js:161-400) over the reference's
    shaders: chunk sort, log2(chunks) merges ping-ponging between the buffers
    and scratch, the reverse pass when `reverse`, and the readback of `size`
    values from offset alignedSize - size (reverse) or 0.  Returns the sorted
    values.  For n <= 64 the reverse pass races in the reference (64 threads
    each swapping a pair both ways); the fibers here run it sequentially."""
    L = load()
    n = len(keys)
    chunks = _next_pow2(-(-n // 64))
    aligned = chunks * 64
    steps = chunks.bit_length() - 1
    buf_k = np.zeros(aligned, np.uint32)
    buf_v = np.zeros(aligned, np.uint32)
    buf_k[:n] = keys
    buf_v[:n] = values
    scr_k = np.zeros(aligned, np.uint32)
    scr_v = np.zeros(aligned, np.uint32)
    L.ref_radix_sort_chunk(_p(buf_k), _p(buf_v), n, chunks)
    for i in range(steps):
        groups = chunks // (2 << i)
        src, dst = ((buf_k, buf_v), (scr_k, scr_v)) if i % 2 == 0 else ((scr_k, scr_v), (buf_k, buf_v))
        L.ref_merge_sorted_chunks(_p(src[0]), _p(src[1]), _p(dst[0]), _p(dst[1]), n, groups)
    vals = buf_v if steps % 2 == 0 else scr_v
    if reverse:
        L.ref_reverse_buffer(_p(vals), n, -(-chunks // 2))
    off = aligned - n if reverse else 0
    return vals[off: off + n].copy()
