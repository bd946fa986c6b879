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
    "ref_lru_age_slots": [P, U32, U32, U32, U32],
    "ref_lru_mark_new_items": [P, P, P, P, U32, U32, U32],
    "ref_lru_extract_slot_available": [P, P, U32, U32, U32, U32],
    "ref_lru_init": [P, U32, U32, U32, U32, U32],
    "ref_lru_copy_available_slot_age": [P, P, P, U32, U32, U32, U32],
    "ref_lru_update": [P, P, P, P, U32, U32, U32, U32],
    "ref_prefix_sum": [P, P, U32],
    "ref_block_prefix_sum": [P, P],
    "ref_add_block_sums": [P, P, U32],
    "ref_stream_compact": [P, P, U32, P, U32],
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


# ---------------------------------------------------------------------------
# The reference's GPU primitives and LRU cache, driven as its JavaScript does.
# Buffers are numpy arrays; WebGPU zero-initialises every new buffer, and so do
# these.  A binding at a byte offset is a pointer into the array.

SCAN_BLOCK = 512  # ScanBlockSize (shaders/embed_shaders.py:30, BLOCK_SIZE)
MAX_WORKGROUPS = 65535  # device.limits.maxComputeWorkgroupsPerDimension
COMPACT_CHUNK = 65280  # StreamCompact.maxDispatchSize (js/stream_compact.js:11)


def _align(v: int, a: int) -> int:
    return (v + a - 1) // a * a


def _ptr(a: np.ndarray, elem_offset: int = 0):
    return C.c_void_p(a.ctypes.data + elem_offset * a.itemsize)


def push_constant_chunks(total_wg: int):
    """buildPushConstantsBuffer (js/util.js:10-66): per dispatch chunk the
    workgroup id offset, the total and the chunk's workgroup count.  The last
    chunk's count is `total % 65535`, which is 0 when the total is a multiple
    of 65535 (the dispatch then does nothing)."""
    n = -(-total_wg // MAX_WORKGROUPS)
    return [(MAX_WORKGROUPS * i, total_wg, MAX_WORKGROUPS if i + 1 < n else total_wg % MAX_WORKGROUPS)
            for i in range(n)]


class ExclusiveScanner:
    """ExclusiveScanPipeline.prepareGPUInput + ExclusiveScanner
    (js/exclusive_scan.js:116-295) over a caller-owned u32 buffer of
    `aligned_size` elements, scanned in place."""

    def __init__(self, buf: np.ndarray, aligned_size: int):
        assert aligned_size % SCAN_BLOCK == 0 and len(buf) >= aligned_size
        self.buf = buf
        self.input_size = aligned_size
        self.block_sums = np.zeros(SCAN_BLOCK, np.uint32)
        self.carry = np.zeros(2, np.uint32)

    def scan(self, data_size: int) -> int:
        L = load()
        max_scan = SCAN_BLOCK * SCAN_BLOCK
        chunks = -(-data_size // max_scan)
        if data_size < self.input_size:  # the element holding the total starts at 0
            self.buf[data_size] = 0
        self.carry[:] = 0
        for i in range(chunks):
            groups = min((self.input_size - i * max_scan) // SCAN_BLOCK, SCAN_BLOCK)
            self.block_sums[:] = 0
            L.ref_prefix_sum(_ptr(self.buf, i * max_scan), _ptr(self.block_sums), groups)
            L.ref_block_prefix_sum(_ptr(self.block_sums), _ptr(self.carry))
            L.ref_add_block_sums(_ptr(self.buf, i * max_scan), _ptr(self.block_sums), groups)
            self.carry[0] = self.carry[1]
        return int(self.buf[data_size] if data_size < self.input_size else self.carry[1])


def compact_active_ids(n: int, flags: np.ndarray, offsets: np.ndarray, out: np.ndarray):
    """StreamCompact.compactActiveIDs (js/stream_compact.js:56-165)."""
    L = load()
    for i in range(-(-n // COMPACT_CHUNK)):
        groups = min(n - i * COMPACT_CHUNK, COMPACT_CHUNK)
        base = i * COMPACT_CHUNK
        L.ref_stream_compact(_ptr(flags, base), _ptr(offsets, base), base, _ptr(out), groups)


def sort_aligned_size(n: int) -> int:
    """RadixSorter.getAlignedSize (js/radix_sort_by_key.js:155-158)."""
    return _next_pow2(-(-n // 64)) * 64


def sort_in_place(keys: np.ndarray, values: np.ndarray, n: int, reverse: bool):
    """RadixSorter.sort (js/radix_sort_by_key.js:161-400): the sorted values are
    copied to the start of `values`.  For n <= 64 the reference's reverse pass
    races (one 64-invocation workgroup swapping each pair from both ends); the
    intended full reversal is used there instead."""
    if n <= 64 and reverse:
        order = sorted(range(n), key=lambda i: (int(keys[i]), i))  # stable, as the chunk sort is
        values[:n] = values[:n][order][::-1].copy()
        return
    values[:n] = sort_by_key(keys[:n], values[:n], reverse)


class LRUCache:
    """LRUCache (js/lru_cache.js:4-903) over the reference's LRU, scan,
    compaction and sort shaders.  The slot data stay the reference's AoS
    `Slot {age, available, item_id}` array."""

    SLOT = np.dtype([("age", np.uint32), ("available", np.uint32), ("item_id", np.int32)])

    def __init__(self, initial_size: int, total_elements: int, element_size: int = 256):
        self.total = total_elements
        self.aligned_total = _align(total_elements, 32)
        self.cache_size = _align(initial_size, 32)
        self.element_size = element_size
        self.cached_item_slots = np.full(self.aligned_total, -1, np.int32)
        self.needs_caching = np.zeros(self.aligned_total, np.uint32)
        self.needs_caching_offsets = np.zeros(_align(self.aligned_total, SCAN_BLOCK), np.uint32)
        self.slot_data = np.zeros(self.cache_size, self.SLOT)
        self.slot_data["age"] = 2 + np.arange(self.cache_size, dtype=np.uint32)
        self.slot_data["available"] = 1
        self.slot_data["item_id"] = -1
        self.slot_available_offsets = np.zeros(_align(self.cache_size, SCAN_BLOCK), np.uint32)
        self.slot_available_for_compact = np.zeros(self.cache_size, np.uint32)
        self.slot_available_ids = np.zeros(self.cache_size, np.uint32)
        self.cache = np.zeros(self.cache_size * element_size // 4, np.float32)
        self.scan_needed = ExclusiveScanner(self.needs_caching_offsets, _align(total_elements, SCAN_BLOCK))
        self.slot_available_scanner = ExclusiveScanner(self.slot_available_offsets,
                                                       _align(self.cache_size, SCAN_BLOCK))
        self.display_num_slots_available = 0
        self.num_slots_available = 0

    def _extract_available(self, out: np.ndarray, size: int):
        for off, tot, groups in push_constant_chunks(size // 32):
            load().ref_lru_extract_slot_available(_ptr(self.slot_data), _ptr(out), off, tot, size, groups)

    def update(self, item_needed: np.ndarray):
        """LRUCache.update (js/lru_cache.js:312-843).  `item_needed` has one u32
        per item; the mark pass reads it up to the 32-aligned item count, so it
        is zero-padded to that.  Returns the new item ids (ascending)."""
        L = load()
        needed = np.zeros(self.aligned_total, np.uint32)
        needed[:self.total] = item_needed[:self.total]
        old_size = self.cache_size  # the cacheSizeBuf upload (:352-365)
        for off, tot, groups in push_constant_chunks(self.cache_size // 32):  # age (:374-395)
            L.ref_lru_age_slots(_ptr(self.slot_data), off, tot, self.cache_size, groups)
        for off, tot, groups in push_constant_chunks(self.aligned_total // 32):  # mark (:397-418)
            L.ref_lru_mark_new_items(_ptr(self.cached_item_slots), _ptr(self.slot_data), _ptr(needed),
                                     _ptr(self.needs_caching), off, tot, groups)
        self._extract_available(self.slot_available_offsets, self.cache_size)  # (:420-438)
        self.needs_caching_offsets[:self.total] = self.needs_caching[:self.total]  # (:441-442)
        num_new = self.scan_needed.scan(self.total)  # (:463)
        if num_new == 0:
            return np.zeros(0, np.uint32)
        new_ids = np.zeros(num_new, np.uint32)  # (:484-491)
        compact_active_ids(self.total, self.needs_caching, self.needs_caching_offsets, new_ids)
        num_avail = self.slot_available_scanner.scan(self.cache_size)  # (:501)
        if num_avail < num_new:  # grow (:510-672)
            new_size = min(self.cache_size + int(np.ceil((num_new - num_avail) * 1.5)), self.total)
            new_size = _align(new_size, 32)
            slot_data = np.zeros(new_size, self.SLOT)
            cache = np.zeros(new_size * self.element_size // 4, np.float32)
            self.slot_available_for_compact = np.zeros(new_size, np.uint32)
            self.slot_available_ids = np.zeros(new_size, np.uint32)
            for off, tot, groups in push_constant_chunks((new_size - self.cache_size) // 32):
                L.ref_lru_init(_ptr(slot_data), old_size, off, tot, new_size, groups)
            slot_data[:self.cache_size] = self.slot_data[:self.cache_size]
            cache[:len(self.cache)] = self.cache
            self.slot_data, self.cache = slot_data, cache
            self.slot_available_offsets = np.zeros(_align(new_size, SCAN_BLOCK), np.uint32)
            self._extract_available(self.slot_available_offsets, new_size)
            self.slot_available_scanner = ExclusiveScanner(self.slot_available_offsets,
                                                           _align(new_size, SCAN_BLOCK))
            num_avail = self.slot_available_scanner.scan(new_size)
            self.cache_size = new_size
        self.num_slots_available = num_avail
        self.display_num_slots_available = num_avail - num_new
        self._extract_available(self.slot_available_for_compact, self.cache_size)  # (:684-713)
        compact_active_ids(self.cache_size, self.slot_available_for_compact, self.slot_available_offsets,
                           self.slot_available_ids)
        aligned = sort_aligned_size(num_avail)  # sort keys and values (:717-766)
        keys = np.zeros(aligned, np.uint32)
        sorted_ids = np.zeros(aligned, np.uint32)
        sorted_ids[:num_avail] = self.slot_available_ids[:num_avail]
        for off, tot, groups in push_constant_chunks(-(-num_avail // 32)):
            L.ref_lru_copy_available_slot_age(_ptr(self.slot_available_ids), _ptr(self.slot_data), _ptr(keys),
                                              off, tot, num_avail, groups)
        sort_in_place(keys, sorted_ids, num_avail, True)  # (:769)
        for off, tot, groups in push_constant_chunks(-(-num_new // 32)):  # assign (:810-834)
            L.ref_lru_update(_ptr(self.cached_item_slots), _ptr(sorted_ids), _ptr(self.slot_data), _ptr(new_ids),
                             off, tot, num_new, groups)
        return new_ids

    def reset(self):
        """LRUCache.reset (js/lru_cache.js:846-903): lru_cache_init from slot 0,
        then cachedItemSlots set to -1."""
        for off, tot, groups in push_constant_chunks(self.cache_size // 32):
            load().ref_lru_init(_ptr(self.slot_data), 0, off, tot, self.cache_size, groups)
        self.cached_item_slots[:self.total] = -1

    def state(self) -> dict:
        return {"item_slots": self.cached_item_slots[:self.total].copy(),
                "age": self.slot_data["age"].copy(), "avail": self.slot_data["available"].copy(),
                "item": self.slot_data["item_id"].copy(), "cache_size": self.cache_size}


class CompressedMarchingCubes:
    """CompressedMarchingCubes (js/compressed_marching_cubes.js) with its LRU
    cache: setCompressedVolume (:432-520, initial cache ceil(5 % of the blocks)
    unless `initial_cache_fraction` says otherwise) and computeSurface
    (:580-809).  The active flags are scanned and compacted by the reference's
    scan and compaction shaders, the LRU update runs as LRUCache above, the new
    blocks are decoded into their slots by zfp_decompress_block, and the MC
    programs read the blocks through cachedItemSlots.  The scans of the MC
    stage's per-block counts are numpy sums, as in `surface`."""

    def __init__(self, words, rate: int, dims, initial_cache_fraction: float = 0.05):
        self.words = _words(words)
        self.rate = rate
        self.dims = tuple(int(d) for d in dims)
        self.total_blocks = int(np.prod([(d + 3) // 4 for d in self.dims]))
        self.lru = LRUCache(int(np.ceil(self.total_blocks * initial_cache_fraction)), self.total_blocks)
        self.ranges = block_ranges(words, rate, dims)
        self.active_offsets = np.zeros(_align(self.total_blocks, SCAN_BLOCK), np.uint32)
        self.active_scanner = ExclusiveScanner(self.active_offsets, len(self.active_offsets))
        self.last = {}

    def compute_surface(self, iso: float) -> int:
        L = load()
        d = _dims(self.dims)
        active = block_active(self.ranges, self.dims, iso)
        self.active_offsets[:self.total_blocks] = active
        n = self.active_scanner.scan(self.total_blocks)
        self.last = {"active": active, "numActiveBlocks": n, "newDecompressed": 0, "numVertices": 0,
                     "numBlocksWithVertices": 0, "vertices": np.zeros((0, 2), np.uint32)}
        if n == 0:
            return 0
        new_ids = self.lru.update(active)
        slots = self.lru.cached_item_slots[:self.total_blocks]
        uslots = np.ascontiguousarray(slots).view(np.uint32)
        cache = self.lru.cache
        if len(new_ids):
            L.ref_zfp_decompress_blocks(_p(self.words), 64 * self.rate, _p(new_ids), len(new_ids), _p(uslots),
                                        _p(cache))
        ids = np.zeros(n, np.uint32)
        compact_active_ids(self.total_blocks, active, self.active_offsets, ids)
        has = np.zeros(n, np.uint32)
        L.ref_block_has_vertices(_p(d), F32(iso), _p(cache), _p(active), _p(uslots), _p(ids), n, _p(has))
        with_verts = np.nonzero(has)[0].astype(np.uint32)
        m = len(with_verts)
        counts = np.zeros(max(m, 1), np.uint32)
        if m:
            L.ref_block_num_verts(_p(d), F32(iso), _p(cache), _p(active), _p(uslots), _p(ids), _p(with_verts), m,
                                  _p(counts))
        counts = counts[:m]
        offsets = (np.cumsum(counts.astype(np.uint64)) - counts).astype(np.uint32)
        nverts = int(counts.astype(np.uint64).sum())
        verts = np.zeros((max(nverts, 1), 2), np.uint32)
        if m and nverts:
            info = np.ascontiguousarray(np.stack([with_verts, offsets], axis=1).astype(np.uint32))
            L.ref_block_vertices(_p(d), F32(iso), _p(cache), _p(active), _p(uslots), _p(ids), _p(info), m,
                                 _p(verts))
        self.last.update({"newDecompressed": len(new_ids), "numBlocksWithVertices": m, "numVertices": nverts,
                          "active_ids": ids, "vertices": verts[:nverts]})
        return nverts

    def cache_reset(self):
        self.lru.reset()
