"""ctypes front end of the CPU oracle (oracle/bcmc_oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` load this module, to check the CUDA results
against it and to time it.  The product library never imports it.

The oracle restates Twinklebear/webgpu-bcmc's compute shaders and JavaScript
orchestration (citations live in bcmc_oracle.c) and adds a fixed-rate ZFP
encoder written from the published method, because the reference only decodes.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# BCMC_ORACLE_SANITIZE=1 selects the AddressSanitizer + UBSan build (`make
# asan`); the Python process must then preload libasan and libubsan
# (LD_PRELOAD), since the interpreter is not built with them
_SANITIZE = os.environ.get("BCMC_ORACLE_SANITIZE") == "1"
_LIB_PATH = os.path.join(_HERE, "_build", "libbcmc_oracle_asan.so" if _SANITIZE else "libbcmc_oracle.so")
_lib = None

u32p = C.POINTER(C.c_uint32)
i32p = C.POINTER(C.c_int32)
u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)


def build() -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE] + (["asan"] if _SANITIZE else []), check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "bcmc_oracle.c")
        ):
            build()
        L = C.CDLL(_LIB_PATH)
        L.bcmc_oracle_stream_words.restype = C.c_uint64
        L.bcmc_oracle_stream_words.argtypes = [u32p, C.c_uint32]
        L.bcmc_oracle_zfp_encode.restype = C.c_int
        L.bcmc_oracle_zfp_encode.argtypes = [f32p, u32p, C.c_uint32, u64p]
        L.bcmc_oracle_decode_block.argtypes = [u64p, C.c_uint64, C.c_uint32, C.c_int, f32p]
        L.bcmc_oracle_decode_block_native.argtypes = [u64p, C.c_uint64, C.c_uint32, f32p]
        L.bcmc_oracle_decode_block_ints.argtypes = [u64p, C.c_uint64, C.c_uint32, u32p, u32p, i32p]
        L.bcmc_oracle_decode_volume.argtypes = [u64p, C.c_uint64, C.c_uint32, f32p]
        L.bcmc_oracle_block_ranges.argtypes = [u64p, u32p, C.c_uint32, f32p]
        L.bcmc_oracle_block_active.argtypes = [f32p, u32p, C.c_float, u32p]
        L.bcmc_oracle_unpack_vertices.argtypes = [u32p, C.c_uint64, u32p, f32p, f32p, f32p, f32p]
        L.bcmc_oracle_fog_enter.argtypes = [f32p, C.c_uint64, f32p, f32p, f32p]
        L.bcmc_oracle_shade.argtypes = [f32p, C.c_float, f32p, f32p, C.c_int, f32p]
        L.bcmc_oracle_render.argtypes = [u32p, C.c_uint64, u32p, f32p, f32p, f32p, C.c_int, C.c_uint32,
                                         C.c_uint32, f32p, f32p, u32p]
        L.bcmc_oracle_render.restype = C.c_int
        L.bcmc_oracle_exclusive_scan.restype = C.c_uint32
        L.bcmc_oracle_exclusive_scan.argtypes = [u32p, C.c_uint32, C.c_uint32]
        L.bcmc_oracle_compact.argtypes = [u32p, u32p, C.c_uint32, u32p]
        L.bcmc_oracle_sort_aligned_size.restype = C.c_uint32
        L.bcmc_oracle_sort_aligned_size.argtypes = [C.c_uint32]
        L.bcmc_oracle_sort_by_key.argtypes = [u32p, u32p, C.c_uint32, C.c_int]
        L.bcmc_oracle_lru_create.restype = C.c_void_p
        L.bcmc_oracle_lru_create.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        L.bcmc_oracle_lru_destroy.argtypes = [C.c_void_p]
        L.bcmc_oracle_lru_update.restype = C.c_uint32
        L.bcmc_oracle_lru_update.argtypes = [C.c_void_p, u32p, u32p]
        L.bcmc_oracle_lru_reset.argtypes = [C.c_void_p]
        L.bcmc_oracle_lru_cache_size.restype = C.c_uint32
        L.bcmc_oracle_lru_cache_size.argtypes = [C.c_void_p]
        L.bcmc_oracle_lru_slots_available.restype = C.c_uint32
        L.bcmc_oracle_lru_slots_available.argtypes = [C.c_void_p]
        for name, rt in (
            ("bcmc_oracle_lru_item_slots", i32p),
            ("bcmc_oracle_lru_slot_age", u32p),
            ("bcmc_oracle_lru_slot_avail", u32p),
            ("bcmc_oracle_lru_slot_item", i32p),
            ("bcmc_oracle_lru_cache_data", f32p),
        ):
            getattr(L, name).restype = rt
            getattr(L, name).argtypes = [C.c_void_p]
        L.bcmc_oracle_lru_last_sorted.restype = u32p
        L.bcmc_oracle_lru_last_sorted.argtypes = [C.c_void_p, u32p]
        L.bcmc_oracle_mc_create.restype = C.c_void_p
        L.bcmc_oracle_mc_create.argtypes = [u64p, C.c_uint64, C.c_uint32, u32p, f32p, C.c_double]
        L.bcmc_oracle_mc_destroy.argtypes = [C.c_void_p]
        L.bcmc_oracle_mc_compute_surface.restype = C.c_uint32
        L.bcmc_oracle_mc_compute_surface.argtypes = [C.c_void_p, C.c_float]
        L.bcmc_oracle_mc_cache_reset.argtypes = [C.c_void_p]
        L.bcmc_oracle_mc_lru.restype = C.c_void_p
        L.bcmc_oracle_mc_lru.argtypes = [C.c_void_p]
        for name, rt in (
            ("bcmc_oracle_mc_vertices", u32p),
            ("bcmc_oracle_mc_ranges", f32p),
            ("bcmc_oracle_mc_active", u32p),
            ("bcmc_oracle_mc_active_ids", u32p),
            ("bcmc_oracle_mc_with_verts", u32p),
            ("bcmc_oracle_mc_vert_offsets", u32p),
            ("bcmc_oracle_mc_new_items", u32p),
        ):
            getattr(L, name).restype = rt
            getattr(L, name).argtypes = [C.c_void_p]
        L.bcmc_oracle_mc_stats.argtypes = [C.c_void_p, u32p]
        L.bcmc_oracle_case_vertex_count.restype = C.c_uint32
        L.bcmc_oracle_case_vertex_count.argtypes = [C.c_uint32]
        L.bcmc_oracle_tri_table.restype = i32p
        L.bcmc_oracle_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray, t):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(t)


def _dims(dims) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(dims, dtype=np.uint32).reshape(3))


def threads() -> int:
    return int(lib().bcmc_oracle_threads())


def padded_blocks(dims) -> tuple:
    return tuple(int((d + 3) // 4) for d in dims)


def stream_words(dims, max_bits: int) -> int:
    return int(lib().bcmc_oracle_stream_words(_p(_dims(dims), u32p), max_bits))


def zfp_encode(field: np.ndarray, rate: int) -> np.ndarray:
    """field: float32 array indexed [z, y, x] (x fastest).  Returns uint64 words
    (fixed rate, 64*rate bits per 4^3 block, one trailing zero pad word)."""
    f = np.ascontiguousarray(field, dtype=np.float32)
    dims = _dims((f.shape[2], f.shape[1], f.shape[0]))
    max_bits = 64 * int(rate)
    out = np.zeros(stream_words(dims, max_bits), dtype=np.uint64)
    rc = lib().bcmc_oracle_zfp_encode(_p(f, f32p), _p(dims, u32p), max_bits, _p(out, u64p))
    if rc != 0:
        raise ValueError("zfp_encode failed")
    return out


def decode_block(words: np.ndarray, block: int, max_bits: int, emulate_u32_offset=False,
                 native=False) -> np.ndarray:
    out = np.zeros(64, dtype=np.float32)
    if native:
        lib().bcmc_oracle_decode_block_native(_p(words, u64p), block, max_bits, _p(out, f32p))
    else:
        lib().bcmc_oracle_decode_block(_p(words, u64p), block, max_bits, int(emulate_u32_offset),
                                       _p(out, f32p))
    return out


def decode_volume(words: np.ndarray, nblocks: int, max_bits: int) -> np.ndarray:
    out = np.zeros(nblocks * 64, dtype=np.float32)
    lib().bcmc_oracle_decode_volume(_p(words, u64p), nblocks, max_bits, _p(out, f32p))
    return out


def block_ranges(words: np.ndarray, dims, max_bits: int) -> np.ndarray:
    nb = int(np.prod(padded_blocks(dims)))
    out = np.zeros(2 * nb, dtype=np.float32)
    lib().bcmc_oracle_block_ranges(_p(words, u64p), _p(_dims(dims), u32p), max_bits, _p(out, f32p))
    return out


def unpack_vertices(verts: np.ndarray, dims, scale=(1.0, 1.0, 1.0), proj_view=None):
    """mc_isosurface.vert:51-60: world positions [n, 3] (and clip [n, 4])."""
    v = np.ascontiguousarray(verts, dtype=np.uint32).reshape(-1, 2)
    n = len(v)
    world = np.zeros((n, 3), np.float32)
    sc = np.ascontiguousarray(np.asarray(scale, np.float32))
    clip = np.zeros((n, 4), np.float32) if proj_view is not None else None
    pv = np.ascontiguousarray(np.asarray(proj_view, np.float32).reshape(16)) if proj_view is not None else None
    lib().bcmc_oracle_unpack_vertices(_p(v, u32p), n, _p(_dims(dims), u32p), _p(sc, f32p),
                                      _p(pv, f32p) if pv is not None else None, _p(world, f32p),
                                      _p(clip, f32p) if clip is not None else None)
    return (world, clip) if clip is not None else world


def fog_enter(world: np.ndarray, eye, scale=(1.0, 1.0, 1.0)) -> np.ndarray:
    """mc_isosurface.vert:35-49 (DRAW_FOG): per vertex where the eye ray enters the volume's box."""
    w = np.ascontiguousarray(world, dtype=np.float32).reshape(-1, 3)
    out = np.zeros(len(w), np.float32)
    e = np.ascontiguousarray(np.asarray(eye, np.float32))
    sc = np.ascontiguousarray(np.asarray(scale, np.float32))
    lib().bcmc_oracle_fog_enter(_p(w, f32p), len(w), _p(e, f32p), _p(sc, f32p), _p(out, f32p))
    return out


def shade(world_pos, t_enter: float, eye, tri_world, fog: bool) -> np.ndarray:
    """mc_isosurface.frag:15-40 for one fragment."""
    wp = np.ascontiguousarray(np.asarray(world_pos, np.float32))
    e = np.ascontiguousarray(np.asarray(eye, np.float32))
    tw = np.ascontiguousarray(np.asarray(tri_world, np.float32).reshape(9))
    out = np.zeros(4, np.float32)
    lib().bcmc_oracle_shade(_p(wp, f32p), float(t_enter), _p(e, f32p), _p(tw, f32p), 1 if fog else 0,
                            _p(out, f32p))
    return out


def render(verts: np.ndarray, dims, proj_view, eye, width: int, height: int, scale=(1.0, 1.0, 1.0),
           fog: bool = False):
    """The render pass, headless: (rgba [h, w, 4], depth [h, w], triangle [h, w] u32)."""
    v = np.ascontiguousarray(verts, dtype=np.uint32).reshape(-1, 2)
    rgba = np.zeros((height, width, 4), np.float32)
    depth = np.zeros((height, width), np.float32)
    tri = np.zeros((height, width), np.uint32)
    pv = np.ascontiguousarray(np.asarray(proj_view, np.float32).reshape(16))
    e = np.ascontiguousarray(np.asarray(eye, np.float32))
    sc = np.ascontiguousarray(np.asarray(scale, np.float32))
    rc = lib().bcmc_oracle_render(_p(v, u32p), len(v), _p(_dims(dims), u32p), _p(sc, f32p), _p(pv, f32p),
                                  _p(e, f32p), 1 if fog else 0, width, height, _p(rgba, f32p), _p(depth, f32p),
                                  _p(tri, u32p))
    if rc != 0:
        raise MemoryError("oracle render: host allocation failed")
    return rgba, depth, tri


def block_active(ranges: np.ndarray, dims, iso: float) -> np.ndarray:
    nb = int(np.prod(padded_blocks(dims)))
    out = np.zeros(nb, dtype=np.uint32)
    r = np.ascontiguousarray(ranges, dtype=np.float32)
    lib().bcmc_oracle_block_active(_p(r, f32p), _p(_dims(dims), u32p), float(iso), _p(out, u32p))
    return out


def exclusive_scan(data: np.ndarray, n: int, aligned_n: int) -> tuple:
    d = np.array(data, dtype=np.uint32, copy=True)
    assert len(d) >= aligned_n or n == aligned_n
    tot = lib().bcmc_oracle_exclusive_scan(_p(d, u32p), n, aligned_n)
    return d, int(tot)


def compact(flags: np.ndarray, offsets: np.ndarray, n: int, out_len: int) -> np.ndarray:
    out = np.zeros(max(out_len, 1), dtype=np.uint32)
    f = np.ascontiguousarray(flags, dtype=np.uint32)
    o = np.ascontiguousarray(offsets, dtype=np.uint32)
    lib().bcmc_oracle_compact(_p(f, u32p), _p(o, u32p), n, _p(out, u32p))
    return out[:out_len]


def sort_aligned_size(n: int) -> int:
    return int(lib().bcmc_oracle_sort_aligned_size(n))


def sort_by_key(keys: np.ndarray, values: np.ndarray, reverse: bool) -> tuple:
    """Returns (keys, values) in the reference RadixSorter's output order."""
    n = len(keys)
    a = sort_aligned_size(n)
    k = np.zeros(a, dtype=np.uint32)
    v = np.zeros(a, dtype=np.uint32)
    k[:n] = keys
    v[:n] = values
    lib().bcmc_oracle_sort_by_key(_p(k, u32p), _p(v, u32p), n, int(reverse))
    return k[:n].copy(), v[:n].copy()


class LRUCache:
    """Oracle LRUCache (js/lru_cache.js), element size fixed at 256 B."""

    def __init__(self, initial_size: int, total_elements: int, element_size: int = 256):
        self.total = total_elements
        self._h = lib().bcmc_oracle_lru_create(initial_size, element_size, total_elements)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().bcmc_oracle_lru_destroy(self._h)
            self._h = None

    def update(self, needed: np.ndarray) -> np.ndarray:
        nd = np.ascontiguousarray(needed, dtype=np.uint32)
        out = np.zeros(max(self.total, 1), dtype=np.uint32)
        n = lib().bcmc_oracle_lru_update(self._h, _p(nd, u32p), _p(out, u32p))
        return out[:n].copy()

    def reset(self):
        lib().bcmc_oracle_lru_reset(self._h)

    @property
    def cache_size(self) -> int:
        return int(lib().bcmc_oracle_lru_cache_size(self._h))

    @property
    def slots_available(self) -> int:
        return int(lib().bcmc_oracle_lru_slots_available(self._h))

    def state(self) -> dict:
        L = lib()
        cs = self.cache_size
        return {
            "item_slots": np.ctypeslib.as_array(L.bcmc_oracle_lru_item_slots(self._h), (self.total,)).copy(),
            "age": np.ctypeslib.as_array(L.bcmc_oracle_lru_slot_age(self._h), (cs,)).copy(),
            "avail": np.ctypeslib.as_array(L.bcmc_oracle_lru_slot_avail(self._h), (cs,)).copy(),
            "item": np.ctypeslib.as_array(L.bcmc_oracle_lru_slot_item(self._h), (cs,)).copy(),
        }

    def last_sorted(self) -> np.ndarray:
        n = C.c_uint32(0)
        p = lib().bcmc_oracle_lru_last_sorted(self._h, C.byref(n))
        if n.value == 0:
            return np.zeros(0, dtype=np.uint32)
        return np.ctypeslib.as_array(p, (n.value,)).copy()


class CompressedMarchingCubes:
    """Oracle of js/compressed_marching_cubes.js: the plain one-query-at-a-time
    pipeline on the CPU."""

    def __init__(self, words: np.ndarray, rate: int, dims, scale=(1.0, 1.0, 1.0),
                 initial_cache_fraction: float = 0.05):
        self.words = np.ascontiguousarray(words, dtype=np.uint64)
        self.dims = tuple(int(d) for d in dims)
        d = _dims(dims)
        s = np.ascontiguousarray(np.asarray(scale, dtype=np.float32))
        self._h = lib().bcmc_oracle_mc_create(_p(self.words, u64p), len(self.words), rate,
                                              _p(d, u32p), _p(s, f32p), initial_cache_fraction)
        self.total_blocks = int(np.prod(padded_blocks(dims)))
        self._lru_view = None

    def __del__(self):
        if getattr(self, "_h", None):
            lib().bcmc_oracle_mc_destroy(self._h)
            self._h = None

    def compute_surface(self, iso: float) -> int:
        return int(lib().bcmc_oracle_mc_compute_surface(self._h, float(iso)))

    def cache_reset(self):
        lib().bcmc_oracle_mc_cache_reset(self._h)

    def vertices(self, n: int) -> np.ndarray:
        if n == 0:
            return np.zeros((0, 2), dtype=np.uint32)
        p = lib().bcmc_oracle_mc_vertices(self._h)
        return np.ctypeslib.as_array(p, (n, 2)).copy()

    def vertices_view(self, n: int) -> np.ndarray:
        """The last query's vertices without a copy: valid until the next query."""
        if n == 0:
            return np.zeros((0, 2), dtype=np.uint32)
        return np.ctypeslib.as_array(lib().bcmc_oracle_mc_vertices(self._h), (n, 2))

    def ranges(self) -> np.ndarray:
        return np.ctypeslib.as_array(lib().bcmc_oracle_mc_ranges(self._h), (2 * self.total_blocks,)).copy()

    def active(self) -> np.ndarray:
        return np.ctypeslib.as_array(lib().bcmc_oracle_mc_active(self._h), (self.total_blocks,)).copy()

    def _arr(self, fn, n):
        if n == 0:
            return np.zeros(0, dtype=np.uint32)
        return np.ctypeslib.as_array(getattr(lib(), fn)(self._h), (n,)).copy()

    def active_ids(self, n):
        return self._arr("bcmc_oracle_mc_active_ids", n)

    def with_verts(self, n):
        return self._arr("bcmc_oracle_mc_with_verts", n)

    def vert_offsets(self, n):
        return self._arr("bcmc_oracle_mc_vert_offsets", n)

    def new_items(self, n):
        return self._arr("bcmc_oracle_mc_new_items", n)

    def stats(self) -> dict:
        s = np.zeros(7, dtype=np.uint32)
        lib().bcmc_oracle_mc_stats(self._h, _p(s, u32p))
        keys = ("totalBlocks", "numActiveBlocks", "newDecompressed", "numBlocksWithVertices",
                "numVertices", "cacheSize", "slotsAvailable")
        return {k: int(v) for k, v in zip(keys, s)}

    def lru_state(self) -> dict:
        h = lib().bcmc_oracle_mc_lru(self._h)
        L = lib()
        cs = int(L.bcmc_oracle_lru_cache_size(h))
        return {
            "item_slots": np.ctypeslib.as_array(L.bcmc_oracle_lru_item_slots(h), (self.total_blocks,)).copy(),
            "age": np.ctypeslib.as_array(L.bcmc_oracle_lru_slot_age(h), (cs,)).copy(),
            "avail": np.ctypeslib.as_array(L.bcmc_oracle_lru_slot_avail(h), (cs,)).copy(),
            "item": np.ctypeslib.as_array(L.bcmc_oracle_lru_slot_item(h), (cs,)).copy(),
            "cache_size": cs,
        }

    def cache_data(self) -> np.ndarray:
        h = lib().bcmc_oracle_mc_lru(self._h)
        cs = int(lib().bcmc_oracle_lru_cache_size(h))
        return np.ctypeslib.as_array(lib().bcmc_oracle_lru_cache_data(h), (cs * 64,)).copy()


def tri_table() -> np.ndarray:
    return np.ctypeslib.as_array(lib().bcmc_oracle_tri_table(), (256, 16)).copy()


def case_vertex_count(c: int) -> int:
    return int(lib().bcmc_oracle_case_vertex_count(c))
