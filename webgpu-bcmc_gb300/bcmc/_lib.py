"""ctypes binding of libbcmc_gb300.so (the C ABI in include/bcmc.h).

The shared library is the product; this module only declares its entry points.
Loading fails loudly when the library has not been built: there is no CPU
fallback behind it.
"""
from __future__ import annotations

import ctypes as C
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libbcmc_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG_ROOT), "include", "bcmc.h")

BCMC_OK = 0
STATUS_NAMES = {0: "BCMC_OK", 1: "BCMC_E_ARG", 2: "BCMC_E_OOM", 3: "BCMC_E_CUDA", 4: "BCMC_E_TIMEOUT",
                5: "BCMC_E_ADMISSION", 6: "BCMC_E_STATE",
                7: "BCMC_E_LIMIT"}


class bcmc_opts(C.Structure):
    _fields_ = [("device", C.c_int), ("initial_cache_fraction", C.c_double), ("flags", C.c_uint32)]


class bcmc_perf(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("computeActiveBlocks", "cacheUpdate", "decompression",
                                          "computeVertices", "total")]


class bcmc_stats(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("totalBlocks", "numActiveBlocks", "newDecompressed",
                                           "numBlocksWithVertices", "numVertices", "cacheSize",
                                           "displayNumSlotsAvailable", "lastNumVertices")]


class bcmc_memory(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("compressedData", "vertexBuffer", "blockActive", "blockRanges",
                                           "activeBlockIDs", "blocksWithVertices", "blockVertexOffsets",
                                           "cache", "cachedItemSlots", "slotData", "scratch", "deviceTotal")]


class bcmc_vol_views(C.Structure):
    _fields_ = [("d_block_ranges", C.c_void_p), ("d_block_active", C.c_void_p),
                ("d_active_block_ids", C.c_void_p), ("d_blocks_with_vertices", C.c_void_p),
                ("d_block_vertex_offsets", C.c_void_p), ("d_new_item_ids", C.c_void_p), ("lru", C.c_void_p)]


class bcmc_lru_view(C.Structure):
    _fields_ = [("cacheSize", C.c_uint32), ("totalElements", C.c_uint32), ("elementSize", C.c_uint32),
                ("displayNumSlotsAvailable", C.c_uint32), ("d_cached_item_slots", C.c_void_p),
                ("d_slot_age", C.c_void_p), ("d_slot_available", C.c_void_p), ("d_slot_item", C.c_void_p),
                ("d_cache", C.c_void_p), ("d_last_sorted_slots", C.c_void_p),
                ("lastNumSlotsAvailable", C.c_uint32)]


class bcmc_engine_opts(C.Structure):
    _fields_ = [("pool_slots", C.c_uint64), ("vertex_capacity", C.c_uint64), ("vertex_budget", C.c_uint64),
                ("max_batch", C.c_uint32), ("flags", C.c_uint32)]


class bcmc_tune_report(C.Structure):
    _fields_ = [("bucket", C.c_uint32)] + [(n, C.c_int32) for n in ("act_ctas_per_sm", "decode_threads",
                                                                     "decode_ctas_per_sm", "mc_ctas_per_sm")] + \
               [(n, C.c_double) for n in ("batch_ms_default", "batch_ms_tuned", "decode_ms_default",
                                          "decode_ms_tuned")] + [("mc_blocks_per_tile", C.c_int32)]


class bcmc_render_params(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("proj_view", C.c_float * 16),
                ("eye_pos", C.c_float * 3), ("fog", C.c_int32)]


class bcmc_server_opts(C.Structure):
    _fields_ = [("max_batch", C.c_uint32), ("max_wait_us", C.c_uint32)]


class bcmc_load_spec(C.Structure):
    _fields_ = [("rate_qps", C.c_double), ("requests", C.c_uint32), ("num_volumes", C.c_uint32),
                ("seed", C.c_uint64), ("volumes", C.POINTER(C.c_uint32)), ("weights", C.POINTER(C.c_float)),
                ("iso_lo", C.POINTER(C.c_float)), ("iso_hi", C.POINTER(C.c_float))]


class bcmc_load_report(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("offered_qps", "achieved_qps", "p50_ms", "p95_ms", "p99_ms", "mean_ms",
                                           "max_ms", "mean_batch", "duration_s")] + \
               [(n, C.c_uint64) for n in ("completed", "batches", "vertices", "overlapped_batches")]


class bcmc_query(C.Structure):
    _fields_ = [("volume", C.c_uint32), ("isovalue", C.c_float)]


class bcmc_query_result(C.Structure):
    _fields_ = [("vertex_offset", C.c_uint64), ("num_vertices", C.c_uint32), ("num_active_blocks", C.c_uint32)]


class bcmc_engine_stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("batches", "launch_sequences", "queries", "decoded_blocks",
                                           "evicted_blocks", "pool_slots", "pool_used", "vertex_capacity",
                                           "device_bytes")] + [("last_batch_ms", C.c_double),
                                                                ("overlapped_batches", C.c_uint64)]


P = C.c_void_p
U32 = C.c_uint32
U64 = C.c_uint64
U32P = C.POINTER(C.c_uint32)

# name -> (restype, argtypes); mirrors include/bcmc.h
SIGNATURES = {
    "bcmc_opts_default": (None, [C.POINTER(bcmc_opts)]),
    "bcmc_ctx_create": (C.c_int, [C.POINTER(bcmc_opts), C.POINTER(P)]),
    "bcmc_ctx_destroy": (None, [P]),
    "bcmc_last_error": (C.c_char_p, [P]),
    "bcmc_ctx_stream": (P, [P]),
    "bcmc_ctx_synchronize": (C.c_int, [P]),
    "bcmc_kernel_launches": (U64, []),
    "bcmc_debug_drop_tile": (C.c_int, [P, U32]),
    "bcmc_volume_create": (C.c_int, [P, P, C.c_size_t, U32, U32P, C.POINTER(C.c_float), C.POINTER(P)]),
    "bcmc_volume_create_device": (C.c_int, [P, P, C.c_size_t, U32, U32P, C.POINTER(C.c_float), C.POINTER(P)]),
    "bcmc_volume_destroy": (None, [P]),
    "bcmc_compute_surface": (C.c_int, [P, C.c_float, C.POINTER(bcmc_perf), U32P]),
    "bcmc_compute_surface_host": (C.c_int, [P, C.c_float, P, U64, C.POINTER(U32)]),
    "bcmc_compute_surfaces_host": (C.c_int, [P, C.POINTER(C.c_float), U32, P, U64, C.POINTER(U32)]),
    "bcmc_vertices": (C.c_int, [P, C.POINTER(P), C.POINTER(U64)]),
    "bcmc_copy_vertices": (C.c_int, [P, P, U64]),
    "bcmc_stats_get": (C.c_int, [P, C.POINTER(bcmc_stats)]),
    "bcmc_memory_report": (C.c_int, [P, C.POINTER(bcmc_memory)]),
    "bcmc_cache_reset": (C.c_int, [P]),
    "bcmc_volume_views": (C.c_int, [P, C.POINTER(bcmc_vol_views)]),
    "bcmc_lru_create": (C.c_int, [P, U32, U32, U32, C.POINTER(P)]),
    "bcmc_lru_destroy": (None, [P]),
    "bcmc_lru_update": (C.c_int, [P, P, U32P, C.POINTER(P)]),
    "bcmc_lru_reset": (C.c_int, [P]),
    "bcmc_lru_view_get": (C.c_int, [P, C.POINTER(bcmc_lru_view)]),
    "bcmc_scan_aligned_size": (U32, [U32]),
    "bcmc_scan_exclusive_u32": (C.c_int, [P, P, U32, U32, U32P]),
    "bcmc_scan_exclusive_u32_async": (C.c_int, [P, P, P, U32, P, P]),
    "bcmc_scan_exclusive_u32_noalloc": (C.c_int, [P, P, U32, P, P]),
    "bcmc_unpack_vertices": (C.c_int, [P, P, U64, U32P, C.POINTER(C.c_float), P, C.POINTER(C.c_float), P, P]),
    "bcmc_render": (C.c_int, [P, P, U64, U32P, C.POINTER(C.c_float), C.POINTER(bcmc_render_params), P, P, P, P]),
    "bcmc_engine_create": (C.c_int, [P, C.POINTER(bcmc_engine_opts), C.POINTER(P)]),
    "bcmc_engine_destroy": (None, [P]),
    "bcmc_engine_add_volume": (C.c_int, [P, P, C.c_size_t, U32, U32P, U32P]),
    "bcmc_engine_run": (C.c_int, [P, C.POINTER(bcmc_query), U32, C.POINTER(bcmc_query_result)]),
    "bcmc_engine_run_admit": (C.c_int, [P, C.POINTER(bcmc_query), U32, C.POINTER(bcmc_query_result), U32P]),
    "bcmc_engine_vertices": (C.c_int, [P, C.POINTER(P), C.POINTER(U64)]),
    "bcmc_engine_copy_vertices": (C.c_int, [P, U64, U64, P]),
    "bcmc_engine_stats_get": (C.c_int, [P, C.POINTER(bcmc_engine_stats)]),
    "bcmc_engine_autotune": (C.c_int, [P, C.POINTER(bcmc_query), U32, C.POINTER(bcmc_tune_report)]),
    "bcmc_engine_set_tuning": (C.c_int, [P, C.POINTER(bcmc_tune_report)]),
    "bcmc_server_create": (C.c_int, [P, C.POINTER(bcmc_server_opts), C.POINTER(P)]),
    "bcmc_server_destroy": (None, [P]),
    "bcmc_server_submit": (C.c_int, [P, U32, C.c_float, P, U64, C.POINTER(U64)]),
    "bcmc_server_wait": (C.c_int, [P, U64, C.POINTER(bcmc_query_result), C.POINTER(C.c_double)]),
    "bcmc_server_run_load": (C.c_int, [P, C.POINTER(bcmc_load_spec), C.POINTER(bcmc_load_report)]),
    "bcmc_compact_ids": (C.c_int, [P, U32, P, P, P, P]),
    "bcmc_select_ids": (C.c_int, [P, U32, P, P, P, P]),
    "bcmc_sort_aligned_size": (U32, [U32]),
    "bcmc_sort_pairs_u32": (C.c_int, [P, P, P, U32, C.c_int, P]),
    "bcmc_zfp_block_ranges": (C.c_int, [P, P, U32P, U32, P, P]),
    "bcmc_zfp_decode_blocks": (C.c_int, [P, P, U32, P, U32, P, P, P]),
    "bcmc_zfp_decode_volume": (C.c_int, [P, P, U64, U32, P, P]),
    "bcmc_zfp_stream_words": (U64, [U32P, U32]),
    "bcmc_zfp_encode": (C.c_int, [P, P, U32P, U32, P, P]),
    "bcmc_block_active": (C.c_int, [P, P, U32P, C.c_float, P, P]),
}

_lib = None


class BcmcError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


def load():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python webgpu-bcmc_gb300/build.py` "
                              "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (rt, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = rt
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int, ctx=None) -> None:
    if code != BCMC_OK:
        msg = ""
        if ctx:
            raw = load().bcmc_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise BcmcError(code, msg)


def dims3(dims) -> C.Array:
    return (C.c_uint32 * 3)(*[int(d) for d in dims])


def scale3(scale) -> C.Array:
    return (C.c_float * 3)(*[float(s) for s in scale])
