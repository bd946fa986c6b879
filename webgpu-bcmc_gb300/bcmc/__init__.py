"""bcmc -- GB300-native block-compressed marching cubes.

Python mirror of the JavaScript API of Twinklebear/webgpu-bcmc's compute path,
over the CUDA library libbcmc_gb300.so (C ABI: include/bcmc.h):

* ``CompressedMarchingCubes``  js/compressed_marching_cubes.js
* ``LRUCache``                 js/lru_cache.js
* ``ExclusiveScanPipeline`` / ``ExclusiveScanner``  js/exclusive_scan.js
* ``StreamCompact``            js/stream_compact.js
* ``RadixSorter``              js/radix_sort_by_key.js
* ``Engine``                   (no reference counterpart) batched queries over
                               several resident volumes, shared slot pool
* ``Server``                   (no reference counterpart) continuous-batching
                               request loop over an Engine

Method names, argument meaning and return values follow the reference.  The
WebGPU ``device`` argument becomes a CUDA device ordinal or a ``Context``;
GPUBuffers become CUDA device buffers (torch tensors or any object with
``__cuda_array_interface__``).  Errors the reference reports with ``alert``
raise ``BcmcError``.  All compute runs in the CUDA library; nothing here falls
back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _lib
from ._lib import BcmcError, check, dims3, scale3

__all__ = ["Context", "CompressedMarchingCubes", "LRUCache", "ExclusiveScanPipeline", "ExclusiveScanner",
           "StreamCompact", "RadixSorter", "DeviceArray", "BcmcError", "zfp_encode", "zfp_decode_volume", "render",
           "zfp_block_ranges", "block_active", "stream_words", "Engine", "Server", "unpack_vertices"]


def _torch():
    import torch

    return torch


class DeviceArray:
    """A view of device memory owned by the library (no copy).  Wrap it with
    ``torch.as_tensor(arr, device="cuda")`` to use it from PyTorch."""

    def __init__(self, ptr: int, shape, typestr: str, owner=None):
        self.ptr = int(ptr or 0)
        self.shape = tuple(int(s) for s in shape)
        self.typestr = typestr
        self._owner = owner

    @property
    def __cuda_array_interface__(self):
        return {"shape": self.shape, "typestr": self.typestr, "data": (self.ptr, False), "version": 3,
                "strides": None}

    def torch(self):
        """Zero-copy torch view; unsigned words appear as int32/int64 (same bits)."""
        t = _torch()
        signed = {"<u4": "<i4", "<u8": "<i8"}.get(self.typestr, self.typestr)
        if int(np.prod(self.shape)) == 0:
            dt = {"<i4": t.int32, "<f4": t.float32, "<i8": t.int64}[signed]
            return t.zeros(self.shape, dtype=dt, device="cuda")
        return t.as_tensor(DeviceArray(self.ptr, self.shape, signed, self), device="cuda")

    def numpy(self) -> np.ndarray:
        return self.torch().cpu().numpy().view(np.dtype(self.typestr))


def _ptr(buf) -> int:
    """Device address of a torch tensor / __cuda_array_interface__ object / int."""
    if buf is None:
        return 0
    if isinstance(buf, int):
        return buf
    if hasattr(buf, "data_ptr"):
        if not buf.is_cuda:
            raise BcmcError(1, "buffer must live on the CUDA device")
        return int(buf.data_ptr())
    if hasattr(buf, "__cuda_array_interface__"):
        return int(buf.__cuda_array_interface__["data"][0])
    raise BcmcError(1, f"not a device buffer: {type(buf)!r}")


_CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the legacy default stream, named explicitly


def _torch_stream() -> int:
    """torch's current stream as a cudaStream_t value.  torch reports its
    default stream as 0, which the C ABI reads as "the context's own stream",
    so it is passed as cudaStreamLegacy to keep the call ordered with torch."""
    t = _torch()
    s = int(t.cuda.current_stream().cuda_stream)
    return s if s != 0 else _CUDA_STREAM_LEGACY


def _sync_torch():
    t = _torch()
    if t.cuda.is_available():
        t.cuda.current_stream().synchronize()


class Context:
    """The CUDA device a pipeline runs on (the reference's WebGPU device)."""

    FULL_RANGES = 1  # BCMC_FLAG_FULL_RANGES

    def __init__(self, device: int = 0, initial_cache_fraction: float = 0.05, flags: int = 0):
        L = _lib.load()
        opts = _lib.bcmc_opts()
        L.bcmc_opts_default(C.byref(opts))
        opts.device = int(device)
        opts.initial_cache_fraction = float(initial_cache_fraction)
        opts.flags = int(flags)
        h = C.c_void_p()
        rc = L.bcmc_ctx_create(C.byref(opts), C.byref(h))
        if rc != 0:
            raise BcmcError(rc, "bcmc_ctx_create failed (is a CUDA device visible?)")
        self.handle = h
        self.device = int(device)
        self.initial_cache_fraction = float(initial_cache_fraction)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            _lib.load().bcmc_ctx_destroy(h)
            self.handle = None

    @property
    def stream(self) -> int:
        return int(_lib.load().bcmc_ctx_stream(self.handle) or 0)

    def synchronize(self):
        check(_lib.load().bcmc_ctx_synchronize(self.handle), self.handle)


def _ctx(device) -> Context:
    if isinstance(device, Context):
        return device
    return Context(0 if device is None else int(device))


def _host_bytes(volume) -> tuple:
    """(ctypes pointer, nbytes, keepalive, on_device) for a compressed stream."""
    if hasattr(volume, "data_ptr") and getattr(volume, "is_cuda", False):
        return C.c_void_p(int(volume.data_ptr())), volume.numel() * volume.element_size(), volume, True
    if isinstance(volume, (bytes, bytearray, memoryview)):
        arr = np.frombuffer(bytes(volume), dtype=np.uint8)
    else:
        arr = np.ascontiguousarray(np.asarray(volume))
    arr = np.ascontiguousarray(arr).view(np.uint8).reshape(-1)
    return arr.ctypes.data_as(C.c_void_p), arr.nbytes, arr, False


class _VolumeLRU:
    """The cache of a CompressedMarchingCubes (``this.lruCache``)."""

    def __init__(self, mc: "CompressedMarchingCubes"):
        self._ref = weakref.ref(mc)  # no reference cycle with its volume

    @property
    def _mc(self) -> "CompressedMarchingCubes":
        mc = self._ref()
        if mc is None:
            raise BcmcError(6, "the volume of this cache was destroyed")
        return mc

    def _view(self) -> _lib.bcmc_lru_view:
        vv = _lib.bcmc_vol_views()
        check(_lib.load().bcmc_volume_views(self._mc._vol, C.byref(vv)), self._mc.ctx.handle)
        v = _lib.bcmc_lru_view()
        check(_lib.load().bcmc_lru_view_get(vv.lru, C.byref(v)), self._mc.ctx.handle)
        return v

    def reset(self):
        check(_lib.load().bcmc_cache_reset(self._mc._vol), self._mc.ctx.handle)

    @property
    def cacheSize(self) -> int:
        return int(self._view().cacheSize)

    @property
    def displayNumSlotsAvailable(self) -> int:
        return int(self._view().displayNumSlotsAvailable)

    @property
    def totalElements(self) -> int:
        return int(self._view().totalElements)

    @property
    def elementSize(self) -> int:
        return int(self._view().elementSize)

    def state(self) -> dict:
        return _lru_state(self._view())


def _lru_state(v: _lib.bcmc_lru_view) -> dict:
    cs, tot = int(v.cacheSize), int(v.totalElements)
    return {
        "cache_size": cs,
        "item_slots": DeviceArray(v.d_cached_item_slots, (tot,), "<i4").numpy(),
        "age": DeviceArray(v.d_slot_age, (cs,), "<u4").numpy(),
        "avail": DeviceArray(v.d_slot_available, (cs,), "<u4").numpy(),
        "item": DeviceArray(v.d_slot_item, (cs,), "<i4").numpy(),
    }


_PERF_KEYS = ("computeActiveBlocks", "numActiveBlocks", "cacheUpdate", "numBlocksDecompressed", "decompression",
              "compactActiveIDs", "computeBlockHasVertices", "numBlocksWithVertices", "compactBlocksWithVertices",
              "numVertices", "computeVertices")


class CompressedMarchingCubes:
    """js/compressed_marching_cubes.js: isosurfaces of a ZFP fixed-rate
    compressed volume through an LRU cache of decoded 4^3 blocks."""

    def __init__(self, device=0):
        self.ctx = _ctx(device)
        self._vol = None
        self.totalBlocks = 0

    def __del__(self):
        if getattr(self, "_vol", None):
            _lib.load().bcmc_volume_destroy(self._vol)
            self._vol = None

    # setCompressedVolume (js/compressed_marching_cubes.js:432-520)
    def setCompressedVolume(self, volume, compressionRate: int, volumeDims, volumeScale=(1.0, 1.0, 1.0)):
        L = _lib.load()
        if self._vol:
            L.bcmc_volume_destroy(self._vol)
            self._vol = None
        ptr, nbytes, keep, on_dev = _host_bytes(volume)
        if on_dev:
            _sync_torch()
        h = C.c_void_p()
        fn = L.bcmc_volume_create_device if on_dev else L.bcmc_volume_create
        check(fn(self.ctx.handle, ptr, nbytes, int(compressionRate), dims3(volumeDims), scale3(volumeScale),
                 C.byref(h)), self.ctx.handle)
        del keep
        self._vol = h
        self.volumeDims = tuple(int(d) for d in volumeDims)
        self.paddedDims = tuple((d + 3) // 4 * 4 for d in self.volumeDims)
        self.compressionRate = int(compressionRate)
        self.totalBlocks = int(np.prod([p // 4 for p in self.paddedDims]))
        self.compressedDataSize = int(nbytes)
        self.lruCache = _VolumeLRU(self)

    # computeSurface (js/compressed_marching_cubes.js:580-809)
    def computeSurface(self, isovalue: float, perfTracker: dict | None = None) -> int:
        if not self._vol:
            raise BcmcError(6, "setCompressedVolume must be called first")
        n = C.c_uint32(0)
        perf = _lib.bcmc_perf() if perfTracker is not None else None
        check(_lib.load().bcmc_compute_surface(self._vol, float(isovalue), C.byref(perf) if perf else None,
                                               C.byref(n)), self.ctx.handle)
        if perfTracker is not None:
            for k in _PERF_KEYS:
                perfTracker.setdefault(k, [])
            perfTracker["totalBlocks"] = self.totalBlocks
            st = self.stats()
            perfTracker["computeActiveBlocks"].append(perf.computeActiveBlocks)
            perfTracker["numActiveBlocks"].append(st["numActiveBlocks"])
            perfTracker["cacheUpdate"].append(perf.cacheUpdate)
            perfTracker["numBlocksDecompressed"].append(st["newDecompressed"])
            perfTracker["decompression"].append(perf.decompression)
            perfTracker["compactActiveIDs"].append(0.0)  # fused into computeActiveBlocks
            perfTracker["computeBlockHasVertices"].append(0.0)  # fused into computeVertices
            perfTracker["numBlocksWithVertices"].append(st["numBlocksWithVertices"])
            perfTracker["compactBlocksWithVertices"].append(0.0)
            perfTracker["numVertices"].append(int(n.value))
            perfTracker["computeVertices"].append(perf.computeVertices)
        return int(n.value)

    def computeSurfaceToHost(self, isovalue: float, out: np.ndarray) -> int:
        """computeSurface with the vertices written by the kernels straight into
        `out`, a page-locked host array (e.g. from torch.empty(...,
        pin_memory=True).numpy()) of shape (capacity, 2) uint32: the transfer
        overlaps the vertex computation.  Returns the vertex count; raises
        BcmcError (BCMC_E_LIMIT) when the query has more vertices than `out`
        holds.  The device vertexBuffer is not written by this call."""
        if out.dtype.itemsize * out.size < 8 or out.ctypes.data % 8:
            raise ValueError("out must be an 8-byte aligned array of packed vertices")
        n = C.c_uint32()
        check(_lib.load().bcmc_compute_surface_host(self._vol, float(isovalue), out.ctypes.data_as(C.c_void_p),
                                                    out.nbytes // 8, C.byref(n)), self.ctx.handle)
        return int(n.value)

    def computeSurfacesToHost(self, isovalues, out: np.ndarray) -> list:
        """computeSurface for each isovalue in order, the vertices of all the
        queries back to back in `out` (a page-locked array of shape
        (capacity, 2) uint32); query i+1 computes while query i's vertices are
        copied out.  Returns the vertex count of each query; raises BcmcError
        (BCMC_E_LIMIT) when `out` runs out of room."""
        if out.dtype.itemsize * out.size < 8 or out.ctypes.data % 8:
            raise ValueError("out must be an 8-byte aligned array of packed vertices")
        isos = np.ascontiguousarray(np.asarray(isovalues, dtype=np.float32))
        counts = (C.c_uint32 * max(len(isos), 1))()
        check(_lib.load().bcmc_compute_surfaces_host(self._vol, isos.ctypes.data_as(C.POINTER(C.c_float)),
                                                     len(isos), out.ctypes.data_as(C.c_void_p), out.nbytes // 8,
                                                     counts), self.ctx.handle)
        return [int(counts[i]) for i in range(len(isos))]

    def stats(self) -> dict:
        s = _lib.bcmc_stats()
        check(_lib.load().bcmc_stats_get(self._vol, C.byref(s)), self.ctx.handle)
        return {k: int(getattr(s, k)) for k, _ in _lib.bcmc_stats._fields_}

    @property
    def numActiveBlocks(self) -> int:
        return self.stats()["numActiveBlocks"]

    @property
    def numBlocksWithVertices(self) -> int:
        return self.stats()["numBlocksWithVertices"]

    @property
    def newDecompressed(self) -> int:
        return self.stats()["newDecompressed"]

    @property
    def numVertices(self) -> int:
        return self.stats()["numVertices"]

    @property
    def vertexBuffer(self) -> DeviceArray:
        """Vertices of the last query: (n, 2) uint32 {packed position, block id}."""
        p = C.c_void_p()
        nbytes = C.c_uint64()
        check(_lib.load().bcmc_vertices(self._vol, C.byref(p), C.byref(nbytes)), self.ctx.handle)
        return DeviceArray(p.value, (int(nbytes.value) // 8, 2), "<u4", self)

    def copyVertices(self, out: np.ndarray | None = None) -> np.ndarray:
        n = self.stats()["lastNumVertices"]
        if out is None:
            out = np.empty((n, 2), dtype=np.uint32)
        if n:
            check(_lib.load().bcmc_copy_vertices(self._vol, out.ctypes.data_as(C.c_void_p), n * 8),
                  self.ctx.handle)
        return out[:n]

    # reportMemoryUse (js/compressed_marching_cubes.js:366-430)
    def reportMemoryUse(self):
        m = _lib.bcmc_memory()
        check(_lib.load().bcmc_memory_report(self._vol, C.byref(m)), self.ctx.handle)
        mem = {k: int(getattr(m, k)) for k, _ in _lib.bcmc_memory._fields_}

        def fmt(c):
            for lim, unit in ((1e9, "GB"), (1e6, "MB"), (1e3, "KB")):
                if c > lim:
                    return f"{c / lim:.2f} {unit}"
            return f"{c} B"

        mc_keys = ("compressedData", "vertexBuffer", "blockActive", "blockRanges", "activeBlockIDs",
                   "blocksWithVertices", "blockVertexOffsets", "scratch")
        cache_keys = ("cache", "cachedItemSlots", "slotData")
        mc_text = "Marching Cubes Data:<ul>" + "".join(f"<li>{k}: {fmt(mem[k])}</li>" for k in mc_keys) + "</ul>"
        cache_text = "LRU Cache Data:<ul>" + "".join(f"<li>{k}: {fmt(mem[k])}</li>" for k in cache_keys) + "</ul>"
        use = {"mc": {k: mem[k] for k in mc_keys}, "cache": {k: mem[k] for k in cache_keys}}
        return [mc_text, cache_text, fmt(mem["deviceTotal"]), use]

    # debug views used by the parity tests
    def views(self) -> dict:
        vv = _lib.bcmc_vol_views()
        check(_lib.load().bcmc_volume_views(self._vol, C.byref(vv)), self.ctx.handle)
        st = self.stats()
        nb = self.totalBlocks
        return {
            "ranges": DeviceArray(vv.d_block_ranges, (2 * nb,), "<f4"),
            "active": DeviceArray(vv.d_block_active, (nb,), "<u4"),
            "active_ids": DeviceArray(vv.d_active_block_ids, (st["numActiveBlocks"],), "<u4"),
            "with_verts": DeviceArray(vv.d_blocks_with_vertices, (st["numBlocksWithVertices"],), "<u4"),
            "vert_offsets": DeviceArray(vv.d_block_vertex_offsets, (st["numBlocksWithVertices"],), "<u4"),
            "new_items": DeviceArray(vv.d_new_item_ids, (st["newDecompressed"],), "<u4"),
        }


class LRUCache:
    """js/lru_cache.js: slots of fixed-size elements, oldest evicted first."""

    def __init__(self, device, scanPipeline=None, streamCompact=None, initialSize: int = 0,
                 elementSize: int = 256, totalElements: int = 0):
        self.ctx = scanPipeline.ctx if isinstance(scanPipeline, ExclusiveScanPipeline) else _ctx(device)
        h = C.c_void_p()
        check(_lib.load().bcmc_lru_create(self.ctx.handle, int(initialSize), int(elementSize), int(totalElements),
                                          C.byref(h)), self.ctx.handle)
        self._h = h
        self.totalElements = int(totalElements)
        self.elementSize = int(elementSize)

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.load().bcmc_lru_destroy(self._h)
            self._h = None

    def _view(self):
        v = _lib.bcmc_lru_view()
        check(_lib.load().bcmc_lru_view_get(self._h, C.byref(v)), self.ctx.handle)
        return v

    def update(self, itemNeeded, perfTracker: dict | None = None):
        """Returns [numNewItems, newItemIDs] (js/lru_cache.js:312-843)."""
        _sync_torch()
        n = C.c_uint32(0)
        p = C.c_void_p()
        check(_lib.load().bcmc_lru_update(self._h, C.c_void_p(_ptr(itemNeeded)), C.byref(n), C.byref(p)),
              self.ctx.handle)
        if n.value == 0:
            return [0, None]
        return [int(n.value), DeviceArray(p.value, (int(n.value),), "<u4", self)]

    def reset(self):
        check(_lib.load().bcmc_lru_reset(self._h), self.ctx.handle)

    @property
    def cacheSize(self) -> int:
        return int(self._view().cacheSize)

    @property
    def displayNumSlotsAvailable(self) -> int:
        return int(self._view().displayNumSlotsAvailable)

    @property
    def cache(self) -> DeviceArray:
        v = self._view()
        return DeviceArray(v.d_cache, (int(v.cacheSize) * self.elementSize // 4,), "<u4", self)

    def state(self) -> dict:
        return _lru_state(self._view())


class ExclusiveScanPipeline:
    """js/exclusive_scan.js:14-120."""

    def __init__(self, device=0):
        self.ctx = _ctx(device)

    @staticmethod
    def getAlignedSize(size: int) -> int:
        return int(_lib.load().bcmc_scan_aligned_size(int(size)))

    def prepareInput(self, cpuArray) -> "ExclusiveScanner":
        t = _torch()
        a = np.asarray(cpuArray, dtype=np.uint32)
        aligned = self.getAlignedSize(len(a))
        buf = t.zeros(max(aligned, 1), dtype=t.int32, device="cuda")
        if len(a):
            buf[: len(a)] = t.from_numpy(a.view(np.int32).copy()).cuda()
        return ExclusiveScanner(self, buf, aligned, len(a))

    def prepareGPUInput(self, gpuBuffer, alignedSize: int, dataSize: int | None = None) -> "ExclusiveScanner":
        if self.getAlignedSize(alignedSize) != alignedSize:
            raise BcmcError(1, "GPU input must be aligned to getAlignedSize")  # exclusive_scan.js:117-119
        return ExclusiveScanner(self, gpuBuffer, alignedSize, dataSize)


class ExclusiveScanner:
    """js/exclusive_scan.js:122-295: in-place exclusive scan of a device
    buffer; ``scan(dataSize)`` returns the total and writes it at
    ``[dataSize]`` when ``dataSize < alignedSize``."""

    def __init__(self, pipeline: ExclusiveScanPipeline, gpuBuffer, alignedSize: int, dataSize=None):
        self.scanPipeline = pipeline
        self.inputBuf = gpuBuffer
        self.inputSize = int(alignedSize)
        self.dataSize = dataSize

    def scan(self, dataSize: int) -> int:
        _sync_torch()
        tot = C.c_uint32(0)
        ctx = self.scanPipeline.ctx
        check(_lib.load().bcmc_scan_exclusive_u32(ctx.handle, C.c_void_p(_ptr(self.inputBuf)), int(dataSize),
                                                  self.inputSize, C.byref(tot)), ctx.handle)
        return int(tot.value)


class StreamCompact:
    """js/stream_compact.js."""

    def __init__(self, device=0):
        self.ctx = device.ctx if isinstance(device, ExclusiveScanPipeline) else _ctx(device)

    def compactActiveIDs(self, numElements: int, isActiveBuffer, offsetsBuffer, outputBuffer):
        check(_lib.load().bcmc_compact_ids(self.ctx.handle, int(numElements), C.c_void_p(_ptr(isActiveBuffer)),
                                           C.c_void_p(_ptr(offsetsBuffer)), C.c_void_p(_ptr(outputBuffer)),
                                           C.c_void_p(_torch_stream())), self.ctx.handle)


class RadixSorter:
    """js/radix_sort_by_key.js."""

    def __init__(self, device=0):
        self.ctx = _ctx(device)

    @staticmethod
    def getAlignedSize(size: int) -> int:
        return int(_lib.load().bcmc_sort_aligned_size(int(size)))

    def sort(self, keys, values, size: int, reverse: bool):
        check(_lib.load().bcmc_sort_pairs_u32(self.ctx.handle, C.c_void_p(_ptr(keys)), C.c_void_p(_ptr(values)),
                                              int(size), 1 if reverse else 0, C.c_void_p(_torch_stream())),
              self.ctx.handle)


# ---- ZFP helpers on device buffers -------------------------------------------
def stream_words(dims, rate: int) -> int:
    return int(_lib.load().bcmc_zfp_stream_words(dims3(dims), int(rate)))


def zfp_encode(ctx: Context, field, rate: int):
    """Encodes a float32 CUDA tensor indexed [z, y, x] into a fixed-rate stream
    (int64 CUDA tensor of stream_words() words)."""
    t = _torch()
    f = field.contiguous()
    dims = (f.shape[2], f.shape[1], f.shape[0])
    words = t.empty(stream_words(dims, rate), dtype=t.int64, device=f.device)
    check(_lib.load().bcmc_zfp_encode(ctx.handle, C.c_void_p(f.data_ptr()), dims3(dims), int(rate),
                                      C.c_void_p(words.data_ptr()), C.c_void_p(_torch_stream())), ctx.handle)
    return words


def _check_stream(words, nblocks: int, rate: int):
    """The kernels read rate 64-bit words per block and take no length: refuse
    a device stream shorter than that before it reaches them."""
    have = int(words.numel()) * int(words.element_size()) if hasattr(words, "numel") else None
    if have is not None and have < int(nblocks) * int(rate) * 8:
        raise ValueError(f"compressed stream holds {have} bytes; {nblocks} blocks at rate {rate} need "
                         f"{int(nblocks) * int(rate) * 8}")


def zfp_decode_volume(ctx: Context, words, nblocks: int, rate: int):
    _check_stream(words, nblocks, rate)
    t = _torch()
    out = t.empty(nblocks * 64, dtype=t.float32, device="cuda")
    check(_lib.load().bcmc_zfp_decode_volume(ctx.handle, C.c_void_p(_ptr(words)), int(nblocks), int(rate),
                                             C.c_void_p(out.data_ptr()), C.c_void_p(_torch_stream())), ctx.handle)
    return out


def unpack_vertices(ctx: Context, vertices, dims, scale=(1.0, 1.0, 1.0), proj_view=None):
    """World-space positions of packed vertices (mc_isosurface.vert:51-60):
    float32 CUDA tensor [n, 3]; with proj_view (4x4, column-major order as the
    reference's gl-matrix uses) also the clip positions [n, 4]."""
    t = _torch()
    n = int(vertices.shape[0]) if hasattr(vertices, "shape") else 0
    world = t.empty((n, 3), dtype=t.float32, device="cuda")
    clip = t.empty((n, 4), dtype=t.float32, device="cuda") if proj_view is not None else None
    pv = None
    if proj_view is not None:
        m = np.ascontiguousarray(np.asarray(proj_view, dtype=np.float32).reshape(16))
        pv = m.ctypes.data_as(C.POINTER(C.c_float))
    check(_lib.load().bcmc_unpack_vertices(ctx.handle, C.c_void_p(_ptr(vertices) if n else 0), n, dims3(dims),
                                           scale3(scale), C.c_void_p(world.data_ptr()), pv,
                                           C.c_void_p(clip.data_ptr()) if clip is not None else None,
                                           C.c_void_p(_torch_stream())), ctx.handle)
    return (world, clip) if clip is not None else world


def render(ctx: Context, vertices, n: int, dims, proj_view, eye_pos, width: int, height: int, scale=(1.0, 1.0, 1.0),
           fog: bool = False, depth: bool = True, triangle: bool = True):
    """The reference's render pass (js/bcmc.js:174-190,237-265,377-391 with
    shaders/mc_isosurface.vert/.frag), headless: the first n packed vertices
    of `vertices` (a CUDA tensor, 2 x u32 each) drawn as triangles into a
    height x width image.  proj_view: 4x4 in column-major order (gl-matrix's
    layout); eye_pos: the camera position.  Returns (rgba [h, w, 4] float32,
    depth [h, w] float32 or None, triangle [h, w] int32 or None) as CUDA
    tensors; row 0 is the top of the image, background (1, 1, 1, 1), depth 1.0
    and triangle -1."""
    t = _torch()
    p = _lib.bcmc_render_params()
    p.width, p.height = int(width), int(height)
    m = np.asarray(proj_view, dtype=np.float32).reshape(16)
    for i in range(16):
        p.proj_view[i] = float(m[i])
    for i in range(3):
        p.eye_pos[i] = float(eye_pos[i])
    p.fog = 1 if fog else 0
    rgba = t.empty((height, width, 4), dtype=t.float32, device="cuda")
    dep = t.empty((height, width), dtype=t.float32, device="cuda") if depth else None
    tri = t.empty((height, width), dtype=t.int32, device="cuda") if triangle else None
    check(_lib.load().bcmc_render(ctx.handle, C.c_void_p(_ptr(vertices) if n else 0), int(n), dims3(dims),
                                  scale3(scale), C.byref(p), C.c_void_p(rgba.data_ptr()),
                                  C.c_void_p(dep.data_ptr()) if dep is not None else None,
                                  C.c_void_p(tri.data_ptr()) if tri is not None else None,
                                  C.c_void_p(_torch_stream())), ctx.handle)
    return rgba, dep, tri


def zfp_block_ranges(ctx: Context, words, dims, rate: int):
    t = _torch()
    nb = int(np.prod([(d + 3) // 4 for d in dims]))
    _check_stream(words, nb, rate)
    out = t.empty(2 * nb, dtype=t.float32, device="cuda")
    check(_lib.load().bcmc_zfp_block_ranges(ctx.handle, C.c_void_p(_ptr(words)), dims3(dims), int(rate),
                                            C.c_void_p(out.data_ptr()), C.c_void_p(_torch_stream())), ctx.handle)
    return out


def block_active(ctx: Context, ranges, dims, isovalue: float):
    t = _torch()
    nb = int(np.prod([(d + 3) // 4 for d in dims]))
    out = t.empty(nb, dtype=t.int32, device="cuda")
    _sync_torch()
    check(_lib.load().bcmc_block_active(ctx.handle, C.c_void_p(_ptr(ranges)), dims3(dims), float(isovalue),
                                        C.c_void_p(out.data_ptr()), None), ctx.handle)
    ctx.synchronize()
    return out


class Engine:
    """Batched isosurface queries over several resident compressed volumes
    with one shared pool of decoded-block slots (bcmc_engine_*).  Every query's
    vertices equal what CompressedMarchingCubes.computeSurface returns for it
    on its volume, bit for bit."""

    def __init__(self, device=0, pool_slots: int = 0, vertex_capacity: int = 0, max_batch: int = 0,
                 vertex_budget: int = 0):
        self.ctx = _ctx(device)
        o = _lib.bcmc_engine_opts(int(pool_slots), int(vertex_capacity), int(vertex_budget), int(max_batch), 0)
        h = C.c_void_p()
        check(_lib.load().bcmc_engine_create(self.ctx.handle, C.byref(o), C.byref(h)), self.ctx.handle)
        self._h = h
        self.volumes = []

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.load().bcmc_engine_destroy(self._h)
            self._h = None

    def addVolume(self, volume, compressionRate: int, volumeDims) -> int:
        ptr, nbytes, keep, on_dev = _host_bytes(volume)
        if on_dev:
            raise ValueError("Engine.addVolume takes the compressed stream in host memory")
        vid = C.c_uint32()
        check(_lib.load().bcmc_engine_add_volume(self._h, ptr, nbytes, int(compressionRate), dims3(volumeDims),
                                                 C.byref(vid)), self.ctx.handle)
        del keep
        self.volumes.append((tuple(int(d) for d in volumeDims), int(compressionRate)))
        return int(vid.value)

    def run(self, queries) -> np.ndarray:
        """queries: sequence of (volume id, isovalue).  Returns a structured
        array (vertex_offset, num_vertices, num_active_blocks) per query."""
        n = len(queries)
        qs = (_lib.bcmc_query * max(n, 1))()
        for i, (v, iso) in enumerate(queries):
            qs[i].volume = int(v)
            qs[i].isovalue = float(iso)
        res = (_lib.bcmc_query_result * max(n, 1))()
        check(_lib.load().bcmc_engine_run(self._h, qs, n, res), self.ctx.handle)
        out = np.zeros(n, dtype=[("vertex_offset", "<u8"), ("num_vertices", "<u4"), ("num_active_blocks", "<u4")])
        for i in range(n):
            out[i] = (res[i].vertex_offset, res[i].num_vertices, res[i].num_active_blocks)
        return out

    def autotune(self, queries) -> dict:
        """Chooses the launch parameters for the batch-size bucket of these
        queries by timing them (bcmc_engine_autotune)."""
        n = len(queries)
        qs = (_lib.bcmc_query * max(n, 1))()
        for i, (v, iso) in enumerate(queries):
            qs[i].volume = int(v)
            qs[i].isovalue = float(iso)
        rep = _lib.bcmc_tune_report()
        check(_lib.load().bcmc_engine_autotune(self._h, qs, n, C.byref(rep)), self.ctx.handle)
        return {k: getattr(rep, k) for k, _ in _lib.bcmc_tune_report._fields_}

    def set_tuning(self, report: dict):
        """Applies a tune report (as autotune returns it) to its bucket
        (bcmc_engine_set_tuning)."""
        rep = _lib.bcmc_tune_report()
        for k, _ in _lib.bcmc_tune_report._fields_:
            if k in report:
                setattr(rep, k, report[k])
        check(_lib.load().bcmc_engine_set_tuning(self._h, C.byref(rep)), self.ctx.handle)

    def force_config(self, n: int, **params):
        """The default launch parameters of n queries' bucket with `params`
        changed (the tune report's field names), applied by set_tuning."""
        b = 1
        while b < n:
            b <<= 1
        cfg = {"bucket": b, "act_ctas_per_sm": 8, "decode_threads": 128, "decode_ctas_per_sm": 16,
               "mc_ctas_per_sm": 6, "mc_blocks_per_tile": 16}
        cfg.update(params)
        self.set_tuning(cfg)

    def run_admit(self, queries):
        """Runs the longest prefix of `queries` that the slot pool and the
        vertex budget admit; returns (results of that prefix, its length)."""
        n = len(queries)
        qs = (_lib.bcmc_query * max(n, 1))()
        for i, (v, iso) in enumerate(queries):
            qs[i].volume = int(v)
            qs[i].isovalue = float(iso)
        res = (_lib.bcmc_query_result * max(n, 1))()
        adm = C.c_uint32()
        check(_lib.load().bcmc_engine_run_admit(self._h, qs, n, res, C.byref(adm)), self.ctx.handle)
        m = int(adm.value)
        out = np.zeros(m, dtype=[("vertex_offset", "<u8"), ("num_vertices", "<u4"), ("num_active_blocks", "<u4")])
        for i in range(m):
            out[i] = (res[i].vertex_offset, res[i].num_vertices, res[i].num_active_blocks)
        return out, m

    @property
    def vertexBuffer(self) -> DeviceArray:
        p = C.c_void_p()
        cnt = C.c_uint64()
        check(_lib.load().bcmc_engine_vertices(self._h, C.byref(p), C.byref(cnt)), self.ctx.handle)
        return DeviceArray(p.value, (int(cnt.value), 2), "<u4", self)

    def copyVertices(self, first: int = 0, count: int | None = None, out: np.ndarray | None = None) -> np.ndarray:
        if count is None:
            p = C.c_void_p()
            cnt = C.c_uint64()
            check(_lib.load().bcmc_engine_vertices(self._h, C.byref(p), C.byref(cnt)), self.ctx.handle)
            count = int(cnt.value) - int(first)
        if out is None:
            out = np.empty((count, 2), dtype=np.uint32)
        check(_lib.load().bcmc_engine_copy_vertices(self._h, int(first), int(count), out.ctypes.data_as(C.c_void_p)),
              self.ctx.handle)
        return out[:count]

    def stats(self) -> dict:
        st = _lib.bcmc_engine_stats()
        check(_lib.load().bcmc_engine_stats_get(self._h, C.byref(st)), self.ctx.handle)
        return {k: getattr(st, k) for k, _ in _lib.bcmc_engine_stats._fields_}


class Server:
    """Continuous-batching isosurface server over an Engine (bcmc_server_*).
    While it exists only the server uses the engine."""

    def __init__(self, engine: Engine, max_batch: int = 0, max_wait_us: int = 0):
        self.engine = engine
        o = _lib.bcmc_server_opts(int(max_batch), int(max_wait_us))
        h = C.c_void_p()
        check(_lib.load().bcmc_server_create(engine._h, C.byref(o), C.byref(h)), engine.ctx.handle)
        self._h = h
        self._bufs = {}

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().bcmc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def submit(self, volume: int, isovalue: float, max_vertices: int = 0) -> int:
        """Queues a request; with max_vertices > 0 its vertices are copied to
        a host array returned by wait()."""
        t = C.c_uint64()
        buf = np.empty((max_vertices, 2), dtype=np.uint32) if max_vertices else None
        ptr = buf.ctypes.data_as(C.c_void_p) if buf is not None else None
        check(_lib.load().bcmc_server_submit(self._h, int(volume), float(isovalue), ptr, int(max_vertices),
                                             C.byref(t)), self.engine.ctx.handle)
        self._bufs[int(t.value)] = buf
        return int(t.value)

    def wait(self, ticket: int):
        """(num_vertices, num_active_blocks, latency_ms, vertices or None)."""
        r = _lib.bcmc_query_result()
        lat = C.c_double()
        check(_lib.load().bcmc_server_wait(self._h, int(ticket), C.byref(r), C.byref(lat)), self.engine.ctx.handle)
        buf = self._bufs.pop(int(ticket), None)
        n = int(r.num_vertices)
        return n, int(r.num_active_blocks), float(lat.value), (buf[: min(n, len(buf))] if buf is not None else None)

    def run_load(self, rate_qps: float, requests: int, volumes, weights, iso_lo, iso_hi, seed: int = 0) -> dict:
        nv = len(volumes)
        v = (C.c_uint32 * nv)(*[int(x) for x in volumes])
        w = (C.c_float * nv)(*[float(x) for x in weights])
        lo = (C.c_float * nv)(*[float(x) for x in iso_lo])
        hi = (C.c_float * nv)(*[float(x) for x in iso_hi])
        spec = _lib.bcmc_load_spec(float(rate_qps), int(requests), nv, int(seed), v, w, lo, hi)
        rep = _lib.bcmc_load_report()
        check(_lib.load().bcmc_server_run_load(self._h, C.byref(spec), C.byref(rep)), self.engine.ctx.handle)
        return {k: getattr(rep, k) for k, _ in _lib.bcmc_load_report._fields_}
