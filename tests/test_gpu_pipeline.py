"""CompressedMarchingCubes on the GPU vs the oracle's plain one-query-at-a-time
pipeline: every query's vertex buffer bit for bit, plus ranges, active flags,
active/with-vertex block lists, vertex offsets, cache state and statistics."""
import numpy as np
import pytest

import bcmc
from bcmc import datasets as D
from gpu_util import bits

pytestmark = pytest.mark.gpu


def _run(ctx, oracle, field, dims, rate, isos, cache_fraction, check_state=True, reset_at=None):
    w = oracle.zfp_encode(field, rate)
    ref = oracle.CompressedMarchingCubes(w, rate, dims, initial_cache_fraction=cache_fraction)
    c = bcmc.Context(ctx.device, initial_cache_fraction=cache_fraction)
    mc = bcmc.CompressedMarchingCubes(c)
    mc.setCompressedVolume(w.view(np.uint8)[: (int(np.prod(oracle.padded_blocks(dims))) * 64 * rate + 7) // 8],
                           rate, dims)
    v = mc.views()
    assert np.array_equal(bits(v["ranges"].numpy()), bits(ref.ranges()))
    for qi, iso in enumerate(isos):
        if reset_at is not None and qi == reset_at:
            mc.lruCache.reset()
            ref.cache_reset()
        n_ref = ref.compute_surface(float(iso))
        n = mc.computeSurface(float(iso))
        assert n == n_ref, (qi, iso)
        got = mc.copyVertices()
        assert np.array_equal(got, ref.vertices(n_ref)), (qi, iso)
        st, rs = mc.stats(), ref.stats()
        for k in ("numActiveBlocks", "newDecompressed", "numBlocksWithVertices", "numVertices", "cacheSize"):
            assert st[k] == rs[k], (qi, k, st[k], rs[k])
        if check_state:
            v = mc.views()
            assert np.array_equal(v["active"].numpy(), ref.active())
            if rs["numActiveBlocks"] and n_ref:
                assert np.array_equal(v["active_ids"].numpy(), ref.active_ids(rs["numActiveBlocks"]))
                assert np.array_equal(v["with_verts"].numpy(), ref.with_verts(rs["numBlocksWithVertices"]))
                assert np.array_equal(v["vert_offsets"].numpy(), ref.vert_offsets(rs["numBlocksWithVertices"]))
            g = mc.lruCache.state()
            r = ref.lru_state()
            assert g["cache_size"] == r["cache_size"]
            for k in ("item_slots", "age", "avail", "item"):
                assert np.array_equal(g[k], r[k]), (qi, k)
    return mc, ref


def test_blobs64_single_query(ctx, oracle):
    """64^3 Gaussian blobs, rate 8, iso 0.5, cache large enough for all blocks."""
    f = D.blobs((64, 64, 64), 1)
    mc, _ = _run(ctx, oracle, f, (64, 64, 64), 8, [0.5], 1.0)
    assert mc.numVertices > 0


def test_blobs64_sweep_small_cache(ctx, oracle):
    f = D.blobs((64, 64, 64), 1)
    isos = list(np.linspace(0.1, 1.0, 12)) + [5.0, 0.5, -1.0, 0.5]
    _run(ctx, oracle, f, (64, 64, 64), 8, isos, 0.05, reset_at=9)


@pytest.mark.parametrize("dims", [(61, 47, 53), (17, 5, 33), (4, 4, 4), (5, 5, 5)])
def test_partial_blocks(ctx, oracle, dims):
    f = D.blobs(dims, 8, n_blobs=5)
    isos = np.linspace(float(f.min()), float(f.max()), 7)
    _run(ctx, oracle, f, dims, 4, isos, 0.05)


def test_ct_like_96(ctx, oracle):
    f = D.ct_like((96, 96, 96), 2)
    _run(ctx, oracle, f, (96, 96, 96), 4, np.linspace(30.0, 220.0, 16), 0.5)


def test_turbulence_random_walk(ctx, oracle):
    f = D.turbulence((64, 64, 64), 3)
    _run(ctx, oracle, f, (64, 64, 64), 2, D.random_walk(24, 3), 0.25)


def test_ct256_config(ctx, oracle):
    """The 256^3 CT-like configuration: rate 4, 16 isovalues in [30, 220],
    cache 50 % of the blocks."""
    f = D.ct_like((256, 256, 256), 2)
    _run(ctx, oracle, f, (256, 256, 256), 4, np.linspace(30.0, 220.0, 16), 0.5, check_state=False)


def test_rows_wider_than_the_staged_active_test(ctx, oracle):
    """24,600 voxels in x (6,150 blocks per row): the active test's shared-memory
    windows would exceed 48 KB, so the row-load kernel runs instead."""
    dims = (24600, 8, 4)
    f = D.blobs(dims, 9, n_blobs=40)
    isos = np.linspace(float(f.min()), float(f.max()), 5)[1:-1]
    _run(ctx, oracle, f, dims, 4, isos, 0.5)


def test_empty_and_full_queries(ctx, oracle):
    f = D.blobs((32, 32, 32), 4)
    _run(ctx, oracle, f, (32, 32, 32), 4, [1e9, -1e9, float(np.median(f)), 1e9], 0.05)


def test_perf_tracker_and_memory_report(ctx, oracle):
    f = D.blobs((32, 32, 32), 4)
    w = oracle.zfp_encode(f, 4)
    mc = bcmc.CompressedMarchingCubes(ctx)
    mc.setCompressedVolume(w, 4, (32, 32, 32))
    perf = {}
    for iso in (float(np.median(f)), float(f.max()) + 1):
        mc.computeSurface(iso, perf)
    assert len(perf["computeVertices"]) == 2 and perf["totalBlocks"] == 512
    mc_text, cache_text, total, use = mc.reportMemoryUse()
    assert "compressedData" in mc_text and "cache" in cache_text and use["cache"]["cache"] > 0


def test_surface_straight_to_host(ctx, oracle):
    """computeSurfaceToHost gives the same vertices as computeSurface +
    copyVertices, refuses a buffer that is too small (reporting the size
    needed) and pageable memory, and leaves the cache state as a normal query."""
    import torch

    dims = (64, 64, 64)
    f = D.blobs(dims, 1)
    w = oracle.zfp_encode(f, 8)
    stream = w.view(np.uint8)[: 4096 * 64].copy()
    a = bcmc.CompressedMarchingCubes(bcmc.Context(ctx.device, initial_cache_fraction=0.3))
    a.setCompressedVolume(stream, 8, dims)
    b = bcmc.CompressedMarchingCubes(bcmc.Context(ctx.device, initial_cache_fraction=0.3))
    b.setCompressedVolume(stream, 8, dims)
    pinned = torch.empty((1 << 20, 2), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    for iso in (0.5, 0.3, 0.9, 5.0, 0.5):
        n = a.computeSurface(iso)
        want = a.copyVertices().copy()
        m = b.computeSurfaceToHost(iso, pinned)
        assert m == n
        assert np.array_equal(pinned[:m], want), iso
        assert a.stats() == b.stats()
        assert np.array_equal(a.lruCache.state()["item_slots"], b.lruCache.state()["item_slots"])
    with pytest.raises(bcmc.BcmcError):
        b.vertexBuffer  # noqa: B018 -- the last query went to host memory
    # a buffer 8-byte aligned but off every 256-byte boundary (the kernel
    # aligns each warp's stores to 256-byte windows of the host buffer)
    for off in (1, 5, 31):
        n = a.computeSurface(0.42)
        m = b.computeSurfaceToHost(0.42, pinned[off:])
        assert m == n and np.array_equal(pinned[off:off + m], a.copyVertices()), off
    n = a.computeSurface(0.5)
    small = pinned[:10]
    with pytest.raises(bcmc.BcmcError):
        b.computeSurfaceToHost(0.5, small)
    with pytest.raises(bcmc.BcmcError):
        b.computeSurfaceToHost(0.5, np.zeros((n, 2), np.uint32))  # pageable
    assert b.computeSurface(0.5) == n and np.array_equal(b.copyVertices(), a.copyVertices())


def test_surface_sequence_to_host(ctx, oracle):
    """computeSurfacesToHost: the same vertices, counts and cache state as one
    computeSurface per isovalue, the queries back to back in one buffer, with
    queries that grow the vertex buffers mid-sequence; a buffer that runs out
    of room stops the sequence at that query (its count reported, the cache
    advanced through it); the device buffer afterwards holds the last query."""
    import torch

    dims = (64, 64, 64)
    f = D.blobs(dims, 2)
    w = oracle.zfp_encode(f, 8)
    stream = w.view(np.uint8)[: 4096 * 64].copy()
    isos = [0.9, 0.5, 0.3, 5.0, 0.2, 0.5, 0.7, 0.25, 0.6]

    def fresh():
        m = bcmc.CompressedMarchingCubes(bcmc.Context(ctx.device, initial_cache_fraction=0.2))
        m.setCompressedVolume(stream, 8, dims)
        return m

    a, b = fresh(), fresh()
    want, counts = [], []
    for iso in isos:
        counts.append(a.computeSurface(iso))
        want.append(a.copyVertices().copy())
    pinned = torch.empty((sum(counts) + 7, 2), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    got = b.computeSurfacesToHost(isos, pinned)
    assert got == counts
    off = 0
    for n, v in zip(counts, want):
        assert np.array_equal(pinned[off:off + n], v)
        off += n
    assert a.stats() == b.stats()
    assert np.array_equal(a.lruCache.state()["item_slots"], b.lruCache.state()["item_slots"])
    assert np.array_equal(b.copyVertices(), want[-1])
    # the next plain query on either buffer
    assert b.computeSurface(0.45) == a.computeSurface(0.45)
    assert np.array_equal(b.copyVertices(), a.copyVertices())
    # too small: stops at the first query that does not fit
    c, d = fresh(), fresh()
    room = counts[0] + counts[1] + counts[2] // 2
    with pytest.raises(bcmc.BcmcError):
        c.computeSurfacesToHost(isos, pinned[:room])
    for iso in isos[:3]:
        d.computeSurface(iso)
    assert c.stats() == d.stats()
    assert np.array_equal(c.lruCache.state()["item_slots"], d.lruCache.state()["item_slots"])
    with pytest.raises(bcmc.BcmcError):
        c.computeSurfacesToHost(isos, np.zeros((16, 2), np.uint32))  # pageable
    assert c.computeSurfacesToHost([], pinned) == []
