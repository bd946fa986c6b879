"""Full-size workloads, checked through properties that do not need the
oracle to run the whole workload:

* 512^3 spectral field, rate 2, cache 25 %, a 64-isovalue random walk: every
  query against the oracle (vertices, statistics, LRU slot arrays and
  cachedItemSlots), then every query of the walk through the batched engine,
  which must agree with the plain path bit for bit.
* 1024x1024x1080 at rate 4 (17,694,720 blocks): block bit offsets pass 2^32
  (block 2^24 and beyond), where the reference's u32 offset would wrap; the
  decoder must follow the 64-bit offset -- checked block by block against the
  oracle's decoder on a random stream, with the full-volume decode and the
  block ranges -- and queries on the CT-like volume of that size must agree
  between the plain path and the engine, and one of them with the oracle
  (vertices, statistics and LRU state)."""
import numpy as np
import pytest

import bcmc
from bcmc import datasets as D

pytestmark = pytest.mark.gpu


def _encode_on_gpu(ctx, field_dev, rate, dims):
    import torch

    words = bcmc.zfp_encode(ctx, field_dev, rate)
    torch.cuda.synchronize()
    nb = int(np.prod([(d + 3) // 4 for d in dims]))
    host = words.cpu().numpy().view(np.uint64)
    return words, host, host.view(np.uint8)[: nb * 8 * rate].copy()


def test_spectral512_random_walk(ctx, oracle):
    import torch

    dims, rate = (512, 512, 512), 2
    field = D.turbulence(dims, 3)
    _, words, stream = _encode_on_gpu(ctx, torch.from_numpy(field).cuda(), rate, dims)
    del field
    isos = [float(np.float32(v)) for v in D.random_walk(64, 3)]
    ref = oracle.CompressedMarchingCubes(words, rate, dims, initial_cache_fraction=0.25)
    c = bcmc.Context(ctx.device, initial_cache_fraction=0.25)
    mc = bcmc.CompressedMarchingCubes(c)
    mc.setCompressedVolume(stream, rate, dims)
    plain = []
    for qi, iso in enumerate(isos):
        n = mc.computeSurface(iso)
        verts = mc.copyVertices().copy()
        plain.append((n, verts))
        n_ref = ref.compute_surface(iso)
        assert n == n_ref and n > 0, (qi, n, n_ref)
        assert np.array_equal(verts, ref.vertices_view(n_ref)), qi
        st, rs = mc.stats(), ref.stats()
        for k in ("numActiveBlocks", "newDecompressed", "numBlocksWithVertices", "cacheSize"):
            assert st[k] == rs[k], (qi, k)
        g, r = mc.lruCache.state(), ref.lru_state()
        for k in ("item_slots", "age", "avail", "item"):
            assert np.array_equal(g[k], r[k]), (qi, k)
    del ref
    eng = bcmc.Engine(ctx)
    vid = eng.addVolume(stream, rate, dims)
    for first in range(0, 64, 16):
        res = eng.run([(vid, iso) for iso in isos[first: first + 16]])
        allv = eng.copyVertices()
        for i, r in enumerate(res):
            n, verts = plain[first + i]
            assert int(r["num_vertices"]) == n, first + i
            off = int(r["vertex_offset"])
            assert np.array_equal(allv[off: off + n], verts), first + i


BIG_DIMS = (1024, 1024, 1080)
BIG_BLOCKS = 256 * 256 * 270  # 17,694,720


def test_1024x1024x1080_block_offsets_past_2_24(ctx, oracle):
    """Random 32-byte blocks (rate 4): every bit pattern is a valid block."""
    import torch

    rate, max_bits = 4, 256
    assert BIG_BLOCKS > (1 << 24)
    g = torch.Generator(device="cuda").manual_seed(11)
    # rate 4: 256 bits = 4 words per block, plus the word the reader may fetch past the end
    nwords = BIG_BLOCKS * max_bits // 64 + 2
    words = torch.randint(-(1 << 63), (1 << 63) - 1, (nwords,), dtype=torch.int64, device="cuda", generator=g)
    assert words.numel() * 64 >= BIG_BLOCKS * max_bits + 64
    host = words.cpu().numpy().view(np.uint64)
    dec = bcmc.zfp_decode_volume(ctx, words, BIG_BLOCKS, rate)
    ranges = bcmc.zfp_block_ranges(ctx, words, BIG_DIMS, rate)
    torch.cuda.synchronize()
    sample = list(range((1 << 24) - 64, (1 << 24) + 64)) + list(range(BIG_BLOCKS - 64, BIG_BLOCKS)) + \
        [int(b) for b in np.random.default_rng(4).integers(0, BIG_BLOCKS, 128)]
    idx = torch.tensor(sample, dtype=torch.int64, device="cuda")
    got = dec.view(BIG_BLOCKS, 64)[idx].cpu().numpy()
    got_r = ranges.view(BIG_BLOCKS, 2)[idx].cpu().numpy()
    for i, b in enumerate(sample):
        want = oracle.decode_block(host, b, max_bits)
        assert np.array_equal(got[i].view(np.uint32), want.view(np.uint32)), b
        # all blocks of this volume are whole (dims multiples of 4): the range folds the 64
        # values in block order into (1e20, -1e20) with GLSL min/max
        # (zfp_compute_block_range.comp:47-59)
        lo, hi = np.float32(1e20), np.float32(-1e20)
        for v in want:
            lo = v if v < lo else lo
            hi = v if hi < v else hi
        assert np.array_equal(got_r[i].view(np.uint32), np.array([lo, hi], np.float32).view(np.uint32)), b
        if b >= (1 << 24):  # where the reference's u32 offset wraps
            wrapped = oracle.decode_block(host, b, max_bits, emulate_u32_offset=True)
            assert not np.array_equal(wrapped.view(np.uint32), want.view(np.uint32)) or not want.any(), b


def test_1024x1024x1080_query_plain_equals_engine_and_oracle(ctx, oracle):
    import torch

    rate = 4
    field = D.ct_uint16_torch(BIG_DIMS, 5)
    _, words, stream = _encode_on_gpu(ctx, field, rate, BIG_DIMS)
    del field
    torch.cuda.empty_cache()
    c = bcmc.Context(ctx.device, initial_cache_fraction=0.1)
    mc = bcmc.CompressedMarchingCubes(c)
    mc.setCompressedVolume(stream, rate, BIG_DIMS)
    eng = bcmc.Engine(ctx)
    vid = eng.addVolume(stream, rate, BIG_DIMS)
    ref = oracle.CompressedMarchingCubes(words, rate, BIG_DIMS, initial_cache_fraction=0.1)
    for qi, iso in enumerate((2500.0, 3600.0)):
        n = mc.computeSurface(iso)
        assert n > 0
        res = eng.run([(vid, iso)])
        assert int(res[0]["num_vertices"]) == n
        a = mc.vertexBuffer.torch()[:n]
        off = int(res[0]["vertex_offset"])
        b = eng.vertexBuffer.torch()[off: off + n]
        assert torch.equal(a, b), iso
        del a, b
        if qi == 0:  # the oracle runs the first query (some 7 M active blocks)
            n_ref = ref.compute_surface(iso)
            assert n == n_ref, (iso, n, n_ref)
            assert np.array_equal(mc.copyVertices(), ref.vertices_view(n_ref)), iso
            st, rs = mc.stats(), ref.stats()
            for k in ("numActiveBlocks", "newDecompressed", "numBlocksWithVertices", "cacheSize"):
                assert st[k] == rs[k], (iso, k)
            g, r = mc.lruCache.state(), ref.lru_state()
            for k in ("item_slots", "age", "avail", "item"):
                assert np.array_equal(g[k], r[k]), (iso, k)
            del ref
