"""The CUDA path against the reference's own shaders, through the golden
fixtures in tests/golden/ (generated by tests/golden/make_golden.py from the
reference's compute shaders compiled as host C++).  Integer/bit data: exact."""
import glob
import os

import numpy as np
import pytest

import bcmc
from gpu_util import bits, to_dev

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MC_FILES = sorted(glob.glob(os.path.join(GOLDEN, "mc_*.npz")))
DECODE_FILES = sorted(glob.glob(os.path.join(GOLDEN, "decode_rate*.npz")))


@pytest.mark.parametrize("path", DECODE_FILES, ids=os.path.basename)
def test_decoder_matches_reference_shader(ctx, path):
    g = np.load(path)
    rate, words, want = int(g["rate"]), g["words"], g["decoded_bits"]
    out = bcmc.zfp_decode_volume(ctx, to_dev(words), want.shape[0], rate)
    got = out.cpu().numpy().view(np.uint32).reshape(want.shape)
    assert np.array_equal(got, want)


def _stream_bytes(g):
    dims = [int(d) for d in g["dims"]]
    nb = int(np.prod([(d + 3) // 4 for d in dims]))
    return g["words"].view(np.uint8)[: nb * 64 * int(g["rate"]) // 8]


@pytest.mark.parametrize("path", MC_FILES, ids=os.path.basename)
@pytest.mark.parametrize("cache_fraction", [1.0, 0.05])
def test_pipeline_matches_reference_shaders(ctx, path, cache_fraction):
    g = np.load(path)
    rate, dims = int(g["rate"]), tuple(int(d) for d in g["dims"])
    c = bcmc.Context(ctx.device, initial_cache_fraction=cache_fraction)
    mc = bcmc.CompressedMarchingCubes(c)
    mc.setCompressedVolume(_stream_bytes(g), rate, dims)
    assert np.array_equal(bits(mc.views()["ranges"].numpy()), bits(g["ranges"].reshape(-1)))
    for i, iso in enumerate(g["isos"]):
        n = mc.computeSurface(float(iso))
        assert n == len(g[f"vertices_{i}"]), (i, iso)
        assert np.array_equal(mc.copyVertices(), g[f"vertices_{i}"]), (i, iso)
        v = mc.views()
        assert np.array_equal(v["active"].numpy(), g[f"active_{i}"])
        if n:
            assert np.array_equal(v["active_ids"].numpy(), g[f"active_ids_{i}"])
            assert np.array_equal(v["with_verts"].numpy(), g[f"with_verts_{i}"])
            assert np.array_equal(v["vert_offsets"].numpy(), g[f"vert_offsets_{i}"])


def test_full_ranges_flag(ctx, oracle):
    """BCMC_FLAG_FULL_RANGES ranges every block, including the ones the reference
    leaves at zero when (x/4)*(y/4) is not a multiple of 4 (44x40x36: 11*10)."""
    g = np.load(os.path.join(GOLDEN, "mc_ct44_r4.npz"))
    rate, dims = int(g["rate"]), tuple(int(d) for d in g["dims"])
    nbx, nby, nbz = ((d + 3) // 4 for d in dims)
    ref_count = (4 * nbx * 4 * nby) // 64 * (4 * nbz)
    assert ref_count < nbx * nby * nbz
    assert not g["ranges"][ref_count:].any()  # the reference's zeros
    dec = oracle.decode_volume(g["words"], nbx * nby * nbz, 64 * rate).reshape(nbz, nby, nbx, 4, 4, 4)
    want = np.zeros((nbz, nby, nbx, 2), np.float32)
    for bz in range(nbz):
        for by in range(nby):
            for bx in range(nbx):
                blk = dec[bz, by, bx][: min(4, dims[2] - 4 * bz), : min(4, dims[1] - 4 * by),
                                       : min(4, dims[0] - 4 * bx)]
                want[bz, by, bx] = (blk.min(), blk.max())
    c = bcmc.Context(ctx.device, initial_cache_fraction=1.0, flags=bcmc.Context.FULL_RANGES)
    mc = bcmc.CompressedMarchingCubes(c)
    mc.setCompressedVolume(_stream_bytes(g), rate, dims)
    got = mc.views()["ranges"].numpy().reshape(-1, 2)
    assert np.array_equal(bits(got), bits(want.reshape(-1, 2)))
    assert np.array_equal(bits(got[:ref_count]), bits(g["ranges"][:ref_count]))


def test_unpack_matches_reference_vertex_stage(ctx):
    import torch

    g = np.load(os.path.join(GOLDEN, "unpack_ct44.npz"))
    verts = torch.from_numpy(g["vertices"].view(np.int32).copy()).cuda()
    world, clip = bcmc.unpack_vertices(ctx, verts, tuple(int(d) for d in g["dims"]), tuple(g["scale"]), g["proj"])
    assert np.array_equal(world.cpu().numpy().view(np.uint32), g["world_bits"])
    assert np.array_equal(clip.cpu().numpy().view(np.uint32), g["clip_bits"])
    w2 = bcmc.unpack_vertices(ctx, verts, tuple(int(d) for d in g["dims"]), tuple(g["scale"]))
    assert np.array_equal(w2.cpu().numpy().view(np.uint32), g["world_bits"])


def test_sort_matches_reference_shaders(ctx):
    from gpu_util import to_host

    g = np.load(os.path.join(GOLDEN, "sort.npz"))
    for i in range(int(g["cases"])):
        k, v = g[f"keys_{i}"], g[f"values_{i}"]
        for rev, want in ((False, g[f"asc_{i}"]), (True, g[f"desc_{i}"])):
            kd, vd = to_dev(k), to_dev(v)
            bcmc.RadixSorter(ctx).sort(kd, vd, len(k), rev)
            assert np.array_equal(to_host(vd, np.uint32), want), (i, rev)


# ---- scan, compaction and the LRU cache against the reference's shaders ----

import golden_lru as GL  # noqa: E402


def test_scan_and_compaction_match_reference_shaders(ctx):
    import torch

    from gpu_util import to_host

    pipe = bcmc.ExclusiveScanPipeline(ctx)
    sc = bcmc.StreamCompact(ctx)
    for n, v, g, i in GL.scan_cases():
        s = pipe.prepareInput(v)
        total = s.scan(n)
        GL.check_scan(g, i, n, to_host(s.inputBuf, np.uint32), total)
        flags = (v != 0).astype(np.uint32)
        fs = pipe.prepareInput(flags)
        m = fs.scan(n)
        out = torch.zeros(max(m, 1), dtype=torch.int32, device="cuda")
        sc.compactActiveIDs(n, to_dev(flags), fs.inputBuf, out)
        GL.check_compact(g, i, n, to_host(out, np.uint32)[:m])


@pytest.mark.parametrize("seq", range(3))
def test_lru_matches_reference_shaders(ctx, seq):
    total, initial, steps, reset_at, recs = list(GL.lru_sequences())[seq]
    c = bcmc.LRUCache(ctx, None, None, initial, 256, total)
    for step, rec in enumerate(recs):
        if step == reset_at:
            c.reset()
        n, ids = c.update(to_dev(rec["needed"]))
        assert n == len(rec["new"]), step
        if n:
            assert np.array_equal(ids.numpy(), rec["new"]), step
            assert c.displayNumSlotsAvailable == rec["display"], step
        assert c.cacheSize == rec["cache_size"], step
        GL.check_lru_state(rec, c.state(), step)


def test_pipeline_lru_matches_reference_shaders(ctx):
    """computeSurface sequences with the cache in the loop: per query the
    counts, the mesh and the LRU's slot arrays and cachedItemSlots."""
    for name, frac, isos, reset_at, recs in GL.lru_pipeline_cases():
        g = np.load(os.path.join(GOLDEN, f"mc_{name}.npz"))
        c = bcmc.Context(ctx.device, initial_cache_fraction=frac)
        mc = bcmc.CompressedMarchingCubes(c)
        mc.setCompressedVolume(_stream_bytes(g), int(g["rate"]), tuple(int(d) for d in g["dims"]))
        for qi, (iso, rec) in enumerate(zip(isos, recs)):
            if qi == reset_at:
                mc.lruCache.reset()
            n = mc.computeSurface(float(iso))
            nverts, n_active, n_new, n_with = rec["counts"]
            assert n == nverts, (name, qi)
            if n_active:
                st = mc.stats()
                assert (st["numActiveBlocks"], st["newDecompressed"], st["numBlocksWithVertices"]) == \
                    (n_active, n_new, n_with), (name, qi)
            assert GL.sha(mc.copyVertices().reshape(-1)) == rec["mesh_sha"], (name, qi)
            GL.check_lru_state(rec, mc.lruCache.state(), (name, qi))
