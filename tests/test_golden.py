"""The CPU oracle against the reference's own shaders.

* Golden fixtures (tests/golden/*.npz, generated by tests/golden/make_golden.py
  from the reference's compute shaders compiled as host C++): decode of random
  bit streams at six rates, and full queries (ranges, active flags, active ids,
  blocks with vertices, vertex offsets, packed vertices) on five volumes.
* Scan and compaction outputs, LRU update sequences (new ids, slot arrays,
  cachedItemSlots after every update) and query sequences with the LRU cache
  in the loop, from the reference's scan, compaction, sort and LRU shaders
  driven the way js/exclusive_scan.js, js/stream_compact.js and
  js/lru_cache.js drive them.
* When the reference checkout is present, the same comparison live on further
  seeded cases (oracle/_ref built by oracle/ref_build.py).

Everything is integer/bit data: compared exactly.
"""
import glob
import os

import numpy as np
import pytest

import golden_lru as GL

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MC_FILES = sorted(glob.glob(os.path.join(GOLDEN, "mc_*.npz")))
DECODE_FILES = sorted(glob.glob(os.path.join(GOLDEN, "decode_rate*.npz")))


def test_fixtures_present():
    assert len(MC_FILES) >= 5 and len(DECODE_FILES) >= 6


@pytest.mark.parametrize("path", DECODE_FILES, ids=os.path.basename)
def test_oracle_decoder_matches_reference_shader(oracle, path):
    g = np.load(path)
    rate, words = int(g["rate"]), g["words"]
    want = g["decoded_bits"]
    for b in range(want.shape[0]):
        got = oracle.decode_block(words, b, 64 * rate)
        assert np.array_equal(np.asarray(got, np.float32).view(np.uint32), want[b]), b
        emu = oracle.decode_block(words, b, 64 * rate, native=True)
        assert np.array_equal(np.asarray(emu, np.float32).view(np.uint32), want[b]), b


def check_mc_against_golden(m, g, i, n):
    """m: an object with the oracle's CompressedMarchingCubes accessors."""
    s = m.stats()
    assert np.array_equal(m.active(), g[f"active_{i}"])
    assert np.array_equal(m.active_ids(s["numActiveBlocks"]), g[f"active_ids_{i}"])
    assert np.array_equal(m.with_verts(s["numBlocksWithVertices"]), g[f"with_verts_{i}"])
    assert np.array_equal(m.vert_offsets(s["numBlocksWithVertices"]), g[f"vert_offsets_{i}"])
    assert n == len(g[f"vertices_{i}"])
    assert np.array_equal(m.vertices(n), g[f"vertices_{i}"])


@pytest.mark.parametrize("path", MC_FILES, ids=os.path.basename)
@pytest.mark.parametrize("cache_fraction", [1.0, 0.05])
def test_oracle_pipeline_matches_reference_shaders(oracle, path, cache_fraction):
    g = np.load(path)
    rate, dims = int(g["rate"]), tuple(int(d) for d in g["dims"])
    m = oracle.CompressedMarchingCubes(g["words"], rate, dims, initial_cache_fraction=cache_fraction)
    assert np.array_equal(m.ranges().view(np.uint32), g["ranges"].reshape(-1).view(np.uint32))
    for i, iso in enumerate(g["isos"]):
        n = m.compute_surface(float(iso))
        check_mc_against_golden(m, g, i, n)


def _ref():
    import ref

    if not ref.available():
        pytest.skip("reference checkout not present: live shader comparison skipped")
    return ref


@pytest.mark.parametrize("kind,dims,seed,rate,isos", [
    ("blobs", (20, 28, 24), 11, 8, [0.4, 0.9]),
    ("ct_like", (33, 29, 27), 12, 3, [45.0, 200.0]),
    ("turbulence", (20, 20, 20), 13, 1, [-0.2, 0.1]),
    ("ct_uint16", (25, 22, 19), 14, 6, [300.0]),
])
def test_oracle_matches_reference_shaders_live(oracle, kind, dims, seed, rate, isos):
    R = _ref()
    from bcmc import datasets as D

    f = D.make_field(kind, dims, seed)
    words = oracle.zfp_encode(f, rate)
    nb = int(np.prod([(d + 3) // 4 for d in dims]))
    ids = np.arange(nb, dtype=np.uint32)
    dec_ref = R.decode_blocks(words, rate, ids, ids.astype(np.int32), nb)
    dec = oracle.decode_volume(words, nb, 64 * rate).reshape(nb, 64)
    assert np.array_equal(dec.view(np.uint32), dec_ref.view(np.uint32))
    m = oracle.CompressedMarchingCubes(words, rate, dims, initial_cache_fraction=0.3)
    for iso in isos:
        s = R.surface(words, rate, dims, float(iso))
        n = m.compute_surface(float(iso))
        assert np.array_equal(m.ranges().view(np.uint32), s["ranges"].reshape(-1).view(np.uint32))
        g = {"active_0": s["active"], "active_ids_0": s["active_ids"], "with_verts_0": s["with_verts"],
             "vert_offsets_0": s["vert_offsets"], "vertices_0": s["vertices"]}
        check_mc_against_golden(m, g, 0, n)


def test_oracle_unpack_matches_reference_vertex_stage(oracle):
    g = np.load(os.path.join(GOLDEN, "unpack_ct44.npz"))
    world, clip = oracle.unpack_vertices(g["vertices"], tuple(g["dims"]), tuple(g["scale"]), g["proj"])
    assert np.array_equal(world.view(np.uint32), g["world_bits"])
    assert np.array_equal(clip.view(np.uint32), g["clip_bits"])


def test_oracle_sort_matches_reference_shaders(oracle):
    g = np.load(os.path.join(GOLDEN, "sort.npz"))
    for i in range(int(g["cases"])):
        k, v = g[f"keys_{i}"], g[f"values_{i}"]
        assert np.array_equal(oracle.sort_by_key(k, v, False)[1], g[f"asc_{i}"]), i
        assert np.array_equal(oracle.sort_by_key(k, v, True)[1], g[f"desc_{i}"]), i


def test_oracle_sort_matches_reference_shaders_live(oracle):
    R = _ref()
    rng = np.random.default_rng(77)
    for _ in range(16):
        n = int(rng.integers(65, 1200))
        k = rng.integers(0, int(rng.choice([2, 9, 300, 2**32 - 2])), size=n, dtype=np.uint64).astype(np.uint32)
        v = rng.permutation(n).astype(np.uint32)
        for rev in (False, True):
            assert np.array_equal(R.sort_by_key(k, v, rev), oracle.sort_by_key(k, v, rev)[1])


# ---- scan, compaction and the LRU cache against the reference's shaders ----

def test_oracle_scan_and_compaction_match_reference_shaders(oracle):
    for n, v, g, i in GL.scan_cases():
        aligned = -(-n // 512) * 512
        buf = np.zeros(aligned, np.uint32)
        buf[:n] = v
        scanned, total = oracle.exclusive_scan(buf, n, aligned)
        GL.check_scan(g, i, n, scanned, total)
        flags = (v != 0).astype(np.uint32)
        offs, m = oracle.exclusive_scan(np.concatenate([flags, np.zeros(aligned - n, np.uint32)]), n, aligned)
        GL.check_compact(g, i, n, oracle.compact(flags, offs, n, m))


@pytest.mark.parametrize("seq", range(3))
def test_oracle_lru_matches_reference_shaders(oracle, seq):
    total, initial, steps, reset_at, recs = list(GL.lru_sequences())[seq]
    c = oracle.LRUCache(initial, total)
    for step, rec in enumerate(recs):
        if step == reset_at:
            c.reset()
        ids = c.update(rec["needed"])
        assert np.array_equal(ids, rec["new"]), step
        assert c.cache_size == rec["cache_size"], step
        if len(ids):
            assert c.slots_available == rec["display"], step
        GL.check_lru_state(rec, c.state(), step)


def test_oracle_pipeline_lru_matches_reference_shaders(oracle):
    for name, frac, isos, reset_at, recs in GL.lru_pipeline_cases():
        g = np.load(os.path.join(GOLDEN, f"mc_{name}.npz"))
        m = oracle.CompressedMarchingCubes(g["words"], int(g["rate"]), tuple(int(d) for d in g["dims"]),
                                           initial_cache_fraction=frac)
        for qi, (iso, rec) in enumerate(zip(isos, recs)):
            if qi == reset_at:
                m.cache_reset()
            n = m.compute_surface(float(iso))
            nverts, n_active, n_new, n_with = rec["counts"]
            assert n == nverts, (name, qi)
            if n_active:
                s = m.stats()
                assert (s["numActiveBlocks"], s["newDecompressed"], s["numBlocksWithVertices"]) == \
                    (n_active, n_new, n_with), (name, qi)
            assert GL.sha(m.vertices(n).reshape(-1)) == rec["mesh_sha"], (name, qi)
            GL.check_lru_state(rec, m.lru_state(), (name, qi))


def test_oracle_lru_matches_reference_shaders_live(oracle):
    """A further seeded sequence (small cache, frequent growth) through the
    reference's LRU, scan, compaction and sort shaders, live."""
    R = _ref()
    rng = np.random.default_rng(4242)
    total = 1200
    a, b = R.LRUCache(40, total), oracle.LRUCache(40, total)
    for step in range(16):
        if step == 12:
            a.reset()
            b.reset()
        needed = (np.convolve(rng.random(total) < rng.uniform(0.002, 0.05), np.ones(6), mode="same") > 0)
        needed = needed.astype(np.uint32)
        assert np.array_equal(a.update(needed), b.update(needed)), step
        sa = a.state()
        assert sa["cache_size"] == b.cache_size
        GL.check_lru_state({**sa, "total": total}, b.state(), step)
