"""CPU checks of the oracle (oracle/bcmc_oracle.c) -- no GPU.

The reference ships no tests or golden vectors, so the oracle is checked
against: a second pure-Python restatement (tests/refpy.py) on small cases,
closed-form properties (encode->decode error bounds, the sort's tie order, scan
totals), and the 256-case marching-cubes table sweep.
"""
import numpy as np
import pytest

import refpy
from bcmc import datasets as D


def _reassemble(dec, dims):
    nbx, nby, nbz = [(d + 3) // 4 for d in dims]
    v = dec.reshape(nbz, nby, nbx, 4, 4, 4).transpose(0, 3, 1, 4, 2, 5).reshape(4 * nbz, 4 * nby, 4 * nbx)
    return v[: dims[2], : dims[1], : dims[0]]


@pytest.mark.parametrize("dims", [(16, 16, 16), (13, 7, 9), (5, 12, 3)])
def test_encode_decode_roundtrip_error_falls_with_rate(oracle, dims):
    f = D.blobs(dims, seed=7, n_blobs=3)
    errs = []
    for rate in (2, 4, 8, 16):
        w = oracle.zfp_encode(f, rate)
        assert len(w) == oracle.stream_words(dims, 64 * rate)
        nb = int(np.prod(oracle.padded_blocks(dims)))
        dec = oracle.decode_volume(w, nb, 64 * rate)
        errs.append(float(np.abs(_reassemble(dec, dims) - f).max()))
    assert errs[-1] < 1e-6 * max(1.0, float(np.abs(f).max()))
    assert all(b <= a * 1.0001 + 1e-12 for a, b in zip(errs, errs[1:]))


def test_zero_block_is_single_bit(oracle):
    f = np.zeros((8, 8, 8), dtype=np.float32)
    w = oracle.zfp_encode(f, 4)
    assert not w.any()
    assert not oracle.decode_volume(w, 8, 256).any()


@pytest.mark.parametrize("max_bits", [64, 96, 128, 200, 256, 512, 1000])
def test_emulated_reader_matches_native(oracle, max_bits):
    """zfp_decompress.comp's {lo,hi} uint64 emulation (WGSL shifts mod 32)
    decodes exactly what a native 64-bit reader decodes, also for bit offsets
    that are not word aligned."""
    rng = np.random.default_rng(max_bits)
    nblocks = 40
    words = rng.integers(0, 2**63, size=(nblocks * max_bits + 63) // 64 + 2, dtype=np.uint64)
    words |= rng.integers(0, 2, size=words.shape, dtype=np.uint64) << np.uint64(63)
    for b in range(nblocks):
        a = oracle.decode_block(words, b, max_bits)
        c = oracle.decode_block(words, b, max_bits, native=True)
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32)), b


def test_u32_block_offset_wraps_in_reference(oracle):
    """zfp_decompress.comp:199 multiplies block_index*max_bits in 32 bits: block
    2^24+3 at 256 bits/block reads block 3's bits.  The oracle (and the CUDA
    decoder) use 64-bit offsets; the switch reproduces the wrap."""
    f = D.blobs((16, 16, 16), 3, n_blobs=2)
    w = oracle.zfp_encode(f, 4)
    wrapped = oracle.decode_block(w, (1 << 24) + 3, 256, emulate_u32_offset=True)
    assert np.array_equal(wrapped, oracle.decode_block(w, 3, 256))


@pytest.mark.parametrize("reverse", [True, False])
def test_sort_matches_literal_reference_algorithm(oracle, reverse):
    rng = np.random.default_rng(11 if reverse else 12)
    for trial in range(60):
        n = int(rng.integers(1, 400))
        keys = rng.integers(0, int(rng.integers(1, 9)), size=n).astype(np.uint32)
        vals = rng.permutation(n).astype(np.uint32)
        _, v = oracle.sort_by_key(keys, vals, reverse)
        assert list(v) == refpy.sort_by_key(list(keys), list(vals), reverse), (trial, n)


@pytest.mark.parametrize("reverse", [True, False])
def test_sort_tie_order_closed_form(oracle, reverse):
    """Among equal keys the reference's chunk sort + anti-stable merges (+
    reversal) order by 64-chunk then index, as documented in sort.cu."""
    rng = np.random.default_rng(5)
    for trial in range(40):
        n = int(rng.integers(1, 3000))
        keys = rng.integers(0, 7, size=n).astype(np.uint32)
        _, v = oracle.sort_by_key(keys, np.arange(n, dtype=np.uint32), reverse)
        if reverse:
            order = sorted(range(n), key=lambda p: (-int(keys[p]), p // 64, -p))
        else:
            order = sorted(range(n), key=lambda p: (int(keys[p]), -(p // 64), p))
        assert list(v) == order


def _age_key16(ages):
    """age_key16 of csrc/bcmc_internal.cuh: the LRU age sort's 16-bit key."""
    a = ages.astype(np.int64)
    return np.where(a < 32768, a, 32768 + (a - 100000)).astype(np.uint32)


def test_age_key16_keeps_the_lru_sort_order(oracle):
    """On ages below 2^15 or in [100000, 100000 + 2^15) (slots in use count up from
    0, the others from lru_cache_init.comp's 100000) the 16-bit key is strictly
    increasing and below 2^16, so the LRU's descending sort by it gives the
    reference's order and ties exactly."""
    edge = np.array([0, 1, 2, 32766, 32767, 100000, 100001, 132766, 132767], np.uint32)
    k16 = _age_key16(edge)
    assert np.all(np.diff(k16.astype(np.int64)) > 0) and int(k16.max()) < 65536
    rng = np.random.default_rng(21)
    for trial in range(24):
        n = int(rng.integers(1, 5000))
        if trial % 3 == 0:
            ages = rng.choice(edge, n).astype(np.uint32)
        else:
            small = rng.integers(0, 20, n)
            big = 100000 + rng.integers(0, 20, n)
            ages = np.where(rng.random(n) < 0.5, small, big).astype(np.uint32)
        vals = np.arange(n, dtype=np.uint32)
        _, v_raw = oracle.sort_by_key(ages, vals, True)
        _, v_16 = oracle.sort_by_key(_age_key16(ages), vals, True)
        assert np.array_equal(v_raw, v_16), (trial, n)


def test_scan_and_compact(oracle):
    rng = np.random.default_rng(3)
    x = rng.integers(0, 2, size=1000).astype(np.uint32)
    out, tot = oracle.exclusive_scan(np.concatenate([x, np.zeros(24, np.uint32)]), 1000, 1024)
    assert tot == int(x.sum())
    assert np.array_equal(out[:1000], np.concatenate([[0], np.cumsum(x)[:-1]]).astype(np.uint32))
    assert out[1000] == tot
    ids = oracle.compact(x, out, 1000, tot)
    assert np.array_equal(ids, np.nonzero(x)[0].astype(np.uint32))


def test_case_table_sweep(oracle):
    """All 256 corner sign patterns: vertex counts are multiples of 3, at most
    15, 0 exactly for the empty and full cases, and complementary cases cross
    the same set of edges."""
    tri = oracle.tri_table()
    counts = [oracle.case_vertex_count(c) for c in range(256)]
    assert counts[0] == 0 and counts[255] == 0
    for c in range(256):
        assert counts[c] % 3 == 0 and counts[c] <= 15
        assert all(0 <= e < 12 for e in tri[c][: counts[c]])
        if 0 < c < 255:
            assert counts[c] > 0
            assert set(tri[c][: counts[c]]) == set(tri[255 - c][: counts[255 - c]])


def test_lru_matches_python_restatement(oracle):
    rng = np.random.default_rng(9)
    total = 300
    c = oracle.LRUCache(20, total)
    r = refpy.LRU(20, total)
    for step in range(40):
        if step == 25:
            c.reset()
            r.reset()
        p = rng.uniform(0.02, 0.5)
        needed = (rng.random(total) < p).astype(np.uint32)
        new_c = c.update(needed)
        new_r = r.update(list(needed))
        assert list(new_c) == new_r, step
        st = c.state()
        assert c.cache_size == r.cache_size
        assert list(st["item_slots"]) == r.item_slots[:total]
        assert list(st["age"]) == r.age
        assert list(st["avail"]) == r.avail
        assert list(st["item"]) == r.item
        if new_r:
            assert c.slots_available == r.display


@pytest.mark.parametrize("dims,iso", [((12, 12, 12), 1.7), ((13, 9, 11), 1.5), ((13, 9, 11), 2.1)])
def test_mc_matches_python_restatement(oracle, dims, iso):
    f = D.blobs(dims, seed=21, n_blobs=4)
    w = oracle.zfp_encode(f, 8)
    m = oracle.CompressedMarchingCubes(w, 8, dims, initial_cache_fraction=0.5)
    n = m.compute_surface(iso)
    verts = m.vertices(n)
    nb = oracle.padded_blocks(dims)
    active = m.active()
    tri = oracle.tri_table()
    decoded = lambda b: oracle.decode_block(w, b, 512)
    expect = []
    for b in np.nonzero(active)[0]:
        expect += refpy.block_vertices(decoded, active, nb, int(b), iso, tri)
    assert n == len(expect) and n > 0
    assert [tuple(v) for v in verts] == expect


def test_mc_zero_active_keeps_cache_untouched(oracle):
    f = D.blobs((16, 16, 16), 2)
    w = oracle.zfp_encode(f, 8)
    m = oracle.CompressedMarchingCubes(w, 8, (16, 16, 16))
    assert m.compute_surface(float(f.min() + f.max()) / 2) > 0
    before = m.lru_state()
    assert m.compute_surface(1e9) == 0
    after = m.lru_state()
    for k in ("age", "avail", "item", "item_slots"):
        assert np.array_equal(before[k], after[k])
