"""Batched engine (bcmc_engine_*): every query's vertices must equal what the
plain per-query path (CompressedMarchingCubes.computeSurface) returns for the
same (volume, isovalue), bit for bit -- alone and in a mix of queries over
volumes of different shapes, rates and fields, through chunking, slot-pool
eviction and vertex-buffer growth."""
import numpy as np
import pytest

import bcmc
from bcmc import datasets as D

pytestmark = pytest.mark.gpu

VOLUMES = [
    ("blobs", (48, 40, 36), 1, 8),
    ("ct_like", (64, 64, 64), 2, 4),
    ("turbulence", (40, 40, 40), 3, 2),
    ("ct_uint16", (30, 21, 17), 5, 4),   # partial blocks; (8*6) % 4 == 0
    ("blobs", (44, 40, 28), 7, 3),       # (11*10) % 4 != 0: the reference's range quirk applies
]


@pytest.fixture(scope="module")
def volumes(oracle):
    out = []
    for kind, dims, seed, rate in VOLUMES:
        f = D.make_field(kind, dims, seed)
        words = oracle.zfp_encode(f, rate)
        nb = int(np.prod([(d + 3) // 4 for d in dims]))
        stream = words.view(np.uint8)[: nb * 64 * rate // 8].copy()
        lo, hi = float(f.min()), float(f.max())
        out.append(dict(kind=kind, dims=dims, rate=rate, stream=stream, lo=lo, hi=hi))
    return out


def _queries(volumes, n, seed):
    rng = np.random.default_rng(seed)
    qs = []
    for _ in range(n):
        v = int(rng.integers(0, len(volumes)))
        lo, hi = volumes[v]["lo"], volumes[v]["hi"]
        qs.append((v, float(np.float32(rng.uniform(lo + 0.05 * (hi - lo), hi - 0.05 * (hi - lo))))))
    return qs


def _plain(ctx, volumes, qs):
    """Per-query vertices from the plain path (one CompressedMarchingCubes per volume)."""
    mcs = {}
    out = []
    for v, iso in qs:
        if v not in mcs:
            mc = bcmc.CompressedMarchingCubes(ctx)
            mc.setCompressedVolume(volumes[v]["stream"], volumes[v]["rate"], volumes[v]["dims"])
            mcs[v] = mc
        n = mcs[v].computeSurface(iso)
        out.append((n, mcs[v].stats()["numActiveBlocks"], mcs[v].copyVertices().copy()))
    return out


def _engine(ctx, volumes, **kw):
    eng = bcmc.Engine(ctx, **kw)
    for vol in volumes:
        eng.addVolume(vol["stream"], vol["rate"], vol["dims"])
    return eng


def _check(eng, res, want):
    allv = eng.copyVertices()
    for i, (n, nact, verts) in enumerate(want):
        r = res[i]
        assert int(r["num_vertices"]) == n, i
        assert int(r["num_active_blocks"]) == nact, i
        off = int(r["vertex_offset"])
        assert np.array_equal(allv[off: off + n], verts), i


def test_batch_matches_plain_path(ctx, volumes):
    qs = _queries(volumes, 48, seed=1)
    want = _plain(ctx, volumes, qs)
    eng = _engine(ctx, volumes)
    res = eng.run(qs)
    _check(eng, res, want)
    # the same batch again: every block now cached, identical output
    res2 = eng.run(qs)
    _check(eng, res2, want)
    st = eng.stats()
    assert st["batches"] == 2 and st["queries"] == 96
    assert st["evicted_blocks"] == 0


def test_alone_equals_in_the_mix(ctx, volumes):
    qs = _queries(volumes, 24, seed=2)
    eng = _engine(ctx, volumes)
    mix = eng.run(qs)
    mix_verts = eng.copyVertices()
    for i, q in enumerate(qs[:6]):
        alone = eng.run([q])
        a = eng.copyVertices()
        n = int(alone[0]["num_vertices"])
        assert n == int(mix[i]["num_vertices"])
        off = int(mix[i]["vertex_offset"])
        assert np.array_equal(a[:n], mix_verts[off: off + n])


def test_chunking_eviction_and_growth(ctx, volumes):
    """max_batch 4 (many launch sequences), a pool smaller than the union of the
    batch's active blocks (evictions and split sequences), a tiny initial vertex
    buffer (growth)."""
    qs = _queries(volumes, 20, seed=3)
    want = _plain(ctx, volumes, qs)
    max_active = max(w[1] for w in want)
    eng = _engine(ctx, volumes, pool_slots=int(max_active * 1.5) + 64, vertex_capacity=1000, max_batch=4)
    res = eng.run(qs)
    _check(eng, res, want)
    st = eng.stats()
    assert st["launch_sequences"] >= 5
    assert st["evicted_blocks"] > 0
    assert st["vertex_capacity"] >= sum(w[0] for w in want)


def test_empty_and_out_of_range_queries(ctx, volumes):
    eng = _engine(ctx, volumes)
    res = eng.run([(0, 1e9), (1, -1e9), (2, float(volumes[2]["lo"]) + 0.3)])
    assert int(res[0]["num_vertices"]) == 0 and int(res[0]["num_active_blocks"]) == 0
    assert int(res[1]["num_vertices"]) == 0
    with pytest.raises(bcmc.BcmcError):
        eng.run([(99, 0.5)])


def test_vertex_budget_admits_a_prefix(ctx, volumes):
    """run_admit runs the longest prefix of the batch whose vertices (known from
    the count pass) fit the budget; the rest is left to the caller."""
    qs = _queries(volumes, 12, seed=8)
    want = _plain(ctx, volumes, qs)
    counts = [w[0] for w in want]
    budget = sum(counts[:5]) + 1  # the first 5 fit, the 6th does not
    assert counts[5] > 1
    eng = _engine(ctx, volumes, vertex_budget=budget, max_batch=16)
    res, m = eng.run_admit(qs)
    assert m == 5
    _check(eng, res, want[:m])
    # the remainder in the next run
    res2, m2 = eng.run_admit(qs[m:])
    assert m2 >= 1
    _check(eng, res2, want[m: m + m2])


def test_autotune_keeps_results(ctx, volumes):
    qs = _queries(volumes, 16, seed=9)
    want = _plain(ctx, volumes, qs)
    eng = _engine(ctx, volumes)
    rep = eng.autotune(qs)
    assert rep["bucket"] == 16
    assert rep["mc_ctas_per_sm"] in (4, 5, 6) and rep["act_ctas_per_sm"] in (4, 8, 16)
    assert rep["mc_blocks_per_tile"] in (8, 16, 32)
    assert rep["decode_threads"] in (64, 128, 256) and rep["decode_ctas_per_sm"] in (8, 16, 32)
    assert rep["batch_ms_tuned"] <= rep["batch_ms_default"] + 1e-9
    res = eng.run(qs)
    _check(eng, res, want)


@pytest.mark.parametrize("mc_blocks", [8, 16, 32])
def test_every_mc_tile_keeps_results(ctx, volumes, mc_blocks):
    """Each compiled MC tile shape the autotuner can pick gives the plain
    path's meshes (the tile is forced through the autotuner's test hook)."""
    qs = _queries(volumes, 12, seed=10 + mc_blocks)
    want = _plain(ctx, volumes, qs)
    eng = _engine(ctx, volumes)
    eng.force_config(len(qs), mc_blocks_per_tile=mc_blocks)
    _check(eng, eng.run(qs), want)
