"""Continuous-batching server (bcmc_server_*): requests submitted together are
batched, each request's vertices equal the plain path's for its (volume,
isovalue) -- alone and in the mix, also when batches overlap on the device --
and the open-loop load generator reports consistent throughput and latency
figures."""
import time
import threading

import numpy as np
import pytest

import bcmc
from bcmc import datasets as D

pytestmark = pytest.mark.gpu

VOLUMES = [("blobs", (48, 40, 36), 1, 8), ("ct_like", (64, 64, 64), 2, 4), ("turbulence", (40, 40, 40), 3, 2)]


@pytest.fixture(scope="module")
def volumes(oracle):
    out = []
    for kind, dims, seed, rate in VOLUMES:
        f = D.make_field(kind, dims, seed)
        words = oracle.zfp_encode(f, rate)
        nb = int(np.prod([(d + 3) // 4 for d in dims]))
        out.append(dict(dims=dims, rate=rate, stream=words.view(np.uint8)[: nb * 64 * rate // 8].copy(),
                        lo=float(f.min()), hi=float(f.max())))
    return out


def _server(ctx, volumes, **kw):
    eng = bcmc.Engine(ctx, max_batch=64)
    for v in volumes:
        eng.addVolume(v["stream"], v["rate"], v["dims"])
    return eng, bcmc.Server(eng, **kw)


def _isos(volumes, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        v = i % len(volumes)
        lo, hi = volumes[v]["lo"], volumes[v]["hi"]
        out.append((v, float(np.float32(rng.uniform(lo + 0.1 * (hi - lo), hi - 0.1 * (hi - lo))))))
    return out


def test_requests_match_plain_path(ctx, volumes):
    reqs = _isos(volumes, 30, seed=5)
    plain = []
    mcs = {}
    for v, iso in reqs:
        if v not in mcs:
            mcs[v] = bcmc.CompressedMarchingCubes(ctx)
            mcs[v].setCompressedVolume(volumes[v]["stream"], volumes[v]["rate"], volumes[v]["dims"])
        n = mcs[v].computeSurface(iso)
        plain.append(mcs[v].copyVertices().copy())
    eng, srv = _server(ctx, volumes, max_wait_us=2000)
    try:
        tickets = [srv.submit(v, iso, max_vertices=len(plain[i]) + 8) for i, (v, iso) in enumerate(reqs)]
        for i, t in enumerate(tickets):
            n, nact, lat, verts = srv.wait(t)
            assert n == len(plain[i]), i
            assert np.array_equal(verts, plain[i]), i
            assert lat > 0.0
        st = eng.stats()
        assert st["batches"] < len(reqs)  # requests were batched
    finally:
        srv.close()


def test_concurrent_clients(ctx, volumes):
    reqs = _isos(volumes, 40, seed=6)
    eng, srv = _server(ctx, volumes)
    results = {}

    def client(lo, hi):
        for i in range(lo, hi):
            t = srv.submit(*reqs[i])
            results[i] = srv.wait(t)[0]

    try:
        threads = [threading.Thread(target=client, args=(k * 10, k * 10 + 10)) for k in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
    finally:
        srv.close()
    alone = bcmc.Engine(ctx)
    for v in volumes:
        alone.addVolume(v["stream"], v["rate"], v["dims"])
    for i, (v, iso) in enumerate(reqs):
        assert results[i] == int(alone.run([(v, iso)])[0]["num_vertices"]), i


def test_open_loop_load_report(ctx, volumes):
    eng, srv = _server(ctx, volumes, max_wait_us=200)
    try:
        rep = srv.run_load(rate_qps=4000.0, requests=400, volumes=[0, 1, 2], weights=[1, 2, 1],
                           iso_lo=[v["lo"] + 0.1 * (v["hi"] - v["lo"]) for v in volumes],
                           iso_hi=[v["hi"] - 0.1 * (v["hi"] - v["lo"]) for v in volumes], seed=7)
    finally:
        srv.close()
    assert rep["completed"] == 400
    assert 0.0 < rep["p50_ms"] <= rep["p95_ms"] <= rep["p99_ms"] <= rep["max_ms"]
    assert rep["batches"] >= 1 and rep["mean_batch"] >= 1.0
    assert rep["achieved_qps"] > 0.0
    assert 0 <= rep["overlapped_batches"] < rep["batches"]


def test_overlapped_batches_match_plain_path(ctx, volumes):
    """A steady stream of requests keeps a batch on the device while the next
    arrives: the next batch is launched at once (its active test, claims and
    decode overlap the first batch's marching cubes).  Every result equals
    the plain path's."""
    reqs = _isos(volumes, 160, seed=8)
    plain = []
    mcs = {}
    for v, iso in reqs:
        if v not in mcs:
            mcs[v] = bcmc.CompressedMarchingCubes(ctx)
            mcs[v].setCompressedVolume(volumes[v]["stream"], volumes[v]["rate"], volumes[v]["dims"])
        mcs[v].computeSurface(iso)
        plain.append(mcs[v].copyVertices().copy())
    eng, srv = _server(ctx, volumes)
    try:
        tickets = []
        for i, (v, iso) in enumerate(reqs):
            tickets.append(srv.submit(v, iso, max_vertices=len(plain[i]) + 8))
            if i % 4 == 3:
                time.sleep(50e-6)
        for i, t in enumerate(tickets):
            n, nact, lat, verts = srv.wait(t)
            assert n == len(plain[i]), i
            assert np.array_equal(verts, plain[i]), i
        st = eng.stats()
        assert st["overlapped_batches"] > 0, st
        assert st["batches"] < len(reqs)
    finally:
        srv.close()


def test_single_request_batches_overlap_and_match_plain_path(ctx, volumes):
    """max_batch=1 (the setting for mixes whose queries each fill the GPU):
    every request is its own batch, the next one is launched while the one
    before it is still on the device, and every result equals the plain
    path's."""
    reqs = _isos(volumes, 60, seed=9)
    plain = []
    mcs = {}
    for v, iso in reqs:
        if v not in mcs:
            mcs[v] = bcmc.CompressedMarchingCubes(ctx)
            mcs[v].setCompressedVolume(volumes[v]["stream"], volumes[v]["rate"], volumes[v]["dims"])
        mcs[v].computeSurface(iso)
        plain.append(mcs[v].copyVertices().copy())
    eng, srv = _server(ctx, volumes, max_batch=1)
    try:
        tickets = [srv.submit(v, iso, max_vertices=len(plain[i]) + 8) for i, (v, iso) in enumerate(reqs)]
        for i, t in enumerate(tickets):
            n, nact, lat, verts = srv.wait(t)
            assert n == len(plain[i]), i
            assert np.array_equal(verts, plain[i]), i
        st = eng.stats()
        assert st["batches"] == len(reqs), st
        assert st["overlapped_batches"] > 0, st
    finally:
        srv.close()


def test_each_ticket_is_waited_for_once(ctx, volumes):
    """A ticket already waited for, or never issued, is refused at once
    instead of blocking its caller; the server keeps serving."""
    eng, srv = _server(ctx, volumes, max_batch=4)
    try:
        (v, iso), = _isos(volumes, 1, seed=11)
        t = srv.submit(v, iso)
        n = srv.wait(t)[0]
        with pytest.raises(bcmc.BcmcError):
            srv.wait(t)
        with pytest.raises(bcmc.BcmcError):
            srv.wait(t + 1000)
        with pytest.raises(bcmc.BcmcError):  # an unknown volume is refused at submission
            srv.submit(len(volumes), iso)
        assert srv.wait(srv.submit(v, iso))[0] == n
    finally:
        srv.close()
