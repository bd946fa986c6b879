"""A bounded device wait that runs out.  Every decoupled look-back has a spin
limit and reports an error status when it runs out (the reference only raises
alerts, js/lru_cache.js:315-317, js/exclusive_scan.js:117-119).

bcmc_debug_drop_tile makes one tile publish no look-back status, so the tiles
after it wait on a status word that nothing sets.  Their spin limit ends the
wait (about a second), the kernel records the site in the query state and
finishes, and the call returns BCMC_E_TIMEOUT.  No fault, no hang.  The same
context then runs normal queries bit-exactly."""
import ctypes as C
import time

import numpy as np
import pytest

import bcmc
from bcmc import _lib
from bcmc import datasets as D

pytestmark = pytest.mark.gpu

BCMC_E_TIMEOUT = 4


def test_scan_wait_runs_out_then_recovers(ctx):
    L = _lib.load()
    c = bcmc.Context(ctx.device)
    n = 4096 * 40 + 17
    a = np.random.default_rng(5).integers(0, 100, n).astype(np.uint32)
    pipe = bcmc.ExclusiveScanPipeline(c)
    assert L.bcmc_debug_drop_tile(c.handle, 3) == 0  # tile 2 publishes nothing
    s = pipe.prepareInput(a)
    t0 = time.perf_counter()
    with pytest.raises(bcmc.BcmcError) as e:
        s.scan(n)
    assert e.value.code == BCMC_E_TIMEOUT
    assert "timed out" in L.bcmc_last_error(c.handle).decode()
    assert time.perf_counter() - t0 < 30.0
    assert L.bcmc_debug_drop_tile(c.handle, 0) == 0
    s = pipe.prepareInput(a)
    total = s.scan(n)
    want = np.concatenate([[0], np.cumsum(a.astype(np.uint64))[:-1]]).astype(np.uint32)
    assert total == int(a.astype(np.uint64).sum() & 0xFFFFFFFF)
    assert np.array_equal(s.inputBuf.cpu().numpy().view(np.uint32)[:n], want)


def test_query_wait_runs_out_then_next_query_matches_oracle(ctx, oracle):
    """The active test's look-back (site 30/31): the query fails with
    BCMC_E_TIMEOUT and resets its cache; the next queries on the same context
    and volume are bit-exact with the oracle's from a reset cache."""
    L = _lib.load()
    dims, rate = (96, 96, 96), 4
    f = D.ct_like(dims, 2)
    words = oracle.zfp_encode(f, rate)
    c = bcmc.Context(ctx.device, initial_cache_fraction=0.05)
    mc = bcmc.CompressedMarchingCubes(c)
    mc.setCompressedVolume(words, rate, dims)
    ref = oracle.CompressedMarchingCubes(words, rate, dims, initial_cache_fraction=0.05)
    assert mc.computeSurface(90.0) == ref.compute_surface(90.0)
    assert mc.totalBlocks > 3 * 4096  # several active-test tiles
    assert L.bcmc_debug_drop_tile(c.handle, 1) == 0  # tile 0 publishes nothing
    with pytest.raises(bcmc.BcmcError) as e:
        mc.computeSurface(150.0)
    assert e.value.code == BCMC_E_TIMEOUT
    msg = L.bcmc_last_error(c.handle).decode()
    assert "site 30" in msg or "site 31" in msg, msg
    assert L.bcmc_debug_drop_tile(c.handle, 0) == 0
    ref.cache_reset()
    for iso in (150.0, 60.0, 200.0):
        n = mc.computeSurface(iso)
        n_ref = ref.compute_surface(iso)
        assert n == n_ref and n > 0, iso
        assert np.array_equal(mc.copyVertices(), ref.vertices(n_ref)), iso
        st, rs = mc.stats(), ref.stats()
        for k in ("numActiveBlocks", "newDecompressed", "numBlocksWithVertices", "numVertices"):
            assert st[k] == rs[k], (iso, k)
