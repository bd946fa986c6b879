"""The host-side rows on the GPU path: a .zfp file written, loaded by the
dataset loader and meshed by the CUDA pipeline against the oracle, and the
benchmark drivers (js/run_benchmark.js, js/bcmc.js:319-370) run on a real
CompressedMarchingCubes."""
import json
import os

import numpy as np
import pytest

import bcmc
from bcmc import benchmark as B
from bcmc import datasets as D
from bcmc import volumes as V

pytestmark = pytest.mark.gpu

# js/compressed_marching_cubes.js:593-610: the keys computeSurface appends to
STAGE_KEYS = ("computeActiveBlocks", "numActiveBlocks", "cacheUpdate", "numBlocksDecompressed", "decompression",
              "compactActiveIDs", "computeBlockHasVertices", "numBlocksWithVertices", "compactBlocksWithVertices",
              "numVertices", "computeVertices")


def test_zfp_file_loaded_and_meshed_against_oracle(ctx, oracle, tmp_path):
    dims, rate = (45, 38, 29), 4
    f = D.ct_like(dims, 7)
    words = oracle.zfp_encode(f, rate)
    name = f"ctfile_{dims[0]}x{dims[1]}x{dims[2]}_float32"
    path = os.path.join(tmp_path, name + ".zfp")
    V.save_zfp(path, np.ascontiguousarray(words).view(np.uint8)[: V.stream_bytes(dims, rate)])
    V.register("ctfile_test", V.Dataset(name, rate, (float(f.min()), float(f.max())), scale=(1.0, 1.0, 2.0)))
    mc, ds = V.open_dataset("ctfile_test", str(tmp_path), ctx)
    assert ds.dims == dims and mc.totalBlocks == int(np.prod([(d + 3) // 4 for d in dims]))
    ref = oracle.CompressedMarchingCubes(words, rate, dims, initial_cache_fraction=0.05)
    for iso in np.linspace(40.0, 200.0, 5):
        n = mc.computeSurface(float(iso))
        n_ref = ref.compute_surface(float(iso))
        assert n == n_ref and n > 0, iso
        assert np.array_equal(mc.copyVertices(), ref.vertices(n_ref)), iso
    with pytest.raises(ValueError):  # a file shorter than the stream the name asks for
        short = os.path.join(tmp_path, "short_8x8x8_float32.zfp")
        V.save_zfp(short, np.zeros(10, np.uint8))
        V.load_zfp(short, rate)


@pytest.mark.parametrize("kind", ["random", "sweepUp", "sweepDown"])
def test_benchmark_driver_on_gpu(ctx, oracle, tmp_path, kind):
    dims, rate = (40, 40, 40), 4
    f = D.blobs(dims, 3)
    words = oracle.zfp_encode(f, rate)
    mc = bcmc.CompressedMarchingCubes(ctx)
    mc.setCompressedVolume(np.ascontiguousarray(words).view(np.uint8)[: V.stream_bytes(dims, rate)], rate, dims)
    rng = (0.05, float(f.max()))
    perf = B.run_benchmark(mc, "blobs40", rng, kind, seed=3, out_dir=str(tmp_path))
    with open(os.path.join(tmp_path, f"bcmc-explicit-blobs40-{kind}.json")) as fh:
        saved = json.load(fh)
    assert saved == json.loads(json.dumps(perf))
    nq = len(perf["isovalue"])
    assert nq == 100
    for k in ("isovalue", "totalTime", "memUse") + STAGE_KEYS:
        assert len(perf[k]) == nq, k
    assert perf["totalBlocks"] == mc.totalBlocks
    # the driver's queries, replayed on the oracle from a reset cache, give the same counts
    ref = oracle.CompressedMarchingCubes(words, rate, dims, initial_cache_fraction=0.05)
    for i, iso in enumerate(perf["isovalue"]):
        n_ref = ref.compute_surface(float(np.float32(iso)))
        assert perf["numVertices"][i] == n_ref, (i, iso)
