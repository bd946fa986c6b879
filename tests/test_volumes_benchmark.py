"""Host logic of the dataset registry / .zfp loader (js/volumes.js) and the
isovalue benchmark drivers (js/run_benchmark.js) -- no GPU."""
import json
import os

import numpy as np
import pytest

from bcmc import benchmark as B
from bcmc import volumes as V


def test_volume_dimensions_follow_the_reference_regex():
    assert V.volume_dimensions("skull_256x256x256_uint8.raw.crate4") == (256, 256, 256)
    assert V.volume_dimensions("/x/y/plane_x_32x32x32_float32.gen.crate2.zfp") == (32, 32, 32)
    assert V.volume_dimensions("foo_1024x1024x1080_uint16.raw") == (1024, 1024, 1080)
    with pytest.raises(ValueError):
        V.volume_dimensions("no_dims_here.zfp")


def test_zfp_file_round_trip(tmp_path, oracle):
    from bcmc import datasets as D

    dims, rate = (20, 16, 12), 8
    f = D.blobs(dims, 3)
    words = oracle.zfp_encode(f, rate)
    name = "blob_20x16x12_float32.gen.crate8"
    path = os.path.join(tmp_path, name + ".zfp")
    V.save_zfp(path, words.view(np.uint8)[: V.stream_bytes(dims, rate)])
    data, d = V.load_zfp(path, rate)
    assert d == dims
    assert np.array_equal(data, words.view(np.uint8)[: V.stream_bytes(dims, rate)])
    with pytest.raises(ValueError):
        V.load_zfp(path, 16)  # too short for rate 16
    ds = V.register("blob_test", V.Dataset(name, rate, (0.0, 1.0)))
    assert ds.dims == dims and ds.zfp_name == name + ".zfp"
    assert V.REGISTRY["blob_test"] is ds


def test_write_synthetic_with_a_host_encoder(tmp_path, oracle):
    path = V.write_synthetic("blobs64", str(tmp_path), encode=oracle.zfp_encode)
    data, dims = V.load_zfp(path, 8)
    assert dims == (64, 64, 64) and data.size == V.stream_bytes(dims, 8)


def test_drivers_issue_the_reference_sequences():
    s = B.IsovalueSlider()
    sweep = B.SweepIsovalueBenchmark(s, {}, (0.0, 2.0), True)
    vals = []
    while sweep.run():
        vals.append(s.value)
    assert len(vals) == 100 and vals[0] == pytest.approx(0.02) and vals[-1] == pytest.approx(2.0)
    down = B.SweepIsovalueBenchmark(s, {}, (0.0, 2.0), False)
    vals = []
    while down.run():
        vals.append(s.value)
    assert vals[0] == pytest.approx(1.98) and vals[-1] == pytest.approx(0.0, abs=1e-9)
    rnd = B.RandomIsovalueBenchmark(s, {}, (10.0, 20.0), seed=1)
    vals = []
    while rnd.run():
        vals.append(s.value)
    assert len(vals) == 100 and all(10.0 <= v < 20.0 for v in vals)
    assert rnd.name == "random" and sweep.name == "sweepUp" and down.name == "sweepDown"


class _FakeMC:
    """Stands in for CompressedMarchingCubes: records queries, fills the
    perfTracker keys the way computeSurface does."""

    def __init__(self):
        self.queries = []
        self.resets = 0
        outer = self

        class _LRU:
            def reset(self):
                outer.resets += 1

        self.lruCache = _LRU()

    def computeSurface(self, iso, perf):
        self.queries.append(iso)
        perf.setdefault("numVertices", []).append(int(iso * 10))
        return int(iso * 10)

    def reportMemoryUse(self):
        return ["", "", "", {"mc": {}, "cache": {}}]


def test_run_benchmark_writes_the_reference_json(tmp_path):
    mc = _FakeMC()
    perf = B.run_benchmark(mc, "fake_8x8x8_float32", (0.0, 1.0), "sweepUp", out_dir=str(tmp_path))
    assert mc.resets == 1 and len(mc.queries) == 100
    for k in ("isovalue", "totalTime", "memUse", "numVertices"):
        assert len(perf[k]) == 100
    with open(os.path.join(tmp_path, "bcmc-explicit-fake_8x8x8_float32-sweepUp.json")) as f:
        assert json.load(f)["isovalue"] == perf["isovalue"]
