"""Isovalue benchmark drivers (js/run_benchmark.js:1-47, js/bcmc.js:319-370).

The reference's page runs 100 isosurface queries per benchmark -- isovalues
drawn uniformly from the dataset's range ("random"), or stepping through it by
range/100 per query from the bottom ("sweepUp") or the top ("sweepDown") --
after resetting the cache, records for every query the isovalue, the wall time
of computeSurface, the memory report and the stage timings computeSurface
appends to its perfTracker, and saves them as
``bcmc-explicit-<dataset>-<benchmark>.json``.  These classes and run_benchmark
do the same against bcmc.CompressedMarchingCubes.  The random benchmark takes
a seed (the reference uses Math.random).

Run from the command line:
    python -m bcmc.benchmark --zfp FILE --rate R --range LO HI --kind random [--out DIR]
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np


class IsovalueSlider:
    """Stands in for the page's isovalue slider: a value the drivers set."""

    def __init__(self, value: float = 0.0):
        self.value = float(value)


class RandomIsovalueBenchmark:
    """js/run_benchmark.js:1-17."""

    def __init__(self, isovalueSlider, perfResults, range_, seed: int = 0):
        self.iteration = 0
        self.isovalueSlider = isovalueSlider
        self.perfResults = perfResults
        self.range = range_
        self.name = "random"
        self._rng = np.random.default_rng(seed)

    def run(self) -> bool:
        if self.iteration == 100:
            return False
        span = self.range[1] - self.range[0]
        self.isovalueSlider.value = float(self._rng.random() * span + self.range[0])
        self.iteration += 1
        return True


class SweepIsovalueBenchmark:
    """js/run_benchmark.js:19-47 (SweepIsovalueBenchark)."""

    def __init__(self, isovalueSlider, perfResults, range_, sweepUp: bool):
        self.iteration = 0
        self.isovalueSlider = isovalueSlider
        self.perfResults = perfResults
        self.range = range_
        self.sweepUp = sweepUp
        self.currentValue = range_[0] if sweepUp else range_[1]
        self.name = "sweepUp" if sweepUp else "sweepDown"

    def run(self) -> bool:
        if self.iteration == 100:
            return False
        step = (self.range[1] - self.range[0]) / 100
        self.currentValue += step if self.sweepUp else -step
        self.isovalueSlider.value = self.currentValue
        self.iteration += 1
        return True


def make_benchmark(kind: str, slider, perf, range_, seed: int = 0):
    if kind == "random":
        return RandomIsovalueBenchmark(slider, perf, range_, seed)
    if kind in ("sweepUp", "sweepDown"):
        return SweepIsovalueBenchmark(slider, perf, range_, kind == "sweepUp")
    raise ValueError(kind)


def run_benchmark(mc, dataset_name: str, range_, kind: str, seed: int = 0, out_dir: str | None = None) -> dict:
    """One benchmark as js/bcmc.js:319-370 runs it: cache reset, then one query
    per driver step; returns perfResults (and writes the JSON when out_dir is
    given)."""
    perf = {"isovalue": [], "totalTime": [], "memUse": []}
    mc.lruCache.reset()
    slider = IsovalueSlider(range_[0])
    bench = make_benchmark(kind, slider, perf, range_, seed)
    current = None
    while bench.run():
        if slider.value == current:  # the page only recomputes when the value changes
            continue
        current = float(slider.value)
        t0 = time.perf_counter()
        mc.computeSurface(current, perf)
        t1 = time.perf_counter()
        perf["isovalue"].append(current)
        perf["totalTime"].append(1000.0 * (t1 - t0))
        perf["memUse"].append(mc.reportMemoryUse()[3])
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
        with open(os.path.join(out_dir, f"bcmc-explicit-{dataset_name}-{bench.name}.json"), "w") as f:
            json.dump(perf, f)
    return perf


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--zfp", required=True)
    ap.add_argument("--rate", type=int, required=True)
    ap.add_argument("--range", type=float, nargs=2, required=True)
    ap.add_argument("--kind", default="random", choices=["random", "sweepUp", "sweepDown"])
    ap.add_argument("--dims", type=int, nargs=3, default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=".")
    a = ap.parse_args()
    import bcmc
    from bcmc import volumes

    data, dims = volumes.load_zfp(a.zfp, a.rate, a.dims)
    mc = bcmc.CompressedMarchingCubes(0)
    mc.setCompressedVolume(data, a.rate, dims)
    name = os.path.basename(a.zfp)[: -len(".zfp")] if a.zfp.endswith(".zfp") else os.path.basename(a.zfp)
    perf = run_benchmark(mc, name, tuple(a.range), a.kind, a.seed, a.out)
    t = np.asarray(perf["totalTime"])
    print(json.dumps({"queries": len(t), "mean_ms": float(t.mean()), "p50_ms": float(np.percentile(t, 50)),
                      "p99_ms": float(np.percentile(t, 99))}))


if __name__ == "__main__":
    main()
