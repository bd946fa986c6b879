"""Benchmark: iso-queries/s of the block-compressed marching-cubes pipeline.

Workload (one "step"): the 256^3 CT-like volume (uint8-range values stored as
float32, ~35 % constant-0 background blocks, interior 20-255 + N(0,3) noise),
ZFP fixed rate 4 bits/value, cache initially 50 % of the 262,144 blocks; the
step resets the cache and runs the 16 isovalues linspace(30, 220, 16) one at a
time through computeSurface.  Synthetic data generated from a seed (the
reference's scans are not shipped).

Lines printed (one JSON line on rank 0):
  value   iso-queries/s, volume resident in HBM, timed with CUDA events on the
          library's stream (L2 flushed with a 512 MB write between steps);
          computeSurface is called without a perf tracker, as by default
  e2e     the same through the C ABI with every query's vertices delivered
          into pinned host memory (bcmc_compute_surfaces_host: the sweep in
          one call, each query's vertices copied out while the next computes;
          per query with bcmc_compute_surface_host alongside)
  roofline  the dominant kernel's algorithmic bytes / its CUDA-event time,
          from a second timed pass with a perf tracker (its stage events
          slow each query down, so the headline pass runs without them)
  cpu_baseline  the CPU oracle (OpenMP, all host cores) on one step
  decode  full-volume ZFP decode of the 512^3 spectral field at rate 2, GB/s
  walk    the plain path on that field's 64-isovalue random walk (cache 25 %),
          with the oracle on the walk's first 8 queries beside it
  batched / served / render_ms  the batched engine, the continuous-batching
          server and the render pass, each summarised; their full records
          (per-rate sweeps, autotune choices) go to the detail file (DETAIL)

`--impl reference` times the CPU restatement of the reference pipeline (the
reference itself is WebGPU/JavaScript and has no CPU path) on the same config.
Under torchrun (N>1) each rank runs an independent replica (the path does not
shard); value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "webgpu-bcmc_gb300"))

CONFIG = dict(workload="ct256: 256^3 CT-like float32, ZFP rate 4, 16 isovalues linspace(30,220,16), "
                       "cache 50% of 262144 blocks, cache reset per step",
              dims=(256, 256, 256), rate=4, seed=2, cache_fraction=0.5)
METRIC = "iso-queries/s (plain per-query path, ct256)"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock and throttle reasons)."""

    def __init__(self, index: int = 0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                           "--format=csv,noheader,nounits", "-lms", "100"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self) -> dict:
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_volume():
    from bcmc import datasets as D

    field = D.ct_like(CONFIG["dims"], CONFIG["seed"])
    isos = np.linspace(30.0, 220.0, 16).astype(np.float32)
    return field, isos


def encode_on_gpu(ctx, field):
    import torch

    import bcmc

    words = bcmc.zfp_encode(ctx, torch.from_numpy(field).cuda(), CONFIG["rate"])
    torch.cuda.synchronize()
    nb = int(np.prod([(d + 3) // 4 for d in CONFIG["dims"]]))
    nbytes = nb * 64 * CONFIG["rate"] // 8
    host = words.cpu().numpy().view(np.uint8)[:nbytes].copy()
    return words, host


def cpu_oracle_time(field, isos, steps: int = 1, warmup: int = 1):
    """The oracle (C, OpenMP over all host threads) on `steps` timed steps after
    `warmup` untimed ones (each: cache reset + the query sequence)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    words = oracle.zfp_encode(field, CONFIG["rate"])
    m = oracle.CompressedMarchingCubes(words, CONFIG["rate"], CONFIG["dims"],
                                       initial_cache_fraction=CONFIG["cache_fraction"])
    for _ in range(warmup):
        m.cache_reset()
        for iso in isos:
            m.compute_surface(float(iso))
    t0 = time.perf_counter()
    for _ in range(steps):
        m.cache_reset()
        for iso in isos:
            m.compute_surface(float(iso))
    dt = time.perf_counter() - t0
    return len(isos) * steps / dt, oracle.threads(), words


def max_over_ranks(value: float, device) -> float:
    """The slowest rank's figure when a process group is up (every rank calls
    it); the value itself for a single process."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    """CPU restatement of the reference pipeline, all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    field, isos = make_volume()
    steps = max(1, args.steps)
    qps, threads, _ = cpu_oracle_time(field, isos, steps=steps, warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1000.0 * len(isos) / qps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded CT-like field, ZFP-encoded by the project's encoder)",
            "config": {"workload": CONFIG["workload"]},
            "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{steps} step(s) of 16 queries, CPU oracle (C, OpenMP)"},
            "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


DECODE = dict(workload="turb512: 512^3 k^-5/3 spectral field, ZFP rate 2, full-volume decode "
                       "(2,097,152 blocks -> 512 MiB float32)", dims=(512, 512, 512), rate=2, seed=3)
WALK = dict(workload="turb512 walk: 512^3 k^-5/3 spectral field, ZFP rate 2, cache 25% of 2,097,152 blocks, "
                     "64 isovalues on a seeded +-0.02 random walk from 0, one at a time, cache reset per step",
            queries=64, seed=3, cache_fraction=0.25, cpu_queries=8)


def turb512_stream(ctx):
    """The 512^3 spectral field, ZFP-encoded at rate 2 on the GPU: (device
    words, host stream bytes, block count)."""
    import torch

    import bcmc
    from bcmc import datasets as D

    dims, rate = DECODE["dims"], DECODE["rate"]
    f = torch.from_numpy(D.turbulence(dims, DECODE["seed"])).cuda()
    words = bcmc.zfp_encode(ctx, f, rate)
    torch.cuda.synchronize()
    del f
    nb = int(np.prod([(d + 3) // 4 for d in dims]))
    host = words.cpu().numpy().view(np.uint8)[: nb * 8 * rate].copy()
    return words, host, nb


def decode_bench(ctx, flush, words, nb, reps: int = 10) -> dict:
    """Full-volume ZFP decode throughput: blocks * (8*rate + 256) B / event time."""
    import torch

    import bcmc

    rate = DECODE["rate"]
    out = torch.empty(nb * 64, dtype=torch.float32, device="cuda")
    L = bcmc._lib.load()
    torch.cuda.synchronize()
    s = torch.cuda.ExternalStream(ctx.stream)  # the library's stream: the kernel and the events share it

    def run():
        st = L.bcmc_zfp_decode_volume(ctx.handle, words.data_ptr(), nb, rate, out.data_ptr(), ctx.stream)
        if st != 0:
            raise RuntimeError(f"bcmc_zfp_decode_volume failed: {st}")

    for _ in range(3):
        run()
    times = []
    for _ in range(reps):
        flush.fill_(2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        run()
        e1.record(s)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    algo = nb * (8 * rate + 256)
    peak, peak_kind = _peaks()
    gbs = algo / (ms / 1000.0) / 1e9
    del out
    return {"workload": DECODE["workload"], "unit": "GB/s", "value": gbs, "ms": ms, "peak": peak,
            "peak_kind": peak_kind, "frac": gbs / peak, "algorithmic_bytes": algo,
            "kernel": "k_decode_volume", "l2": "flushed (512 MB write) before each rep"}


def walk_bench(ctx, flush, host_stream, steps: int, warmup: int, cpu: bool) -> dict:
    """The plain per-query path on the cache-bound 512^3 walk (js/run_benchmark.js
    style: a sequence of isovalues after a cache reset): iso-queries/s from CUDA
    events on the library's stream, per-query host latency, and the oracle on
    the walk's first queries."""
    import torch

    import bcmc
    from bcmc import datasets as D

    dims, rate = DECODE["dims"], DECODE["rate"]
    isos = [float(np.float32(v)) for v in D.random_walk(WALK["queries"], WALK["seed"])]
    c = bcmc.Context(ctx.device, initial_cache_fraction=WALK["cache_fraction"])
    mc = bcmc.CompressedMarchingCubes(c)
    mc.setCompressedVolume(host_stream, rate, dims)
    s = torch.cuda.ExternalStream(c.stream)

    def step(lat=None):
        mc.lruCache.reset()
        for iso in isos:
            t0 = time.perf_counter()
            mc.computeSurface(iso)
            if lat is not None:
                lat.append(1000.0 * (time.perf_counter() - t0))

    for _ in range(max(1, warmup)):
        step()
    times, lat = [], []
    for _ in range(max(1, steps)):
        flush.fill_(3)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        step(lat)
        e1.record(s)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    out = {"workload": WALK["workload"], "value": len(isos) / (ms / 1000.0), "unit": "queries/s",
           "ms_per_step": ms, "steps": max(1, steps), "cache_size": mc.stats()["cacheSize"],
           "p50_ms": float(np.percentile(lat, 50)), "p95_ms": float(np.percentile(lat, 95)),
           "p99_ms": float(np.percentile(lat, 99))}
    del mc
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        words = np.frombuffer(host_stream.tobytes() + bytes(16), dtype=np.uint64)
        m = oracle.CompressedMarchingCubes(words, rate, dims, initial_cache_fraction=WALK["cache_fraction"])
        k = WALK["cpu_queries"]
        m.compute_surface(isos[0])  # warm-up (threads, pages)
        m.cache_reset()
        t0 = time.perf_counter()
        for iso in isos[:k]:
            m.compute_surface(iso)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": k / dt, "unit": "queries/s", "cores": oracle.threads(), "kind": "port",
                               "sample": f"the walk's first {k} queries from a reset cache, CPU oracle (C, OpenMP)"}
    return out


RENDER = dict(width=1920, height=1080, reps=20)


def render_bench(mc, isos) -> dict:
    """The render pass (bcmc_render) on the mesh of the middle isovalue of the
    ct256 workload at 1920x1080, the reference's starting view (eye at +z,
    50 degree field of view), with and without fog.  Each call returns after
    its stream finished, so the host wall time per call is the frame time;
    the launch list attributes it to the kernels."""
    import torch

    import bcmc
    from bcmc import camera

    iso = float(isos[len(isos) // 2])
    mc.computeSurface(iso)
    n = mc.stats()["lastNumVertices"]
    vb = mc.vertexBuffer
    w, h = RENDER["width"], RENDER["height"]
    proj, eye = camera.default_view(w, h)
    out = {"workload": f"ct256 mesh at iso {iso:g}: {n // 3} triangles, {w}x{h}, starting view",
           "triangles": n // 3}
    ctx = mc.ctx
    for fog in (False, True):
        for _ in range(3):
            bcmc.render(ctx, vb, n, CONFIG["dims"], proj, eye, w, h, fog=fog)
        torch.cuda.synchronize()
        times = []
        for _ in range(RENDER["reps"]):
            t0 = time.perf_counter()
            rgba, _, tri = bcmc.render(ctx, vb, n, CONFIG["dims"], proj, eye, w, h, fog=fog)
            times.append(1000.0 * (time.perf_counter() - t0))
        ms = float(np.median(times))
        covered = int((tri >= 0).sum().item())
        out["fog" if fog else "plain"] = {"ms": ms, "frames_per_s": 1000.0 / ms,
                                          "mtriangles_per_s": n / 3 / ms / 1000.0, "covered_pixels": covered}
    return out


BATCH = dict(workload="256 queries over 8 resident volumes (32^3 blobs, 64^3 value noise, 96x128x80 "
                      "spectral, 128^3 blobs, 200^3 value noise, 256^3 spectral, 384x384x256 value noise, "
                      "512^3 spectral), ZFP rate 4, isovalues uniform within each volume's range",
             volumes=[("blobs", (32, 32, 32)), ("ct_like", (64, 64, 64)), ("turbulence", (96, 128, 80)),
                      ("blobs", (128, 128, 128)), ("ct_like", (200, 200, 200)), ("turbulence", (256, 256, 256)),
                      ("ct_like", (384, 384, 256)), ("turbulence", (512, 512, 512))],
             rate=4, queries=256, seed=4)


def _mc_share(mcs, queries) -> dict:
    """The plain path's marching-cubes share on a query mix: the same queries
    again with a perf tracker (CUDA-event stage times).  A batched or served
    path that kept only the MC work per query could reach at most
    wall time / MC time per query times the plain path's rate."""
    perf = {}
    t0 = time.perf_counter()
    for v, iso in queries:
        mcs[v].computeSurface(iso, perf)
    wall = (time.perf_counter() - t0) / len(queries)
    mc = float(np.sum(perf["computeVertices"])) / len(queries) / 1000.0
    stages = sum(float(np.sum(perf[k])) for k in ("computeActiveBlocks", "cacheUpdate", "decompression",
                                                  "computeVertices")) / len(queries) / 1000.0
    return {"mc_ms_per_query": 1000.0 * mc, "stages_ms_per_query": 1000.0 * stages,
            "wall_ms_per_query": 1000.0 * wall, "mc_share_of_wall": mc / wall,
            "max_speedup_if_only_mc_remains": wall / mc if mc > 0 else None}


def batched_bench(reps: int = 5) -> dict:
    """The batched engine against the plain per-query path on the same 256
    queries: iso-queries/s, per-query latency, and a bit-exact check of every
    query's vertices."""
    import torch

    import bcmc
    from bcmc import datasets as D

    rate = BATCH["rate"]
    ctx = bcmc.Context(0)  # plain path: the reference's initial cache of 5 % of the blocks
    streams, ranges = [], []
    for i, (kind, dims) in enumerate(BATCH["volumes"]):
        f = D.make_field(kind, dims, BATCH["seed"] + i)
        ranges.append((float(f.min()), float(f.max())))
        w = bcmc.zfp_encode(ctx, torch.from_numpy(f).cuda(), rate)
        torch.cuda.synchronize()
        nb = int(np.prod([(d + 3) // 4 for d in dims]))
        streams.append(w.cpu().numpy().view(np.uint8)[: nb * 64 * rate // 8].copy())
        del f, w
    rng = np.random.default_rng(BATCH["seed"])
    qs = []
    for i in range(BATCH["queries"]):
        v = i % len(streams)
        lo, hi = ranges[v]
        qs.append((v, float(np.float32(rng.uniform(lo + 0.05 * (hi - lo), hi - 0.05 * (hi - lo))))))
    total_blocks = sum(int(np.prod([(d + 3) // 4 for d in dims])) for _, dims in BATCH["volumes"])

    # plain per-query path: one CompressedMarchingCubes per volume
    mcs = []
    for (kind, dims), st in zip(BATCH["volumes"], streams):
        mc = bcmc.CompressedMarchingCubes(ctx)
        mc.setCompressedVolume(st, rate, dims)
        mcs.append(mc)
    for v, iso in qs:  # warm-up: caches grow to their working size
        mcs[v].computeSurface(iso)
    plain_lat = []
    t0 = time.perf_counter()
    for v, iso in qs:
        tq = time.perf_counter()
        mcs[v].computeSurface(iso)
        plain_lat.append(1000.0 * (time.perf_counter() - tq))
    plain_s = time.perf_counter() - t0
    mc_share = _mc_share(mcs, qs)

    # batched engine: every volume resident, one pool for all of them
    eng = bcmc.Engine(ctx, pool_slots=total_blocks, max_batch=BATCH["queries"])
    for (kind, dims), st in zip(BATCH["volumes"], streams):
        eng.addVolume(st, rate, dims)
    eng.run(qs)  # warm-up: decodes the blocks the batch needs
    tune = eng.autotune(qs)  # launch parameters for this batch size, by timing
    launches0 = bcmc._lib.load().bcmc_kernel_launches()
    batch_ms, dev_ms = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        res = eng.run(qs)
        batch_ms.append(1000.0 * (time.perf_counter() - t0))
        dev_ms.append(eng.stats()["last_batch_ms"])
    launches = bcmc._lib.load().bcmc_kernel_launches() - launches0

    # every query's vertices against the plain path, on the device
    allv = eng.vertexBuffer.torch()
    identical = True
    nverts = 0
    for i, (v, iso) in enumerate(qs):
        n = mcs[v].computeSurface(iso)
        r = res[i]
        nverts += n
        if int(r["num_vertices"]) != n:
            identical = False
            continue
        if n:
            off = int(r["vertex_offset"])
            if not torch.equal(mcs[v].vertexBuffer.torch()[:n], allv[off: off + n]):
                identical = False
    bm = float(np.median(batch_ms))
    # per-query latency (arrival -> result) with all the queries arriving at
    # once, through the continuous-batching server (two batches in flight)
    srv = bcmc.Server(eng, max_batch=BATCH["queries"])
    try:
        srv_lat, srv_s = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            tickets = [srv.submit(v, iso) for v, iso in qs]
            srv_lat.extend(srv.wait(t)[2] for t in tickets)
            srv_s.append(time.perf_counter() - t0)
    finally:
        srv.close()
    return {"workload": BATCH["workload"], "queries": len(qs), "vertices": nverts,
            "served_at_once": {"queries_per_s": len(qs) / float(np.median(srv_s)),
                               "p50_ms": float(np.percentile(srv_lat, 50)),
                               "p99_ms": float(np.percentile(srv_lat, 99)),
                               "what": "all queries submitted at once to bcmc_server; latency = arrival to result"},
            "plain": {"queries_per_s": len(qs) / plain_s, "p50_ms": float(np.percentile(plain_lat, 50)),
                      "p99_ms": float(np.percentile(plain_lat, 99))},
            "batched": {"queries_per_s": len(qs) / (bm / 1000.0), "batch_ms": bm,
                        "device_ms": float(np.median(dev_ms)), "p50_ms": bm, "p99_ms": float(np.max(batch_ms)),
                        "gpu_launches_per_batch": launches / reps},
            "autotune": tune,
            "plain_mc": mc_share,
            "speedup_qps": (len(qs) / (bm / 1000.0)) / (len(qs) / plain_s),
            "identical_to_plain": identical,
            "latency_note": "batched: a batch's queries all complete when the batch does (per-query latency = "
                            "batch wall time); served_at_once gives per-request latencies"}


SERVED = dict(workload="1024x1024x1080 uint16-range value noise (~60% background blocks, 17,694,720 blocks) "
                       "+ 256^3 value noise, 320^3 blobs, 384^3 spectral, 512^3 value noise; ZFP rate 4; Poisson "
                       "arrivals, volume weighted by size, isovalue uniform in its range; 40 GB slot pool; server batches of "
                       "one request, two in flight",
              big=(1024, 1024, 1080),
              others=[("ct_like", (256, 256, 256)), ("blobs", (320, 320, 320)), ("turbulence", (384, 384, 384)),
                      ("ct_like", (512, 512, 512))],
              rate=4, pool_bytes=40 << 30, seed=5, rates=(100.0, 200.0, 300.0, 400.0, 500.0, 600.0), seconds=4.0,
              # one request per batch, two in flight: a query of this mix averages 87 M vertices,
              # enough to fill the GPU on its own, so batching would only make each request wait
              # for its batch-mates (measured: equal-p99 ratios 0.7-1.0 at up to 256 per batch,
              # 1.1-1.9 at one)
              server_max_batch=1)


def served_bench() -> dict:
    """The continuous-batching server on the served mix against the plain
    per-query path: plain = one query at a time, back to back; served = open-loop
    Poisson arrivals at swept rates.  Throughput and latency percentiles."""
    import torch

    import bcmc
    from bcmc import datasets as D

    rate = SERVED["rate"]
    ctx = bcmc.Context(0)
    vols = []  # (dims, host stream, lo, hi)
    big = D.ct_uint16_torch(SERVED["big"], SERVED["seed"])
    w = bcmc.zfp_encode(ctx, big, rate)
    torch.cuda.synchronize()
    lo, hi = float(big.min()), float(big.max())
    del big
    nb = int(np.prod([(d + 3) // 4 for d in SERVED["big"]]))
    vols.append((SERVED["big"], w.cpu().numpy().view(np.uint8)[: nb * 64 * rate // 8].copy(), lo, hi))
    del w
    torch.cuda.empty_cache()
    for i, (kind, dims) in enumerate(SERVED["others"]):
        f = D.make_field(kind, dims, SERVED["seed"] + 1 + i)
        w = bcmc.zfp_encode(ctx, torch.from_numpy(f).cuda(), rate)
        torch.cuda.synchronize()
        nb = int(np.prod([(d + 3) // 4 for d in dims]))
        vols.append((dims, w.cpu().numpy().view(np.uint8)[: nb * 64 * rate // 8].copy(), float(f.min()),
                     float(f.max())))
        del f, w
    sizes = [float(np.prod(d)) for d, _, _, _ in vols]
    weights = [x / sum(sizes) for x in sizes]
    iso_lo = [lo + 0.05 * (hi - lo) for _, _, lo, hi in vols]
    iso_hi = [hi - 0.05 * (hi - lo) for _, _, lo, hi in vols]
    rng = np.random.default_rng(SERVED["seed"])

    def draw(n):
        ks = rng.choice(len(vols), size=n, p=weights)
        return [(int(k), float(np.float32(rng.uniform(iso_lo[k], iso_hi[k])))) for k in ks]

    # plain per-query path, back to back (closed loop)
    mcs = []
    for dims, st, _, _ in vols:
        mc = bcmc.CompressedMarchingCubes(ctx)
        mc.setCompressedVolume(st, rate, dims)
        mcs.append(mc)
    for v, iso in draw(40):  # warm-up: caches grow
        mcs[v].computeSurface(iso)
    plain_q = draw(200)
    lat = []
    t0 = time.perf_counter()
    for v, iso in plain_q:
        tq = time.perf_counter()
        mcs[v].computeSurface(iso)
        lat.append(1000.0 * (time.perf_counter() - tq))
    plain_qps = len(plain_q) / (time.perf_counter() - t0)
    mc_share = _mc_share(mcs, plain_q)
    del mcs
    torch.cuda.empty_cache()

    eng = bcmc.Engine(ctx, pool_slots=SERVED["pool_bytes"] // 256, max_batch=256, vertex_budget=1 << 31)
    for dims, st, _, _ in vols:
        eng.addVolume(st, rate, dims)
    warm = draw(64)
    while warm:  # warm-up: first decodes, graphs, buffer growth
        _, m = eng.run_admit(warm)
        warm = warm[m:]
    srv = bcmc.Server(eng, max_batch=SERVED["server_max_batch"])
    sweeps = []
    try:
        for r in SERVED["rates"]:
            n = max(50, int(r * SERVED["seconds"]))
            rep = srv.run_load(r, n, list(range(len(vols))), weights, iso_lo, iso_hi, seed=int(r))
            sweeps.append({k: rep[k] for k in ("offered_qps", "achieved_qps", "p50_ms", "p95_ms", "p99_ms",
                                                "mean_batch", "completed", "batches", "overlapped_batches")})
    finally:
        srv.close()
    st = eng.stats()
    p99_plain = float(np.percentile(lat, 99))

    def plain_open_loop(rate_qps, n=2000, seed=0):
        """The plain path as a FIFO single server under the same open-loop
        Poisson arrivals, from its measured per-query service times: request i
        starts at max(arrival_i, finish_{i-1}).  Exact for one FIFO server."""
        g = np.random.default_rng(seed)
        arrive = np.cumsum(g.exponential(1.0 / rate_qps, size=n))
        svc = np.asarray(lat)[np.arange(n) % len(lat)] / 1000.0
        finish = np.empty(n)
        t = 0.0
        for i in range(n):
            t = max(t, arrive[i]) + svc[i]
            finish[i] = t
        l_ms = 1000.0 * (finish - arrive)
        return {"offered_qps": rate_qps, "achieved_qps": n / (finish[-1] - arrive[0]),
                "p50_ms": float(np.percentile(l_ms, 50)), "p99_ms": float(np.percentile(l_ms, 99))}

    plain_sweep = [plain_open_loop(s["offered_qps"]) for s in sweeps]

    def plain_rate_at(p99_ms):
        """Highest offered rate the plain path sustains with p99 <= p99_ms."""
        lo, hi = 1.0, plain_qps
        for _ in range(30):
            mid = 0.5 * (lo + hi)
            r = plain_open_loop(mid)
            if r["p99_ms"] <= p99_ms and r["achieved_qps"] >= 0.95 * mid:
                lo = mid
            else:
                hi = mid
        return lo

    ratios = []
    for sv in sweeps:
        if sv["achieved_qps"] >= 0.95 * sv["offered_qps"]:
            ratios.append({"served_qps": sv["achieved_qps"], "p99_ms": sv["p99_ms"],
                           "plain_qps_at_same_p99": plain_rate_at(sv["p99_ms"])})
    for r in ratios:
        r["ratio"] = r["served_qps"] / r["plain_qps_at_same_p99"]
    best = max(ratios, key=lambda r: r["ratio"]) if ratios else None
    return {"workload": SERVED["workload"],
            "plain": {"queries_per_s": plain_qps, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": p99_plain,
                      "what": "back to back, one query at a time (service times)"},
            "plain_mc": mc_share,
            "overlapped_batches": sum(s.get("overlapped_batches", 0) for s in sweeps),
            "plain_open_loop": plain_sweep,
            "served": sweeps,
            "served_vs_plain_at_equal_p99": ratios,
            "best_ratio_at_equal_p99": best["ratio"] if best else None,
            "pool": {"slots": st["pool_slots"], "used": st["pool_used"], "decoded_blocks": st["decoded_blocks"],
                     "evicted_blocks": st["evicted_blocks"]}}


# DRAM bytes (read + write) per launch of k_mc on this workload, from one ncu
# capture of 16 consecutive launches (dram__bytes_read.sum + dram__bytes_write.sum,
# mean over one 16-isovalue sweep): a profile constant, reported as such
NCU_TRAFFIC = {"k_mc": 42.979e6}


def algorithmic_bytes(stage: str, st: dict, rate: int, total_blocks: int) -> float:
    """Algorithmic DRAM bytes per launch of each stage's kernel."""
    if stage == "computeVertices":  # k_mc: block data + ids/slots + vertices
        return st["numActiveBlocks"] * (256 + 4 + 4) + st["numVertices"] * 8 + st["numBlocksWithVertices"] * 8
    if stage == "decompression":  # k_decode_new + k_assign: compressed bits, the decoded
        # block staged, read back and written into its slot, ids
        return st["newDecompressed"] * (8 * rate + 3 * 256 + 8)
    if stage == "computeActiveBlocks":  # k_active: ranges, slots, flags
        return total_blocks * (8 + 4 + 4) + st["numActiveBlocks"] * 4
    if stage == "cacheUpdate":  # k_slots + sort: 3 slot arrays rw + sort passes
        return st["cacheSize"] * (12 + 12) + st["slotsAvailable"] * 16
    return 0.0


# The full per-leg record (per-rate sweeps, autotune choices, stage passes) goes
# to this file; the printed line keeps each leg's headline figures.
DETAIL = "gpurun_out/bench_detail.json"


def _pick(d, keys):
    return None if d is None else {k: d[k] for k in keys if k in d}


def _batched_summary(b):
    if b is None:
        return None
    return {"queries_per_s": b["batched"]["queries_per_s"], "plain_queries_per_s": b["plain"]["queries_per_s"],
            "speedup_qps": b["speedup_qps"], "p50_ms": b["batched"]["p50_ms"], "p99_ms": b["batched"]["p99_ms"],
            "plain_p99_ms": b["plain"]["p99_ms"], "identical_to_plain": b["identical_to_plain"],
            "served_at_once": {k: b["served_at_once"][k] for k in ("queries_per_s", "p50_ms", "p99_ms")},
            "max_speedup_if_only_mc_remains": b["plain_mc"]["max_speedup_if_only_mc_remains"]}


def _served_summary(sv):
    if sv is None:
        return None
    ok = [r for r in sv["served"] if r["achieved_qps"] >= 0.95 * r["offered_qps"]]
    top = max(ok, key=lambda r: r["achieved_qps"]) if ok else None
    return {"plain_queries_per_s": sv["plain"]["queries_per_s"], "plain_p99_ms": sv["plain"]["p99_ms"],
            "max_sustained_qps": top["achieved_qps"] if top else None, "p99_ms_at_max": top["p99_ms"] if top else None,
            "best_ratio_at_equal_p99": sv["best_ratio_at_equal_p99"],
            "ratios_at_equal_p99": [round(r["ratio"], 3) for r in sv["served_vs_plain_at_equal_p99"]],
            "overlapped_batches": sv["overlapped_batches"],
            "max_speedup_if_only_mc_remains": sv["plain_mc"]["max_speedup_if_only_mc_remains"]}


def run_gb300(args):
    import torch
    import torch.distributed as dist

    import bcmc

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    field, isos = make_volume()
    ctx = bcmc.Context(local, initial_cache_fraction=CONFIG["cache_fraction"])
    _, host_stream = encode_on_gpu(ctx, field)
    mc = bcmc.CompressedMarchingCubes(ctx)
    t0 = time.perf_counter()
    mc.setCompressedVolume(host_stream, CONFIG["rate"], CONFIG["dims"])
    load_s = time.perf_counter() - t0
    total_blocks = mc.totalBlocks
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")
    L = bcmc._lib.load()

    def step(perf=None, copy_out=None, lat=None, to_host=None, seq_host=None):
        mc.lruCache.reset()
        if seq_host is not None:  # the whole sweep in one call, transfers overlapping the next query
            return sum(mc.computeSurfacesToHost(isos, seq_host))
        n_tot = 0
        for iso in isos:
            t_q = time.perf_counter()
            if to_host is not None:
                n = mc.computeSurfaceToHost(float(iso), to_host)
            else:
                n = mc.computeSurface(float(iso), perf)
            if lat is not None:
                lat.append(1000.0 * (time.perf_counter() - t_q))
            if copy_out is not None:
                mc.copyVertices(copy_out)
            n_tot += n
        return n_tot

    for _ in range(max(args.warmup, 3)):
        step()
    # timed: device-resident
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    launches0 = L.bcmc_kernel_launches()
    lat = []
    # the headline pass: computeSurface without a perf tracker (the default
    # call; a tracker adds the stage-timing events to the query's graph)
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(None, None, lat)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    launches = L.bcmc_kernel_launches() - launches0
    # the stage pass: the same steps with a perf tracker, whose CUDA events
    # time each stage (and the dominant kernel for the roofline)
    perf = {}
    stage_times = []
    for _ in range(max(3, args.steps // 4)):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(perf)
        e1.record(stream)
        e1.synchronize()
        stage_times.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    ms = max_over_ranks(float(np.mean(times)), "cuda")
    value = world * len(isos) / (ms / 1000.0)

    # e2e: every query's vertices in pinned host memory, through the C ABI:
    # bcmc_compute_surfaces_host (the sweep in one call: each query's vertices
    # are copied out while the next query computes); for comparison
    # bcmc_compute_surface_host per query (the kernels store the vertices into
    # the host buffer) and bcmc_compute_surface + bcmc_copy_vertices
    vmax = 1 << 24
    pinned = torch.empty((vmax, 2), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    sweep_verts = step()
    pinned_seq = torch.empty((sweep_verts + 1024, 2), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)

    def e2e_pass(**kw):
        times, d2h = [], 0
        for _ in range(max(args.warmup, 3)):
            step(**kw)
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            n_tot = step(**kw)
            times.append(time.perf_counter() - t0)
            d2h = n_tot * 8
        return world * len(isos) / max_over_ranks(float(np.mean(times)), "cuda"), d2h

    e2e_value, d2h = e2e_pass(seq_host=pinned_seq)
    e2e_query_value, _ = e2e_pass(to_host=pinned)
    e2e_copy_value, _ = e2e_pass(copy_out=pinned)

    # roofline of the dominant stage (CUDA-event stage times of the stage pass)
    stages = ("computeActiveBlocks", "cacheUpdate", "decompression", "computeVertices")
    tot = {s: float(np.sum(perf[s])) for s in stages}
    dominant = max(stages, key=lambda s: tot[s])
    # per-launch algorithmic bytes, averaged over the queries of the timed steps
    nq = len(perf[dominant])
    stats_seq = []
    mc.lruCache.reset()
    for iso in isos:
        mc.computeSurface(float(iso))
        s = mc.stats()
        s["slotsAvailable"] = mc.lruCache.displayNumSlotsAvailable + s["newDecompressed"]
        stats_seq.append(s)
    bytes_per_launch = float(np.mean([algorithmic_bytes(dominant, s, CONFIG["rate"], total_blocks)
                                      for s in stats_seq]))
    avg_ms = tot[dominant] / nq
    peak, peak_kind = _peaks()
    achieved = bytes_per_launch / (avg_ms / 1000.0) / 1e9 if avg_ms > 0 else 0.0
    kernel_of = {"computeVertices": "k_mc", "decompression": "k_decode_new + k_assign (ZFP decode beside the cache update, slot assignment and copy)",
                 "computeActiveBlocks": "k_active", "cacheUpdate": "k_slots + radix sort"}

    decode = walk = None
    if not (args.no_decode and args.no_walk):
        turb_words, turb_host, turb_nb = turb512_stream(ctx)
        decode = decode_bench(ctx, flush, turb_words, turb_nb) if not args.no_decode else None
        del turb_words
        torch.cuda.empty_cache()
        walk = walk_bench(ctx, flush, turb_host, max(3, args.steps // 10), max(args.warmup, 3),
                          cpu=(rank == 0 and world == 1 and not args.no_cpu)) if not args.no_walk else None
    batched = batched_bench() if not args.no_batched else None
    served = served_bench() if not args.no_served else None
    render = render_bench(mc, isos) if not args.no_render else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        qps, threads, _ = cpu_oracle_time(field, isos, steps=1)
        cpu = {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
               "sample": "1 step (cache reset + 16 queries) of the same workload, CPU oracle (C, OpenMP)"}

    if rank == 0:
        e2e = {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": 4 * len(isos),
               "d2h_bytes_per_step": d2h,
               "what": "bcmc_compute_surfaces_host, the 16 isovalues in one call: each query's vertices "
                       "copied into pinned host memory while the next query computes (host wall time per step)",
               "per_query": {"value": e2e_query_value,
                             "what": "bcmc_compute_surface_host per query: vertices stored into pinned host "
                                     "memory by the kernels"},
               "compute_then_copy": {"value": e2e_copy_value,
                                     "what": "bcmc_compute_surface + bcmc_copy_vertices per query"}}
        roofline = {"bound": "hbm", "kernel": kernel_of[dominant], "achieved": achieved, "peak": peak,
                    "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                    "traffic": NCU_TRAFFIC.get(kernel_of[dominant]), "avg_launch_ms": avg_ms,
                    "algorithmic_bytes": bytes_per_launch,
                    "traffic_source": "a constant from one ncu capture of this kernel on this workload "
                                      "(dram bytes read+write per launch), not measured in this run"}
        line = {"metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded CT-like field, ZFP-encoded on the GPU by the project's encoder)",
                "config": {"workload": CONFIG["workload"], "l2": "flushed (512 MB write) between steps",
                           "parallelism": f"replicas x{world}"},
                "e2e": e2e,
                "roofline": roofline,
                "stage_ms_per_query": {s: tot[s] / nq for s in stages},
                "latency_ms": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                               "p99": float(np.percentile(lat, 99))},
                "decode": _pick(decode, ("value", "unit", "frac", "ms", "peak_kind")),
                "walk": _pick(walk, ("value", "unit", "p50_ms", "p99_ms", "cache_size")),
                "walk_cpu_baseline": _pick((walk or {}).get("cpu_baseline"), ("value", "unit", "cores", "kind")),
                "batched": _batched_summary(batched),
                "served": _served_summary(served),
                "render_ms": {k: render[k]["ms"] for k in ("plain", "fog")} if render else None,
                "gpu_launches": int(launches),
                "clocks": clk,
                "cpu_baseline": cpu,
                "detail_file": DETAIL}
        detail = dict(line, e2e=e2e, roofline=roofline, decode=decode, walk=walk, batched=batched, served=served,
                      render=render, stage_pass_ms_per_step=float(np.mean(stage_times)), volume_load_s=load_s,
                      latency_ms=dict(line["latency_ms"], queries=len(lat),
                                      what="host wall time of each computeSurface call"))
        try:
            os.makedirs(os.path.dirname(os.path.join(ROOT, DETAIL)), exist_ok=True)
            with open(os.path.join(ROOT, DETAIL), "w") as f:
                json.dump(detail, f, indent=1)
        except OSError:
            line["detail_file"] = None
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-decode", action="store_true", help="skip the full-volume decode leg")
    ap.add_argument("--no-walk", action="store_true", help="skip the 512^3 random-walk leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-engine leg")
    ap.add_argument("--no-served", action="store_true", help="skip the served (continuous batching) leg")
    ap.add_argument("--no-render", action="store_true", help="skip the render-pass leg")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
