"""Readers of the scan, compaction and LRU fixtures (tests/golden/scan_compact.npz,
lru_seq.npz, lru_pipeline.npz, generated by tests/golden/make_golden.py from the
reference's own scan, compaction, sort and LRU shaders driven as
js/exclusive_scan.js, js/stream_compact.js and js/lru_cache.js drive them).
Shared by the oracle's CPU tests and the CUDA path's GPU tests; every value is
integer data, compared exactly."""
import hashlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()


def scan_cases():
    """(n, input u32 array, fixture dict view, index) per scan/compaction case."""
    g = np.load(os.path.join(GOLDEN, "scan_compact.npz"))
    for i in range(int(g["cases"])):
        n = int(g[f"n_{i}"])
        raw = g[f"in_{i}"]
        if str(g[f"kind_{i}"]) == "flags":
            v = np.unpackbits(raw)[:n].astype(np.uint32)
        else:
            v = raw.astype(np.uint32)
        yield n, v, g, i


def check_scan(g, i, n, scanned: np.ndarray, total: int):
    assert total == int(g[f"total_{i}"]), (n, total)
    if f"scan_{i}" in g:
        assert np.array_equal(scanned[:n], g[f"scan_{i}"]), n
    assert sha(scanned[:n]) == str(g[f"scan_sha_{i}"]), n


def check_compact(g, i, n, ids: np.ndarray):
    assert len(ids) == int(g[f"compact_count_{i}"]), n
    if f"compact_{i}" in g:
        assert np.array_equal(ids, g[f"compact_{i}"]), n
    assert sha(ids) == str(g[f"compact_sha_{i}"]), n


def lru_sequences():
    """Per sequence: (total, initial, steps, reset_at, [per-update record])."""
    g = np.load(os.path.join(GOLDEN, "lru_seq.npz"))
    for s in range(int(g["seqs"])):
        total, initial, steps, reset_at = (int(x) for x in g[f"s{s}_spec"])
        recs = []
        for step in range(steps):
            p = f"s{s}_{step}_"
            rec = {"total": total, "needed": np.unpackbits(g[p + "needed"])[:total].astype(np.uint32),
                   "new": g[p + "new"],
                   "display": int(g[p + "display"]), "cache_size": int(g[p + "cache_size"])}
            for k in ("item_slots", "age", "avail", "item"):
                rec[k] = g[p + k] if p + k in g else str(g[p + k + "_sha"])
            recs.append(rec)
        yield total, initial, steps, reset_at, recs


def check_lru_state(rec, state: dict, where):
    """`state`: item_slots (at least rec["total"] items), age, avail, item (one per slot)."""
    for k in ("item_slots", "age", "avail", "item"):
        want = rec[k]
        got = np.ascontiguousarray(state[k])
        if k == "item_slots":
            got = got[: rec["total"]]
        if isinstance(want, str):
            assert sha(got.view(np.uint32)) == want, (where, k)
        else:
            assert np.array_equal(got.view(np.uint32), np.asarray(want).view(np.uint32)), (where, k)


def lru_pipeline_cases():
    """Per case: (mc fixture name, cache fraction, isovalues, reset_at, [per-query record])."""
    g = np.load(os.path.join(GOLDEN, "lru_pipeline.npz"))
    for c in range(int(g["cases"])):
        p = f"c{c}_"
        isos = g[p + "isos"]
        recs = []
        for qi in range(len(isos)):
            q = f"{p}{qi}_"
            rec = {"counts": [int(x) for x in g[q + "counts"]], "mesh_sha": str(g[q + "mesh_sha"])}
            for k in ("item_slots", "age", "avail", "item"):
                rec[k] = g[q + k]
            rec["total"] = len(rec["item_slots"])
            recs.append(rec)
        yield str(g[p + "name"]), float(g[p + "frac"]), isos, int(g[p + "reset_at"]), recs
