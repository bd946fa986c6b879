"""ExclusiveScanner / StreamCompact / RadixSorter drop-ins on the GPU vs the
oracle (the reference's algorithms restated on the CPU)."""
import numpy as np
import pytest

import bcmc
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

SCAN_SIZES = [0, 1, 2, 31, 511, 512, 513, 4095, 4096, 4097, 65535, 65536, 262144 + 17, 1 << 20, 17694720]


@pytest.mark.parametrize("n", SCAN_SIZES)
def test_exclusive_scan(ctx, oracle, n):
    import torch

    rs = np.random.default_rng(n)
    pipe = bcmc.ExclusiveScanPipeline(ctx)
    aligned = pipe.getAlignedSize(n)
    host = np.zeros(max(aligned, 1), dtype=np.uint32)
    # mostly 0/1 flags, some large values so the uint32 sum wraps
    host[:n] = rs.integers(0, 2, size=n).astype(np.uint32)
    if n > 10:
        host[rs.integers(0, n, size=5)] = np.uint32(0xF0000000)
    buf = to_dev(host)
    scanner = pipe.prepareGPUInput(buf, aligned)
    total = scanner.scan(n)
    ref, ref_total = oracle.exclusive_scan(host, n, aligned)
    got = to_host(buf, np.uint32)
    assert total == ref_total
    assert np.array_equal(got[:n], ref[:n])
    if n < aligned:
        assert got[n] == ref_total
    del torch


def test_scan_rejects_unaligned_input(ctx):
    pipe = bcmc.ExclusiveScanPipeline(ctx)
    with pytest.raises(bcmc.BcmcError):
        pipe.prepareGPUInput(to_dev(np.zeros(100, np.uint32)), 100)


def test_scan_prepare_input_from_cpu(ctx):
    pipe = bcmc.ExclusiveScanPipeline(ctx)
    data = np.arange(1, 1001, dtype=np.uint32)
    s = pipe.prepareInput(data)
    assert s.scan(1000) == int(data.sum())
    s = pipe.prepareInput(data)
    assert s.scan(10) == 55  # a shorter dataSize within the same buffer
    got = s.inputBuf.cpu().numpy().view(np.uint32)
    assert list(got[:11]) == [0, 1, 3, 6, 10, 15, 21, 28, 36, 45, 55]
    assert got[11] == 12  # untouched beyond dataSize + 1


@pytest.mark.parametrize("n", [0, 1, 100, 65280, 65281, 300000])
def test_stream_compact(ctx, oracle, n):
    rs = np.random.default_rng(n + 1)
    flags = (rs.random(n) < 0.3).astype(np.uint32)
    offs, tot = oracle.exclusive_scan(flags, n, n)
    out = to_dev(np.zeros(max(tot, 1), np.uint32))
    bcmc.StreamCompact(ctx).compactActiveIDs(n, to_dev(flags) if n else to_dev(np.zeros(1, np.uint32)),
                                             to_dev(offs) if n else to_dev(np.zeros(1, np.uint32)), out)
    assert np.array_equal(to_host(out, np.uint32)[:tot], oracle.compact(flags, offs, n, tot))


SORT_CASES = [(1, 3), (7, 2), (63, 4), (64, 5), (65, 5), (200, 3), (1000, 50), (4095, 7), (4096, 1),
              (4097, 3), (100000, 40), (262145, 100000), (1 << 20, 1 << 31), (524288, 4)]


@pytest.mark.parametrize("n,kmax", SORT_CASES)
@pytest.mark.parametrize("reverse", [True, False])
def test_radix_sort_by_key(ctx, oracle, n, kmax, reverse):
    rs = np.random.default_rng(n * 3 + int(reverse))
    keys = rs.integers(0, kmax, size=n, dtype=np.uint64).astype(np.uint32)
    vals = rs.permutation(n).astype(np.uint32)
    k_dev, v_dev = to_dev(keys), to_dev(vals)
    sorter = bcmc.RadixSorter(ctx)
    sorter.sort(k_dev, v_dev, n, reverse)
    ref_k, ref_v = oracle.sort_by_key(keys, vals, reverse)
    assert np.array_equal(to_host(v_dev, np.uint32), ref_v)
    assert np.array_equal(to_host(k_dev, np.uint32), ref_k)


def test_radix_sort_all_equal_and_wide_keys(ctx, oracle):
    rs = np.random.default_rng(2)
    for keys in (np.full(5000, 7, np.uint32), rs.integers(0, 2**32 - 1, size=70000, dtype=np.uint64).astype(np.uint32)):
        n = len(keys)
        vals = np.arange(n, dtype=np.uint32)
        for reverse in (True, False):
            k_dev, v_dev = to_dev(keys), to_dev(vals)
            bcmc.RadixSorter(ctx).sort(k_dev, v_dev, n, reverse)
            _, ref_v = oracle.sort_by_key(keys, vals, reverse)
            assert np.array_equal(to_host(v_dev, np.uint32), ref_v)
