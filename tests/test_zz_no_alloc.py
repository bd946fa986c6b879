"""bcmc_scan_exclusive_u32_noalloc (no reference counterpart): the exclusive
scan without a context or any device allocation, checked against the
context-based bcmc_scan_exclusive_u32_async on the same inputs, two calls in a
row.  Integer work: results must be identical.  Collected last, so it also
runs after every other test in one process; it passes on its own as well."""
import ctypes as C

import numpy as np
import pytest

from bcmc import _lib

BCMC_E_LIMIT = 7


def _scan_np(a: np.ndarray):
    c = np.cumsum(a.astype(np.uint64)) & 0xFFFFFFFF
    excl = np.concatenate([[0], c[:-1]]).astype(np.uint32)
    total = int(c[-1]) if len(a) else 0
    return excl, total


@pytest.mark.gpu
def test_noalloc_scan_matches_context_scan_two_calls_in_a_row(ctx):
    import torch

    L = _lib.load()
    rng = np.random.default_rng(1234)
    # multi-tile with a ragged last tile, then a smaller one that reuses the
    # scratch the first call left behind
    sizes = (3 * 4096 * 37 + 1234, 4096 * 5 + 3)
    inputs = [rng.integers(0, 1 << 31, size=n, dtype=np.uint64).astype(np.uint32) for n in sizes]
    dev_in = [torch.from_numpy(a.view(np.int32).copy()).cuda() for a in inputs]
    out_ref = [torch.empty_like(t) for t in dev_in]
    out_na = [torch.empty_like(t) for t in dev_in]
    tot_ref = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    tot_na = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    # existing entry point (context scratch) on torch's stream
    for i, n in enumerate(sizes):
        st = L.bcmc_scan_exclusive_u32_async(ctx.handle, C.c_void_p(dev_in[i].data_ptr()),
                                             C.c_void_p(out_ref[i].data_ptr()), n,
                                             C.c_void_p(tot_ref.data_ptr() + 4 * i), C.c_void_p(stream))
        assert st == 0
    torch.cuda.synchronize()

    # first no-alloc call does the per-context set-up; the rest must not allocate
    assert L.bcmc_scan_exclusive_u32_noalloc(None, None, 0, C.c_void_p(tot_na.data_ptr()),
                                             C.c_void_p(stream)) == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    launches_before = L.bcmc_kernel_launches()
    for i, n in enumerate(sizes):  # two calls in a row, same stream, no sync between
        st = L.bcmc_scan_exclusive_u32_noalloc(C.c_void_p(dev_in[i].data_ptr()),
                                               C.c_void_p(out_na[i].data_ptr()), n,
                                               C.c_void_p(tot_na.data_ptr() + 4 * i), C.c_void_p(stream))
        assert st == 0
    torch.cuda.synchronize()
    assert L.bcmc_kernel_launches() - launches_before == 2 * len(sizes)
    assert torch.cuda.mem_get_info()[0] == free_before

    for i, n in enumerate(sizes):
        got = out_na[i].cpu().numpy().view(np.uint32)
        ref = out_ref[i].cpu().numpy().view(np.uint32)
        excl, total = _scan_np(inputs[i])
        np.testing.assert_array_equal(got, ref)
        np.testing.assert_array_equal(got, excl)
        assert int(tot_na[i].item()) & 0xFFFFFFFF == int(tot_ref[i].item()) & 0xFFFFFFFF == total


@pytest.mark.gpu
def test_noalloc_scan_in_place_default_stream_and_limits(ctx):
    import torch

    L = _lib.load()
    rng = np.random.default_rng(99)
    a = rng.integers(0, 1000, size=4096 * 3 + 17, dtype=np.uint32)
    t = torch.from_numpy(a.view(np.int32).copy()).cuda()
    tot = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    # in place, on the legacy default stream (NULL)
    assert L.bcmc_scan_exclusive_u32_noalloc(C.c_void_p(t.data_ptr()), C.c_void_p(t.data_ptr()), len(a),
                                             C.c_void_p(tot.data_ptr()), None) == 0
    torch.cuda.synchronize()
    excl, total = _scan_np(a)
    np.testing.assert_array_equal(t.cpu().numpy().view(np.uint32), excl)
    assert int(tot.item()) == total
    # n = 0 writes a zero total
    assert L.bcmc_scan_exclusive_u32_noalloc(None, None, 0, C.c_void_p(tot.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert int(tot.item()) == 0
    # sizes above the limit are refused before anything is launched
    before = L.bcmc_kernel_launches()
    assert L.bcmc_scan_exclusive_u32_noalloc(C.c_void_p(t.data_ptr()), C.c_void_p(t.data_ptr()),
                                             (1 << 26) + 1, None, None) == BCMC_E_LIMIT
    assert L.bcmc_kernel_launches() == before
    # null buffers with n > 0
    assert L.bcmc_scan_exclusive_u32_noalloc(None, None, 5, None, None) == 1
    # the largest size accepted
    big = torch.ones(1 << 26, dtype=torch.int32, device="cuda")
    assert L.bcmc_scan_exclusive_u32_noalloc(C.c_void_p(big.data_ptr()), C.c_void_p(big.data_ptr()), 1 << 26,
                                             C.c_void_p(tot.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert int(tot.item()) == 1 << 26
    assert torch.equal(big[:: 1 << 13].cpu(), torch.arange(0, 1 << 26, 1 << 13, dtype=torch.int32))
