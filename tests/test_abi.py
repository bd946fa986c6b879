"""The C-ABI library builds, loads and exports every entry point of
include/bcmc.h -- no GPU needed (no compute calls are made)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from bcmc import _lib


def _header_functions():
    src = open(_lib.HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bcmc_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_every_header_symbol(lib_built):
    assert os.path.exists(lib_built)
    L = _lib.load()
    names = _header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the ctypes declarations cover exactly the header
    assert sorted(_lib.SIGNATURES) == names


def test_host_side_sizes_match_reference_formulas(lib_built, oracle):
    L = _lib.load()
    for n in (0, 1, 63, 64, 65, 511, 512, 513, 4097, 1 << 20):
        assert L.bcmc_scan_aligned_size(n) == (n + 511) // 512 * 512  # exclusive_scan.js:95-97
        chunks = -(-n // 64)
        p = 1 if chunks else 0
        while 0 < p < chunks:
            p <<= 1
        assert L.bcmc_sort_aligned_size(n) == p * 64  # radix_sort_by_key.js:155-158
        assert L.bcmc_sort_aligned_size(n) == oracle.sort_aligned_size(n)
    for dims in ((64, 64, 64), (13, 7, 9), (1024, 1024, 1080)):
        for rate in (1, 2, 4, 8):
            assert L.bcmc_zfp_stream_words(_lib.dims3(dims), rate) == oracle.stream_words(dims, 64 * rate)


def test_argument_errors_need_no_device(lib_built):
    L = _lib.load()
    out = C.c_void_p()
    assert L.bcmc_volume_create(None, None, 0, 4, _lib.dims3((4, 4, 4)), None, C.byref(out)) == 1
    assert L.bcmc_compute_surface(None, 0.5, None, None) == 1
    assert L.bcmc_lru_update(None, None, None, None) == 1
    assert L.bcmc_sort_pairs_u32(None, None, None, 4, 0, None) == 1
    assert L.bcmc_ctx_create(None, None) == 1
    bad = _lib.bcmc_opts(0, 0.0, 0)
    assert L.bcmc_ctx_create(C.byref(bad), C.byref(out)) == 1  # cache fraction must be in (0, 1]


def test_context_without_device_reports_an_error(lib_built):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    L = _lib.load()
    out = C.c_void_p()
    rc = L.bcmc_ctx_create(None, C.byref(out))
    assert rc in (1, 3) and not out.value


def test_short_stream_is_refused_before_the_kernel():
    """The decode wrappers check the device stream's length (the C calls take
    none); a short buffer raises before anything is launched."""
    import bcmc

    class Fake:  # stands in for a device tensor: only its size is looked at
        def numel(self):
            return 10

        def element_size(self):
            return 8

    with pytest.raises(ValueError):
        bcmc._check_stream(Fake(), 8, 2)  # 8 blocks at rate 2 need 16 words
    bcmc._check_stream(Fake(), 5, 2)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No CPU fallback: without the built library every entry of the host side
    raises instead of computing anything."""
    import bcmc

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libbcmc_gb300.so"))
    with pytest.raises(ImportError, match="no CPU fallback"):
        _lib.load()
    with pytest.raises(ImportError):
        bcmc.Context(0)
