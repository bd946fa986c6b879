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


_C_HOST = r"""
#include <stdio.h>
#include "bcmc.h"
int main(void)
{
    bcmc_opts opts;
    bcmc_ctx* ctx = NULL;
    const uint32_t dims[3] = {13, 7, 9};
    bcmc_opts_default(&opts);
    bcmc_status st = bcmc_ctx_create(&opts, &ctx);
    printf("%d %u %u %llu\n", (int)st, bcmc_scan_aligned_size(1000), bcmc_sort_aligned_size(1000),
           (unsigned long long)bcmc_zfp_stream_words(dims, 4));
    if (st == BCMC_OK) bcmc_ctx_destroy(ctx);
    return 0;
}
"""


def test_header_is_c99_and_links_from_c(lib_built, tmp_path):
    """A C host (a cgo or FFI binding compiles the header as C) builds against
    include/bcmc.h with -std=c99 -pedantic and warnings as errors, links the
    library and calls it."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "host.c"
    src.write_text(_C_HOST)
    exe = tmp_path / "host"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.dirname(_lib.HEADER),
                        str(src), "-L", libdir, "-lbcmc_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    st, scan, sort, words = (int(x) for x in r.stdout.split())
    assert st in (0, 3)  # a context on a GPU machine, BCMC_E_CUDA without one
    assert (scan, sort) == (1024, 1024)
    assert words == (4 * 2 * 3) * 4 + 1  # 24 blocks of 4 u64 words, one pad word


_NULL_CALLS = r"""
import ctypes as C, json, sys
from bcmc import _lib
L = _lib.load()
ints = (C.c_uint8, C.c_int, C.c_int32, C.c_uint32, C.c_int64, C.c_uint64, C.c_size_t)
for name in sorted(_lib.SIGNATURES):
    rt, args = _lib.SIGNATURES[name]
    vals = [0.0 if a in (C.c_float, C.c_double) else (0 if a in ints else None) for a in args]
    print(name, flush=True)  # the last name printed is the culprit if the call crashes
    r = getattr(L, name)(*vals)
    print(json.dumps({"name": name, "r": r if r is None or isinstance(r, int) else str(r)}), flush=True)
"""


def test_every_entry_point_refuses_null_arguments(lib_built):
    """Each entry point of include/bcmc.h, called with null pointers and zero
    sizes, returns an error status (or, for the size helpers, zero) instead of
    dereferencing anything; no device is needed for that."""
    import subprocess
    import sys
    import json

    pkg = os.path.dirname(os.path.dirname(_lib.__file__))
    r = subprocess.run([sys.executable, "-c", _NULL_CALLS], cwd=pkg, capture_output=True, text=True, timeout=120,
                       env=dict(os.environ, PYTHONPATH=pkg))
    lines = r.stdout.splitlines()
    assert r.returncode == 0, (lines[-1:] if lines else None, r.stderr[-2000:])
    got = {d["name"]: d["r"] for d in (json.loads(l) for l in lines if l.startswith("{"))}
    assert sorted(got) == sorted(_lib.SIGNATURES)
    status = {n for n, (rt, _) in _lib.SIGNATURES.items() if rt is C.c_int}
    assert len(status) >= 40
    for n in status - {"bcmc_scan_exclusive_u32_noalloc"}:
        assert got[n] == 1, (n, got[n])  # BCMC_E_ARG
    # n = 0 with null pointers is a valid empty scan: OK with a device, a
    # set-up error (BCMC_E_CUDA) without one
    assert got["bcmc_scan_exclusive_u32_noalloc"] in (0, 3)
    for n in ("bcmc_scan_aligned_size", "bcmc_sort_aligned_size", "bcmc_zfp_stream_words"):
        assert got[n] == 0, n
    assert got["bcmc_ctx_stream"] is None
