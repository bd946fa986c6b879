"""The MC kernels' vertex code (csrc/mc_vertex.cuh: the emit table built at
compile time from the tri table, the table of packed fixed-axis positions and
mc_vertex), compiled as host C++, against the oracle's emit
(compute_block_vertices.comp:62-74,161-162, block_vertex_position.comp:9-17,
restated below in float32 in the reference's operation order) for every
vertex of every case of the oracle's tri table, random cells and corner
values, bit for bit.  Ties (a corner equal to the isovalue), near-equal
corners (the 0.001 test) and values far from the isovalue are included."""
import ctypes
import os
import shlex
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmc_vertex_host.so")

# compute_block_vertices.comp:10-23: each edge's two corners, and each corner's
# offset in the cell (compute_vertex_values.comp:48-57), in the reference's order
EDGE = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (6, 5), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
CORNER = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
F = np.float32


@pytest.fixture(scope="module")
def host_mc():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "host_device", "mc_vertex_host.cpp")
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", os.path.join(HERE, "host_device"),
           "-I", os.path.join(ROOT, "webgpu-bcmc_gb300", "csrc"), src, "-o", LIB]
    cmd += shlex.split(os.environ.get("BCMC_HOST_CXXFLAGS", ""))  # e.g. sanitizers
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(LIB)
    lib.mc_case_count.argtypes = [ctypes.c_uint32]
    lib.mc_case_count.restype = ctypes.c_uint32
    lib.mc_vertex_host.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_float]
    lib.mc_vertex_host.restype = ctypes.c_uint32
    return lib


def _quantize(p):
    """block_vertex_position.comp:9-17 as the oracle's compress_position: u32()
    of ((p - 0.5) * 0.25) * 1023, truncating and saturating, low 10 bits."""
    f = F(F(F(p - F(0.5)) * F(0.25)) * F(1023.0))
    q = 0 if not f > 0 else (0xFFFFFFFF if f >= F(4294967296.0) else int(f))
    return q & 0x3FF


def _ref_vertex(tri, c, k, cc, corners, iso):
    v0, v1 = EDGE[int(tri[c, k])]
    fa, fb = corners[v0], corners[v1]
    with np.errstate(all="ignore"):
        tt = F(0.0) if abs(F(fa - fb)) < F(0.001) else F(F(iso - fa) / F(fb - fa))
        vp = (F(cc % 4), F((cc // 4) % 4), F(cc // 16))
        q = []
        for ax in range(3):
            a, b = CORNER[v0][ax], CORNER[v1][ax]
            lerp = F(F(a) + F(tt * F(b - a)))
            q.append(_quantize(F(F(lerp + vp[ax]) + F(0.5))))
    return (q[0] << 20) | (q[1] << 10) | q[2]


def test_case_counts_match_oracle(host_mc, oracle):
    for c in range(256):
        assert host_mc.mc_case_count(c) == oracle.case_vertex_count(c), c


@pytest.mark.parametrize("seed", range(4))
def test_every_vertex_of_every_case_matches_oracle(host_mc, oracle, seed):
    tri = oracle.tri_table()
    rs = np.random.default_rng(seed)
    for c in range(1, 255):
        n = oracle.case_vertex_count(c)
        for trial in range(3):
            iso = F(rs.uniform(-2.0, 2.0))
            # corners inside (<= iso) for the case's bits, outside otherwise
            d = rs.exponential(0.5, size=8).astype(F)
            if trial == 1:
                d = (d * F(1e-3)).astype(F)  # near-equal corners (the 0.001 test)
            corners = np.array([iso - d[i] if (c >> i) & 1 else iso + d[i] + F(1e-6) for i in range(8)], dtype=F)
            if trial == 2:
                corners[rs.integers(0, 8)] = iso if (c >> 0) & 1 else corners[0]  # a tie on some corner
                if ((corners <= iso).astype(int) * (1 << np.arange(8))).sum() != c:
                    continue
            cc = int(rs.integers(0, 64))
            buf = corners.ctypes.data
            for k in range(n):
                got = host_mc.mc_vertex_host(c, k, cc, buf, float(iso))
                want = _ref_vertex(tri, c, k, cc, corners, iso)
                assert got == want, (c, k, cc, trial, hex(got), hex(want))
