"""The product's device ZFP decoder (csrc/zfp_device.cuh), compiled as host
C++, against the oracle's decode (shaders/zfp_decompress.comp:195-384): every
rate from 1 to 32 bits per value, random bit streams (dense, sparse, single
bits, zero blocks) and encoded fields, compared bit for bit.  This covers the
group-test parse (budget and coefficient-63 limits, 64-bit raw reads, leading
empty planes) and the plane deposit without a GPU.  The device encoder (the
reference only decodes; it makes the benchmark inputs) is checked the same way
against the oracle's encoder, stream word for word."""
import ctypes
import os
import shlex
import shutil
import subprocess

import numpy as np
import pytest

from bcmc import datasets as D

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdecoder_host.so")


@pytest.fixture(scope="module")
def host_decoder():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "host_device", "decoder_host.cpp")
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", os.path.join(HERE, "host_device"),
           "-I", os.path.join(ROOT, "webgpu-bcmc_gb300", "csrc"), src, "-o", LIB]
    cmd += shlex.split(os.environ.get("BCMC_HOST_CXXFLAGS", ""))  # e.g. sanitizers
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(LIB)
    lib.decode_blocks_host.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p]
    lib.decode_blocks_host.restype = None

    def decode(words, nb, rate):
        words = np.ascontiguousarray(words, dtype=np.uint64)
        assert words.size >= nb * rate
        out = np.empty(nb * 64, dtype=np.float32)
        lib.decode_blocks_host(words.ctypes.data, nb, rate, out.ctypes.data)
        return out

    return decode


def _bits(a):
    return np.asarray(a, dtype=np.float32).view(np.uint32)


def _random_stream(rs, nb, rate, kind):
    w = rs.integers(0, 2**63, size=nb * rate + 2, dtype=np.uint64)
    w |= rs.integers(0, 2, size=w.shape, dtype=np.uint64) << np.uint64(63)
    if kind == "sparse":
        for _ in range(3):
            w &= rs.integers(0, 2**63, size=w.shape, dtype=np.uint64) | (
                rs.integers(0, 2, size=w.shape, dtype=np.uint64) << np.uint64(63))
    elif kind == "single":
        w = np.uint64(1) << rs.integers(0, 64, size=w.shape).astype(np.uint64)
    # most blocks nonzero (header flag set), some zero blocks
    start = np.arange(nb, dtype=np.uint64) * np.uint64(64 * rate)
    flag = rs.integers(0, 8, size=nb) != 0
    idx = (start[flag] >> np.uint64(6)).astype(np.int64)
    w[idx] |= np.uint64(1)
    w[(start[~flag] >> np.uint64(6)).astype(np.int64)] &= ~np.uint64(1)
    return w


@pytest.mark.parametrize("rate", [1, 2, 3, 4, 5, 8, 12, 16, 24, 32])
@pytest.mark.parametrize("kind", ["dense", "sparse", "single"])
def test_random_streams_match_oracle(host_decoder, oracle, rate, kind):
    rs = np.random.default_rng(1000 * rate + len(kind))
    nb = 3000
    w = _random_stream(rs, nb, rate, kind)
    got = host_decoder(w, nb, rate)
    ref = oracle.decode_volume(w, nb, 64 * rate)
    assert np.array_equal(_bits(got), _bits(ref))


@pytest.mark.parametrize("kind,dims,rate", [("turbulence", (64, 64, 64), 2), ("turbulence", (48, 48, 48), 1),
                                            ("ct_like", (64, 64, 64), 4), ("ct_like", (48, 40, 36), 2),
                                            ("blobs", (48, 48, 48), 8), ("turbulence", (32, 32, 32), 16)])
def test_encoded_fields_match_oracle(host_decoder, oracle, kind, dims, rate):
    f = D.make_field(kind, dims, 3)
    w = oracle.zfp_encode(f, rate)
    nb = int(np.prod(oracle.padded_blocks(dims)))
    got = host_decoder(w, nb, rate)
    ref = oracle.decode_volume(w, nb, 64 * rate)
    assert np.array_equal(_bits(got), _bits(ref))


@pytest.fixture(scope="module")
def host_encoder(host_decoder):
    lib = ctypes.CDLL(LIB)  # built by host_decoder
    lib.encode_blocks_host.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p]
    lib.encode_blocks_host.restype = None

    def encode(field, rate):
        """field [z, y, x] with every extent a multiple of 4: its blocks
        gathered as the encode kernel gathers them, encoded one by one."""
        Z, Y, X = field.shape
        blocks = np.ascontiguousarray(
            field.reshape(Z // 4, 4, Y // 4, 4, X // 4, 4).transpose(0, 2, 4, 1, 3, 5).reshape(-1, 64),
            dtype=np.float32)
        nb = blocks.shape[0]
        words = np.zeros(nb * rate, dtype=np.uint64)
        lib.encode_blocks_host(blocks.ctypes.data, nb, rate, words.ctypes.data)
        return words

    return encode


def _special_field(rs):
    """Blocks of zeros, constants, denormals, huge and tiny magnitudes, mixed
    signs and values just below a power of two, on a 16^3 grid of 64 blocks."""
    f = rs.standard_normal((16, 16, 16)).astype(np.float32)
    f *= np.float32(10.0) ** rs.integers(-30, 30, size=f.shape).astype(np.float32)
    b = f.reshape(4, 4, 4, 4, 4, 4)  # [bz, z, by, y, bx, x] views of blocks
    b[0, :, 0, :, 0, :] = 0.0
    b[0, :, 0, :, 1, :] = 3.0
    b[0, :, 0, :, 2, :] = np.float32(1e-40) * rs.standard_normal((4, 4, 4)).astype(np.float32)
    b[0, :, 0, :, 3, :] = np.float32(np.nextafter(np.float32(2.0), np.float32(0.0)))
    b[1, :, 0, :, 0, :] = np.float32(3.0e38) * np.sign(rs.standard_normal((4, 4, 4))).astype(np.float32)
    b[1, :, 0, :, 1, :] = -np.float32(1.0)
    b[1, :, 0, 0, 1, 0] = np.float32(1.0)
    return f


@pytest.mark.parametrize("rate", [1, 2, 4, 8, 16, 32])
def test_device_encoder_matches_oracle_encoder(host_encoder, oracle, rate):
    rs = np.random.default_rng(77 + rate)
    fields = [D.make_field("turbulence", (32, 32, 32), 3), D.make_field("ct_like", (32, 32, 32), 4),
              D.make_field("blobs", (32, 32, 32), 5), _special_field(rs)]
    for f in fields:
        nb = f.size // 64
        got = host_encoder(f, rate)
        ref = oracle.zfp_encode(f, rate)[: nb * rate]
        assert np.array_equal(got, ref)
