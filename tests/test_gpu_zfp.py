"""ZFP fixed-rate codec on the GPU vs the oracle, bit for bit."""
import numpy as np
import pytest

import bcmc
from bcmc import datasets as D
from gpu_util import bits, to_dev, to_host

pytestmark = pytest.mark.gpu

CASES = [((16, 16, 16), 8, "blobs"), ((13, 7, 9), 4, "blobs"), ((64, 64, 64), 8, "blobs"),
         ((48, 40, 36), 2, "turbulence"), ((37, 33, 29), 4, "ct_like"), ((5, 3, 6), 1, "blobs"),
         ((24, 24, 24), 16, "turbulence"), ((20, 20, 20), 32, "blobs")]


def _field(kind, dims, seed=4):
    return D.make_field(kind, dims, seed)


@pytest.mark.parametrize("dims,rate,kind", CASES)
def test_encoder_matches_oracle(ctx, oracle, dims, rate, kind):
    f = _field(kind, dims)
    w_gpu = to_host(bcmc.zfp_encode(ctx, to_dev(f), rate), np.uint64)
    w_ref = oracle.zfp_encode(f, rate)
    assert np.array_equal(w_gpu, w_ref)


@pytest.mark.parametrize("dims,rate,kind", CASES)
def test_decode_and_ranges_match_oracle(ctx, oracle, dims, rate, kind):
    f = _field(kind, dims)
    w = oracle.zfp_encode(f, rate)
    nb = int(np.prod(oracle.padded_blocks(dims)))
    dec = to_host(bcmc.zfp_decode_volume(ctx, to_dev(w), nb, rate), np.float32)
    assert np.array_equal(bits(dec), bits(oracle.decode_volume(w, nb, 64 * rate)))
    rng = to_host(bcmc.zfp_block_ranges(ctx, to_dev(w), dims, rate), np.float32)
    assert np.array_equal(bits(rng), bits(oracle.block_ranges(w, dims, 64 * rate)))


def test_decode_random_bitstreams(ctx, oracle):
    """Arbitrary bit patterns exercise every decoder path (budget exhaustion
    inside group tests, 64-bit verbatim reads, all planes)."""
    rs = np.random.default_rng(17)
    for rate in (1, 2, 3, 4, 8, 16, 32):
        nb = 300
        words = rs.integers(0, 2**63, size=(nb * 64 * rate) // 64 + 2, dtype=np.uint64)
        words |= rs.integers(0, 2, size=words.shape, dtype=np.uint64) << np.uint64(63)
        dec = to_host(bcmc.zfp_decode_volume(ctx, to_dev(words), nb, rate), np.float32)
        ref = oracle.decode_volume(words, nb, 64 * rate)
        assert np.array_equal(bits(dec), bits(ref)), rate


def test_block_active_matches_oracle(ctx, oracle):
    dims = (40, 36, 44)
    f = _field("blobs", dims)
    w = oracle.zfp_encode(f, 4)
    ranges = oracle.block_ranges(w, dims, 256)
    for iso in (float(f.min()), float(np.median(f)), float(f.max()), 1e30):
        a = to_host(bcmc.block_active(ctx, to_dev(ranges), dims, iso), np.uint32)
        assert np.array_equal(a, oracle.block_active(ranges, dims, iso)), iso
