"""The seeded synthetic volumes that stand in for the reference's datasets
(none ship with it: js/volumes.js streams them from a CDN) have the shapes and
value distributions of the benchmark workloads: Gaussian blobs, the CT-like
field with 35 % constant-0 background blocks and interior values 20-255, the
k^-5/3 spectral field in [-1, 1], the uint16-range field with 60 % background
blocks (its GPU generator agreeing with the numpy one), and the +-0.02 random
walk of isovalues."""
import numpy as np
import pytest

from bcmc import datasets as D


def test_blobs_are_a_sum_of_gaussians_in_the_box():
    f = D.blobs((64, 64, 64), 1)
    assert f.shape == (64, 64, 64) and f.dtype == np.float32
    assert f.min() >= 0.0 and 0.5 <= f.max() <= 8.0  # 8 blobs of amplitude 0.5-1
    assert np.array_equal(f, D.blobs((64, 64, 64), 1))  # seeded
    # a single isovalue 0.5 cuts a surface: some voxels above, most below
    assert 0.0 < (f > 0.5).mean() < 0.5


def test_ct_like_background_blocks_and_interior_range():
    f = D.ct_like((256, 256, 256), 2)
    assert f.shape == (256, 256, 256) and f.dtype == np.float32
    bmax = D._block_max(f)
    assert abs((bmax == 0.0).mean() - 0.35) < 0.005
    inside = f[f > 0.0]
    assert inside.min() >= 20.0 and inside.max() <= 255.0
    # the 16 isovalues linspace(30, 220) all lie inside the interior range
    isos = D.config_isovalues("ct256")
    assert len(isos) == 16 and isos[0] == 30.0 and isos[-1] == 220.0
    for iso in isos[[0, 8, 15]]:
        assert 0.0 < (inside >= iso).mean() < 1.0


def test_turbulence_is_normalised_with_a_k_minus_five_thirds_spectrum():
    n = 128
    f = D.turbulence((n, n, n), 3)
    assert f.min() == -1.0 and f.max() == 1.0
    spec = np.abs(np.fft.rfftn(f.astype(np.float64))) ** 2
    kz = np.fft.fftfreq(n)[:, None, None] * n
    ky = np.fft.fftfreq(n)[None, :, None] * n
    kx = np.fft.rfftfreq(n)[None, None, :] * n
    k = np.sqrt(kz * kz + ky * ky + kx * kx)
    shell = np.rint(k).astype(np.int64)
    # the energy of each spherical shell (the half-space counts each mode once)
    e = np.bincount(shell.ravel(), weights=spec.ravel())
    ks = np.arange(4, 40)
    slope = np.polyfit(np.log(ks), np.log(e[ks]), 1)[0]
    assert abs(slope - (-5.0 / 3.0)) < 0.1, slope


def test_uint16_field_background_and_integer_range():
    f = D.ct_uint16((128, 128, 136), 5)
    assert abs((D._block_max(f) == 0.0).mean() - 0.60) < 0.005
    assert f.min() == 0.0 and f.max() == 4095.0
    assert np.array_equal(f, np.round(f))


def test_uint16_gpu_generator_matches_the_numpy_one():
    torch = pytest.importorskip("torch")
    ref = D.ct_uint16((128, 128, 136), 5)
    got = D.ct_uint16_torch((128, 128, 136), 5, device="cpu").numpy()
    # float32 against float64 interpolation: a few voxels round the other way
    assert np.abs(got - ref).max() <= 1.0
    assert (got != ref).mean() < 1e-3
    assert (D._block_max(got) == 0.0).mean() == pytest.approx((D._block_max(ref) == 0.0).mean(), abs=1e-3)


def test_random_walk_of_isovalues():
    w = D.config_isovalues("turb512")
    assert len(w) == 64 and w[0] == 0.0
    assert np.allclose(np.abs(np.diff(w.astype(np.float64))), 0.02, atol=1e-6)
    assert w.min() >= -1.0 and w.max() <= 1.0
    assert np.array_equal(w, D.random_walk(64, 3))
