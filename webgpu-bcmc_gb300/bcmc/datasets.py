"""Seeded synthetic volumes standing in for the reference's datasets.

The reference streams ZFP-compressed scans from a CDN (js/volumes.js:4-145);
none ship with it, so every workload here is generated from a seed with the
shapes, rates and value distributions of the benchmark configurations:

* ``blobs``       - sum of isotropic Gaussian blobs (64^3, rate 8, iso 0.5)
* ``ct_like``     - CT-like uint8-range field: smoothed value noise with ~35 % of
                    the 4^3 blocks constant-0 background, interior 20-255 plus
                    N(0, 3) noise (256^3, rate 4, 16 isovalues in [30, 220])
* ``turbulence``  - spectral synthesis with an isotropic k^-5/3 energy spectrum
                    and random phases, normalised to [-1, 1] (512^3, rate 2)
* ``ct_uint16``   - uint16-range (0-4095) smoothed value noise with ~60 %
                    background blocks (the served 1024x1024x1080 volume)

Arrays are float32 indexed ``[z, y, x]`` (x fastest), i.e. ``dims = (X, Y, Z)``.
"""
from __future__ import annotations

import numpy as np


def _interp_matrix(n_out: int, n_lattice: int, spacing: float) -> np.ndarray:
    """Cubic-smoothstep interpolation weights from lattice points to samples."""
    x = np.arange(n_out, dtype=np.float64) / spacing
    i0 = np.floor(x).astype(np.int64)
    t = x - i0
    t = t * t * (3.0 - 2.0 * t)
    w = np.zeros((n_out, n_lattice), dtype=np.float64)
    w[np.arange(n_out), np.clip(i0, 0, n_lattice - 1)] += 1.0 - t
    w[np.arange(n_out), np.clip(i0 + 1, 0, n_lattice - 1)] += t
    return w


def value_noise(dims, seed: int, spacing: float = 24.0, octaves=((1.0, 1.0), (0.25, 0.35))) -> np.ndarray:
    """Smooth value noise in [0, 1]: random lattice values, smoothstep-interpolated,
    summed over octaves (relative spacing, weight)."""
    X, Y, Z = (int(d) for d in dims)
    rng = np.random.default_rng(seed)
    out = np.zeros((Z, Y, X), dtype=np.float32)
    total_w = 0.0
    for rel, weight in octaves:
        sp = spacing * rel
        g = [int(np.ceil(n / sp)) + 2 for n in (Z, Y, X)]
        lattice = rng.random(g, dtype=np.float64)
        wz, wy, wx = (_interp_matrix(n, gn, sp) for n, gn in zip((Z, Y, X), g))
        f = np.einsum("zk,kji->zji", wz, lattice)
        f = np.einsum("yj,zji->zyi", wy, f)
        f = np.einsum("xi,zyi->zyx", wx, f)
        out += (weight * f).astype(np.float32)
        total_w += weight
    out /= total_w
    lo, hi = float(out.min()), float(out.max())
    return ((out - lo) / max(hi - lo, 1e-12)).astype(np.float32)


def _block_max(field: np.ndarray) -> np.ndarray:
    Z, Y, X = field.shape
    pz, py, px = (-Z) % 4, (-Y) % 4, (-X) % 4
    f = np.pad(field, ((0, pz), (0, py), (0, px)), mode="edge")
    return f.reshape(f.shape[0] // 4, 4, f.shape[1] // 4, 4, f.shape[2] // 4, 4).max(axis=(1, 3, 5))


def _background_threshold(noise: np.ndarray, fraction: float) -> float:
    """Threshold t such that ``fraction`` of the 4^3 blocks lie entirely below t."""
    return float(np.quantile(_block_max(noise), fraction))


def blobs(dims=(64, 64, 64), seed: int = 1, n_blobs: int = 8) -> np.ndarray:
    """Sum of isotropic Gaussian blobs: centres uniform in the box, sigma
    uniform in [4, 12] voxels, amplitude uniform in [0.5, 1]."""
    X, Y, Z = (int(d) for d in dims)
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, 1.0, size=(n_blobs, 3)) * np.array([X, Y, Z], dtype=np.float64)
    sigma = rng.uniform(4.0, 12.0, size=n_blobs)
    amp = rng.uniform(0.5, 1.0, size=n_blobs)
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    f = np.zeros((Z, Y, X), dtype=np.float64)
    for (cx, cy, cz), s, a in zip(centres, sigma, amp):
        r2 = (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2
        f += a * np.exp(-r2 / (2.0 * s * s))
    return f.astype(np.float32)


def ct_like(dims=(256, 256, 256), seed: int = 2, background: float = 0.35,
            lo: float = 20.0, hi: float = 255.0, noise_sigma: float = 3.0) -> np.ndarray:
    """CT-like uint8-range field stored as float32."""
    n = value_noise(dims, seed)
    t = _background_threshold(n, background)
    rng = np.random.default_rng(seed + 1000)
    inside = n >= t
    v = lo + (n - t) / max(1.0 - t, 1e-6) * (hi - lo)
    v = v + rng.normal(0.0, noise_sigma, size=n.shape)
    v = np.clip(v, lo, hi)
    return np.where(inside, v, 0.0).astype(np.float32)


def ct_uint16(dims, seed: int = 5, background: float = 0.60, hi: float = 4095.0) -> np.ndarray:
    """uint16-range (0-4095) smoothed value noise with ~60 % background blocks."""
    n = value_noise(dims, seed, spacing=48.0)
    t = _background_threshold(n, background)
    v = np.clip((n - t) / max(1.0 - t, 1e-6), 0.0, 1.0) * hi
    return np.where(n >= t, np.round(v), 0.0).astype(np.float32)


def turbulence(dims=(512, 512, 512), seed: int = 3) -> np.ndarray:
    """Isotropic k^-5/3 spectrum (3-D spectral density k^-11/3), random phases,
    normalised to [-1, 1]."""
    X, Y, Z = (int(d) for d in dims)
    rng = np.random.default_rng(seed)
    kz = np.fft.fftfreq(Z)[:, None, None]
    ky = np.fft.fftfreq(Y)[None, :, None]
    kx = np.fft.rfftfreq(X)[None, None, :]
    k = np.sqrt(kz * kz + ky * ky + kx * kx).astype(np.float32)
    k[0, 0, 0] = np.inf
    amp = k ** (-11.0 / 6.0)
    phase = rng.uniform(0.0, 2.0 * np.pi, size=amp.shape).astype(np.float32)
    spec = (amp * np.exp(1j * phase)).astype(np.complex64)
    try:
        import scipy.fft as sfft

        f = sfft.irfftn(spec, s=(Z, Y, X), workers=-1)
    except ImportError:  # pragma: no cover
        f = np.fft.irfftn(spec, s=(Z, Y, X))
    f = f.astype(np.float32)
    lo, hi = float(f.min()), float(f.max())
    return (2.0 * (f - lo) / max(hi - lo, 1e-12) - 1.0).astype(np.float32)


def ct_uint16_torch(dims, seed: int = 5, background: float = 0.60, hi: float = 4095.0, device="cuda"):
    """ct_uint16 generated on the GPU (torch), for volumes too large for the
    numpy path (the served 1024x1024x1080 volume): same construction --
    smoothstep value noise (spacing 48, two octaves), the threshold below which
    `background` of the 4^3 blocks lie, values 0-4095 -- as a float32 CUDA
    tensor [z, y, x]."""
    import torch

    X, Y, Z = (int(d) for d in dims)
    rng = np.random.default_rng(seed)
    out = torch.zeros((Z, Y, X), dtype=torch.float32, device=device)
    total_w = 0.0
    for rel, weight in ((1.0, 1.0), (0.25, 0.35)):
        sp = 48.0 * rel
        g = [int(np.ceil(n / sp)) + 2 for n in (Z, Y, X)]
        lattice = torch.from_numpy(rng.random(g, dtype=np.float64).astype(np.float32)).to(device)
        wz, wy, wx = (torch.from_numpy(_interp_matrix(n, gn, sp).astype(np.float32)).to(device)
                      for n, gn in zip((Z, Y, X), g))
        f = torch.einsum("yj,kji->kyi", wy, lattice)          # [gz, Y, gx]
        f = torch.einsum("xi,kyi->kyx", wx, f)               # [gz, Y, X]
        for z0 in range(0, Z, 64):                           # [Z, Y, X] in slabs
            out[z0: z0 + 64] += weight * torch.einsum("zk,kyx->zyx", wz[z0: z0 + 64], f)
        total_w += weight
    out /= total_w
    lo, hi_v = float(out.min()), float(out.max())
    out -= lo
    out /= max(hi_v - lo, 1e-12)
    pz, py, px = (-Z) % 4, (-Y) % 4, (-X) % 4
    bm = torch.nn.functional.pad(out[None, None], (0, px, 0, py, 0, pz), mode="replicate")[0, 0]
    bm = bm.reshape(bm.shape[0] // 4, 4, bm.shape[1] // 4, 4, bm.shape[2] // 4, 4).amax(dim=(1, 3, 5)).reshape(-1)
    k = max(1, int(round(background * bm.numel())))
    t = float(torch.kthvalue(bm.cpu(), k).values)
    del bm
    v = torch.clamp((out - t) / max(1.0 - t, 1e-6), 0.0, 1.0) * hi
    v = torch.where(out >= t, torch.round(v), torch.zeros_like(v))
    del out
    return v


def random_walk(n: int, seed: int, step: float = 0.02, start: float = 0.0,
                lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    """Isovalues following a seeded +-step random walk from ``start``."""
    rng = np.random.default_rng(seed)
    vals = [start]
    for _ in range(n - 1):
        s = step if rng.random() < 0.5 else -step
        nxt = vals[-1] + s
        if nxt < lo or nxt > hi:
            nxt = vals[-1] - s
        vals.append(nxt)
    return np.asarray(vals, dtype=np.float32)


# Benchmark configurations (shapes, rates, query sequences, cache sizing).
CONFIGS = {
    "blobs64": dict(dims=(64, 64, 64), rate=8, field="blobs", seed=1,
                    isovalues=[0.5], cache_fraction=1.0),
    "ct256": dict(dims=(256, 256, 256), rate=4, field="ct_like", seed=2,
                  isovalues=list(np.linspace(30.0, 220.0, 16)), cache_fraction=0.5),
    "turb512": dict(dims=(512, 512, 512), rate=2, field="turbulence", seed=3,
                    isovalues=None, cache_fraction=0.25),
}


def make_field(kind: str, dims, seed: int) -> np.ndarray:
    if kind == "blobs":
        return blobs(dims, seed)
    if kind == "ct_like":
        return ct_like(dims, seed)
    if kind == "turbulence":
        return turbulence(dims, seed)
    if kind == "ct_uint16":
        return ct_uint16(dims, seed)
    raise ValueError(kind)


def config_isovalues(name: str) -> np.ndarray:
    c = CONFIGS[name]
    if c["isovalues"] is not None:
        return np.asarray(c["isovalues"], dtype=np.float32)
    return random_walk(64, c["seed"])
