"""Compressed-volume files and the dataset registry (js/volumes.js:4-152,
js/bcmc.js:27-47).

The reference names each dataset file ``<base>_<X>x<Y>x<Z>_<type>.<...>`` and
reads its dimensions from the name with the regex of js/volumes.js:146-151; the
compressed data is ``<name>.zfp``, a headerless fixed-rate ZFP stream (the
bytes setCompressedVolume takes).  A registry entry carries the compression
rate, the name, the value range the isovalue slider (and the benchmark
drivers) span, the voxel scale and an optional slider step.

The reference's own entries point at scans served from its CDN, which are not
part of this repository; the registry here is filled with the seeded synthetic
volumes of bcmc.datasets, and callers add their own with ``register``.
"""
from __future__ import annotations

import os
import re
from dataclasses import dataclass, field

import numpy as np

# js/volumes.js:146: "(\w+)_(\d+)x(\d+)x(\d+)_(\w+)\.*"
FILE_REGEX = re.compile(r"(\w+)_(\d+)x(\d+)x(\d+)_(\w+)\.*")


@dataclass
class Dataset:
    name: str                 # file base name, "<base>_<X>x<Y>x<Z>_<type>.<...>"
    compressionRate: int
    range: tuple              # (lo, hi) of the isovalues worth asking for
    scale: tuple = (1.0, 1.0, 1.0)
    step: float | None = None
    extra: dict = field(default_factory=dict)

    @property
    def dims(self) -> tuple:
        return volume_dimensions(self.name)

    @property
    def zfp_name(self) -> str:
        return self.name + ".zfp"


def volume_dimensions(filename: str) -> tuple:
    """getVolumeDimensions (js/volumes.js:148-151): (X, Y, Z) from a file name."""
    m = FILE_REGEX.search(os.path.basename(filename))
    if m is None:
        raise ValueError(f"no <name>_<X>x<Y>x<Z>_<type> pattern in {filename!r}")
    return int(m.group(2)), int(m.group(3)), int(m.group(4))


def stream_bytes(dims, rate: int) -> int:
    """Bytes of a fixed-rate stream: 64*rate bits per 4^3 block."""
    nb = int(np.prod([(int(d) + 3) // 4 for d in dims]))
    return nb * 64 * int(rate) // 8


def load_zfp(path: str, rate: int, dims=None) -> tuple:
    """Reads a .zfp stream; returns (uint8 array, dims).  dims default to the
    ones in the file name.  The file must hold at least the stream's bytes."""
    dims = tuple(int(d) for d in (dims or volume_dimensions(path)))
    data = np.fromfile(path, dtype=np.uint8)
    need = stream_bytes(dims, rate)
    if data.size < need:
        raise ValueError(f"{path}: {data.size} bytes, a rate-{rate} stream of {dims} needs {need}")
    return data, dims


def save_zfp(path: str, words) -> None:
    """Writes a stream (the encoder's uint64 words or bytes) as a .zfp file."""
    np.ascontiguousarray(np.asarray(words)).view(np.uint8).tofile(path)


REGISTRY: dict = {}


def register(key: str, ds: Dataset) -> Dataset:
    volume_dimensions(ds.name)  # validates the name
    REGISTRY[key] = ds
    return ds


def open_dataset(key: str, root: str, device=0):
    """Loads <root>/<name>.zfp of a registry entry into a CompressedMarchingCubes
    (js/bcmc.js:27-47); returns (mc, dataset)."""
    import bcmc

    ds = REGISTRY[key]
    data, dims = load_zfp(os.path.join(root, ds.zfp_name), ds.compressionRate)
    mc = bcmc.CompressedMarchingCubes(device)
    mc.setCompressedVolume(data, ds.compressionRate, dims, ds.scale)
    return mc, ds


# The seeded synthetic volumes of bcmc.datasets (64^3 blobs, 256^3 CT-like, 512^3 spectral); the
# files themselves are written by write_synthetic().
register("blobs64", Dataset("blobs64_64x64x64_float32.gen.crate8", 8, (0.0, 1.5)))
register("ct256", Dataset("ct256_256x256x256_float32.gen.crate4", 4, (20.0, 255.0)))
register("turb512", Dataset("turb512_512x512x512_float32.gen.crate2", 2, (-1.0, 1.0)))
_SYNTH = {"blobs64": ("blobs", 1), "ct256": ("ct_like", 2), "turb512": ("turbulence", 3)}


def write_synthetic(key: str, root: str, encode=None) -> str:
    """Generates a registry entry's synthetic field, ZFP-encodes it (`encode`:
    (field[z, y, x], rate) -> uint64 words; the CUDA encoder by default) and
    writes <root>/<name>.zfp.  Returns the path."""
    from . import datasets as D

    ds = REGISTRY[key]
    kind, seed = _SYNTH[key]
    f = D.make_field(kind, ds.dims, seed)
    if encode is None:
        import torch

        import bcmc

        words = bcmc.zfp_encode(bcmc.Context(0), torch.from_numpy(f).cuda(), ds.compressionRate).cpu().numpy()
    else:
        words = encode(f, ds.compressionRate)
    os.makedirs(root, exist_ok=True)
    path = os.path.join(root, ds.zfp_name)
    data = np.ascontiguousarray(words).view(np.uint8)[: stream_bytes(ds.dims, ds.compressionRate)]
    save_zfp(path, data)
    return path
