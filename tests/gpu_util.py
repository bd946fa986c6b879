"""Helpers for the GPU tests: numpy <-> CUDA tensors with exact bits."""
import numpy as np


def to_dev(a: np.ndarray):
    import torch

    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    elif a.dtype == np.uint64:
        a = a.view(np.int64)
    return torch.from_numpy(a.copy()).cuda()


def to_host(t, dtype) -> np.ndarray:
    import torch

    torch.cuda.synchronize()
    return t.detach().cpu().numpy().view(dtype)


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
