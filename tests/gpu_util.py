"""Helpers for the GPU tests: device round trips and the error metric."""

import numpy as np


def to_dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def from_dev(t):
    import torch

    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def rel(a, b):
    """max |a - b| / max |b| (the error measure used throughout)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
