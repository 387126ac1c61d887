"""Helpers for the GPU parity tests (device buffers through torch)."""
from __future__ import annotations

import numpy as np


def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def to_dev(a: np.ndarray):
    torch = torch_cuda()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def to_host(t) -> np.ndarray:
    torch = torch_cuda()
    torch.cuda.synchronize()
    return t.cpu().numpy()
