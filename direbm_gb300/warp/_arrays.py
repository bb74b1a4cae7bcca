"""A small device-array wrapper with the parts of ``wp.array`` the reference API exposes.

The reference's GPU functions return Warp arrays, and its callers use ``.numpy()``, ``.shape`` and
``len()`` on them (tests/test_warp_propagation.py, experiments/exp_gpu_bench.py:70).  Here the
storage is a CUDA torch tensor.
"""

from __future__ import annotations

import numpy as np
import torch


class DeviceArray:
    __slots__ = ("tensor",)

    def __init__(self, tensor: torch.Tensor):
        self.tensor = tensor

    def numpy(self) -> np.ndarray:
        return self.tensor.detach().cpu().numpy()

    @property
    def shape(self):
        return tuple(self.tensor.shape)

    @property
    def dtype(self):
        return self.tensor.dtype

    def __len__(self):
        return int(self.tensor.shape[0])

    def __repr__(self):
        return f"DeviceArray(shape={self.shape}, dtype={self.tensor.dtype}, device={self.tensor.device})"


def to_device(x, dtype: torch.dtype, device) -> torch.Tensor:
    """numpy / torch / DeviceArray -> contiguous CUDA tensor of ``dtype``."""
    if isinstance(x, DeviceArray):
        x = x.tensor
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=device).contiguous()
