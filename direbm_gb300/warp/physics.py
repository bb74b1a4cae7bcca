"""BGK physics entry points with the reference's signatures (direbm/warp/physics.py:21-97).

``collide(f_np, tau)`` and ``equilibrium(rho_np, u_np)`` take numpy arrays and return FP32 numpy
arrays of shape (N, 7) exactly like the Warp versions; the work runs in the library's CUDA
kernels (dbm_collide_f32 / dbm_equilibrium_f32).
"""

from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ..lattices import D2Q7, get
from ..sim import _require_cuda, _stream
from ._arrays import to_device


def default_device() -> str:
    """The device the kernels run on (direbm/warp/physics.py:21-22).  The library has no CPU
    path, so every entry point raises when this reports "cpu"."""
    return "cuda:0" if torch.cuda.is_available() else "cpu"


def collide(f_np, tau, device=None, lattice=D2Q7):
    """BGK collision of f (N, Q) on the GPU; returns a new FP32 (N, Q) numpy array."""
    dev = _require_cuda(device)
    lib = _lib.load()
    lat = get(lattice)
    f = to_device(f_np, torch.float32, dev).clone()
    n = int(f.shape[0])
    with torch.cuda.device(dev):
        _lib.check(lib.dbm_collide_f32(f.data_ptr(), n, lat.id, ctypes.c_float(float(tau)), _stream()), "collide")
        torch.cuda.current_stream().synchronize()
    return f.cpu().numpy()


def equilibrium(rho_np, u_np, device=None, lattice=D2Q7):
    """f_eq for (rho (N,), u (N, D)) on the GPU; returns FP32 (N, Q) numpy."""
    dev = _require_cuda(device)
    lib = _lib.load()
    lat = get(lattice)
    rho = to_device(rho_np, torch.float32, dev)
    u = to_device(u_np, torch.float32, dev)
    n = int(rho.shape[0])
    out = torch.empty((n, lat.Q), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.dbm_equilibrium_f32(rho.data_ptr(), u.data_ptr(), n, lat.id, out.data_ptr(), _stream()),
                   "equilibrium")
        torch.cuda.current_stream().synchronize()
    return out.cpu().numpy()


__all__ = ["collide", "equilibrium", "default_device"]

