"""Macroscopic fields from scattered moments, on the device (direbm/fields.py:17-41), in 2D and 3D.

``bin_fields(x, f, xmin, xmax, h)`` has the reference's signature and return value
(rho (ny, nx), u (ny, nx, 2), extent): per-bin mass / h^2 and momentum / mass, zero where a bin is
empty.  Binning, sorting and the per-bin sums run in the library (dbm_bin_fields_f64); ``x`` and
``f`` may be numpy arrays or CUDA tensors (for example a Simulation's state, without a host copy).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .lattices import D2Q7, D3Q19, get
from .sim import _require_cuda, _stream


def bin_fields_device(x, f, edges_x, edges_y, lattice=D2Q7, device=None):
    """Per-bin (mass, momx, momy) as CUDA tensors of shape (ny, nx)."""
    dev = _require_cuda(device)
    lib = _lib.load()
    lat = get(lattice)
    x = torch.as_tensor(x, dtype=torch.float64, device=dev).contiguous()
    f = torch.as_tensor(f, dtype=torch.float64, device=dev).contiguous()
    ex = torch.as_tensor(np.asarray(edges_x, np.float64), device=dev)
    ey = torch.as_tensor(np.asarray(edges_y, np.float64), device=dev)
    n = int(x.shape[0])
    nx, ny = len(edges_x) - 1, len(edges_y) - 1
    mass = torch.empty((ny, nx), dtype=torch.float64, device=dev)
    momx = torch.empty_like(mass)
    momy = torch.empty_like(mass)
    tmp = torch.empty(max(int(lib.dbm_bin_fields_tmp_bytes(n)), 1), dtype=torch.uint8, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.dbm_bin_fields_f64(x.data_ptr(), f.data_ptr(), n, lat.id, ex.data_ptr(), len(edges_x),
                                          ey.data_ptr(), len(edges_y), mass.data_ptr(), momx.data_ptr(),
                                          momy.data_ptr(), tmp.data_ptr(), _stream()), "bin_fields")
    return mass, momx, momy


def bin_fields3_device(x, f, edges_x, edges_y, edges_z, lattice=D3Q19, device=None):
    """Per-bin (mass, momx, momy, momz) as CUDA tensors of shape (nz, ny, nx)."""
    dev = _require_cuda(device)
    lib = _lib.load()
    lat = get(lattice)
    if lat.D != 3:
        raise ValueError("bin_fields3_device: a 3D lattice is required")
    x = torch.as_tensor(x, dtype=torch.float64, device=dev).contiguous()
    f = torch.as_tensor(f, dtype=torch.float64, device=dev).contiguous()
    if x.ndim != 2 or x.shape[1] != 3 or f.shape != (x.shape[0], lat.Q):
        raise ValueError("bin_fields3_device: expected x (n, 3) and f (n, Q)")
    ed = [torch.as_tensor(np.asarray(e, np.float64), device=dev) for e in (edges_x, edges_y, edges_z)]
    n = int(x.shape[0])
    shape = (len(edges_z) - 1, len(edges_y) - 1, len(edges_x) - 1)
    out = [torch.empty(shape, dtype=torch.float64, device=dev) for _ in range(4)]
    tmp = torch.empty(max(int(lib.dbm_bin_fields_tmp_bytes(n)), 1), dtype=torch.uint8, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.dbm_bin_fields3_f64(x.data_ptr(), f.data_ptr(), n, lat.id, ed[0].data_ptr(), len(edges_x),
                                           ed[1].data_ptr(), len(edges_y), ed[2].data_ptr(), len(edges_z),
                                           out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), out[3].data_ptr(),
                                           tmp.data_ptr(), _stream()), "bin_fields3")
    return tuple(out)


def bin_fields3(x, f, xmin, xmax, h, lattice=D3Q19, device=None):
    """3D binning on a cubic grid [xmin, xmax]^3 of cell h: (rho (nz, ny, nx) = mass / h^3,
    u (nz, ny, nx, 3) = momentum / mass, zero where a bin is empty, extent).  The reference's
    bin_fields (direbm/fields.py:17-41) with a third axis and volume in place of area."""
    edges = np.arange(xmin, xmax + h, h)
    mass, mx, my, mz = (t.cpu().numpy() for t in bin_fields3_device(x, f, edges, edges, edges, lattice, device))
    rho = mass / (h * h * h)
    safe = np.where(mass == 0.0, 1.0, mass)
    u = np.stack([mx / safe, my / safe, mz / safe], axis=-1)
    u[mass == 0.0] = 0.0
    return rho, u, (xmin, xmax, xmin, xmax, xmin, xmax)


def bin_fields(x, f, xmin, xmax, h, lattice=D2Q7, device=None):
    """Bin moments onto a regular grid; return (rho, u, extent) as numpy (direbm/fields.py:17-41)."""
    edges = np.arange(xmin, xmax + h, h)
    mass, momx, momy = bin_fields_device(x, f, edges, edges, lattice, device)
    mg = mass.cpu().numpy()
    rho = mg / (h * h)
    safe = np.where(mg == 0.0, 1.0, mg)
    u = np.stack([momx.cpu().numpy() / safe, momy.cpu().numpy() / safe], axis=-1)
    u[mg == 0.0] = 0.0
    return rho, u, (xmin, xmax, xmin, xmax)


__all__ = ["bin_fields", "bin_fields_device", "bin_fields3", "bin_fields3_device"]
