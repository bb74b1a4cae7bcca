"""Propagation stages with the reference's signatures (direbm/warp/propagation.py:115-278).

disperse -> create_control_points -> refine_control_points -> resample, on explicit component
arrays, returning device arrays with ``.numpy()`` as the Warp versions did.  The kernels are the
library's stage functions (dbm_disperse_f32, dbm_create_control_points_f32,
dbm_refine_control_points_f32, dbm_resample_f32): a stable device radix sort for cell thinning,
a sorted-cell index for neighbour queries, and a deterministic two-pass resampling gather in
place of the reference's float atomics.
"""

from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ..lattices import D2Q7, get
from ..sim import _require_cuda, _stream
from ._arrays import DeviceArray, to_device


def disperse(pos_m, f_m, dx, device=None, lattice=D2Q7):
    """Moment -> component cloud: (pos_c (Q*M, 2), val_c (Q*M,), dir_c (Q*M,)) device arrays."""
    dev = _require_cuda(device)
    lib = _lib.load()
    lat = get(lattice)
    pm = to_device(pos_m, torch.float32, dev)
    fm = to_device(f_m, torch.float32, dev)
    m = int(pm.shape[0])
    nc = lat.Q * m
    pos_c = torch.empty((nc, 2), dtype=torch.float32, device=dev)
    val_c = torch.empty(nc, dtype=torch.float32, device=dev)
    dir_c = torch.empty(nc, dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.dbm_disperse_f32(pm.data_ptr(), fm.data_ptr(), m, lat.id, ctypes.c_float(float(dx)),
                                        pos_c.data_ptr(), val_c.data_ptr(), dir_c.data_ptr(), _stream()), "disperse")
    return DeviceArray(pos_c), DeviceArray(val_c), DeviceArray(dir_c)


def create_control_points(pos_c, cs, device=None):
    """Cell-thin a component cloud -> (cp_pos device array (P, 2), P)."""
    dev = _require_cuda(device)
    lib = _lib.load()
    pc = to_device(pos_c, torch.float32, dev)
    nc = int(pc.shape[0])
    cp = torch.empty((max(nc, 1), 2), dtype=torch.float32, device=dev)
    p = ctypes.c_int64()
    with torch.cuda.device(dev):
        _lib.check(lib.dbm_create_control_points_f32(pc.data_ptr(), nc, ctypes.c_float(float(cs)), cp.data_ptr(),
                                                     ctypes.byref(p), _stream()), "create_control_points")
    P = int(p.value)
    return DeviceArray(cp[:P].clone()), P


def refine_control_points(cp_pos, pos_c, val_c, dir_c, dx, kappa_hard, device=None):
    """kappa -> hard_outer (kappa <= kappa_hard) keeps its position, others move to the exp(f)-weighted
    centroid of the components within dx.  Returns the new positions (device array (P, 2))."""
    dev = _require_cuda(device)
    lib = _lib.load()
    cp = to_device(cp_pos, torch.float32, dev)
    pc = to_device(pos_c, torch.float32, dev)
    vc = to_device(val_c, torch.float32, dev)
    dc = to_device(dir_c, torch.int32, dev)
    p, nc = int(cp.shape[0]), int(pc.shape[0])
    out = torch.empty((p, 2), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.dbm_refine_control_points_f32(cp.data_ptr(), p, pc.data_ptr(), vc.data_ptr(), dc.data_ptr(),
                                                     nc, ctypes.c_float(float(dx)), int(kappa_hard), out.data_ptr(),
                                                     _stream()), "refine_control_points")
    return DeviceArray(out)


def resample(pos_c, val_c, dir_c, cp_pos, dx, f_rest, device=None, lattice=D2Q7, eps=1e-6):
    """Scatter components into control points, fill empty directions from f_rest, emit one moment
    per control point.  Returns (out_pos (P, 2), out_f (P, Q)) device arrays."""
    dev = _require_cuda(device)
    lib = _lib.load()
    lat = get(lattice)
    pc = to_device(pos_c, torch.float32, dev)
    vc = to_device(val_c, torch.float32, dev)
    dc = to_device(dir_c, torch.int32, dev)
    cp = to_device(cp_pos, torch.float32, dev)
    fr = to_device(f_rest, torch.float32, dev)
    nc, p = int(pc.shape[0]), int(cp.shape[0])
    out_pos = torch.empty((p, 2), dtype=torch.float32, device=dev)
    out_f = torch.empty((p, lat.Q), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.dbm_resample_f32(pc.data_ptr(), vc.data_ptr(), dc.data_ptr(), nc, cp.data_ptr(), p,
                                        ctypes.c_float(float(dx)), fr.data_ptr(), lat.id, ctypes.c_float(float(eps)),
                                        out_pos.data_ptr(), out_f.data_ptr(), _stream()), "resample")
    return DeviceArray(out_pos), DeviceArray(out_f)


__all__ = ["disperse", "create_control_points", "refine_control_points", "resample"]
