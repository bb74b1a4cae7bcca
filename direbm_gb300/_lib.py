"""ctypes binding of libdirebm_gb300.so (the C ABI declared in include/direbm_gb300.h).

The library is loaded from ``direbm_gb300/_lib/`` (built in-tree by ``direbm_gb300.build``).
There is no fallback: if the library is missing or a CUDA device is absent, the functions that
need it raise.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libdirebm_gb300.so"

DBM_OK = 0
D2Q7, D2Q9, D3Q13, D3Q19 = 0, 1, 2, 3
FP64, FP32DEV = 0, 1

TRACE = {
    "occ": 1, "thin_cnt": 2, "centroid": 3, "mask": 4, "final_cell": 5, "final_off": 6,
    "sorted": 7, "sw": 8, "cpf": 9, "empty": 10, "fstar": 11, "counts": 12, "state_cell": 13, "state_off": 14,
    "import_order": 15,
}

# Arrays of a recorded step (dbm_tape_export): name -> (id, dtype, shape kind).  Shape kinds: "M",
# "QM" (Q, M), "DM" (D, M), "P", "DP", "P+1", "PQ+1", "nref", "Dnref", "nres", "Dnres", "ngap",
# "Dngap", "I+1" (instances + 1).
TAPE = {
    "in_cell": (1, "u32", "M"), "in_off": (2, "f64", "DM"), "in_f": (3, "f64", "QM"), "fstar": (4, "f64", "QM"),
    "thin_cell": (5, "u32", "QM"), "cp_thin": (6, "u32", "P"), "cp_count": (7, "u32", "P"),
    "cp_cen": (8, "f64", "DP"), "cp_moved": (9, "u32", "P"), "out_cell": (10, "u32", "P"),
    "out_off": (11, "f64", "DP"), "empty": (12, "u32", "P"), "inv_sw": (13, "f64", "QM"),
    "ref_start": (14, "u32", "PQ+1"), "ref_item": (15, "u32", "nref"), "ref_e": (16, "f64", "Dnref"),
    "res_start": (17, "u32", "PQ+1"), "res_item": (18, "u32", "nres"), "res_e": (19, "f64", "Dnres"),
    "gap_start": (20, "u32", "P+1"), "gap_item": (21, "u32", "ngap"), "gap_bits": (22, "u32", "ngap"),
    "gap_e": (23, "f64", "Dngap"), "inst_start": (24, "u32", "I+1"),
}

ST_OUT_OF_BOX, ST_CAPACITY, ST_NONFINITE, ST_BAD_INPUT, ST_INTERNAL = 1, 2, 4, 8, 16


class DbmError(RuntimeError):
    pass


class SimDesc(ctypes.Structure):
    _fields_ = [
        ("lattice", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("dx", ctypes.c_double),
        ("r_res", ctypes.c_double),
        ("cell", ctypes.c_double),
        ("kappa_hard", ctypes.c_int32),
        ("eps", ctypes.c_double),
        ("moment_capacity", ctypes.c_int64),
    ]


class InstanceDesc(ctypes.Structure):
    _fields_ = [
        ("dims", ctypes.c_int32 * 3),
        ("origin", ctypes.c_int32 * 3),
        ("periodic", ctypes.c_int32),
        ("tau", ctypes.c_double),
        ("rho_rest", ctypes.c_double),
    ]


_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f32 = ctypes.c_float
_f64 = ctypes.c_double

_SIGS = {
    "dbm_last_error": (ctypes.c_char_p, []),
    "dbm_version": (ctypes.c_int, []),
    "dbm_launch_count": (ctypes.c_ulonglong, []),
    "dbm_device_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    "dbm_collide_f32": (ctypes.c_int, [_vp, _i64, ctypes.c_int, _f32, _vp]),
    "dbm_collide_f64": (ctypes.c_int, [_vp, _i64, ctypes.c_int, _f64, _vp]),
    "dbm_equilibrium_f32": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _vp, _vp]),
    "dbm_equilibrium_f64": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _vp, _vp]),
    "dbm_radix_sort_tmp_bytes": (_i64, [_i64, ctypes.c_int]),
    "dbm_radix_sort_pairs_u32": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _vp, _vp]),
    "dbm_radix_sort_pairs_u64": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _vp, _vp]),
    "dbm_radix_sort_pairs_u32_noalloc": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _vp]),
    "dbm_disperse_f32": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _f32, _vp, _vp, _vp, _vp]),
    "dbm_create_control_points_f32": (ctypes.c_int, [_vp, _i64, _f32, _vp, ctypes.POINTER(_i64), _vp]),
    "dbm_refine_control_points_f32": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp, _i64, _f32, ctypes.c_int, _vp, _vp]),
    "dbm_resample_f32": (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, _i64, _f32, _vp, ctypes.c_int, _f32, _vp, _vp, _vp]),
    "dbm_segmented_sum_f32": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp]),
    "dbm_bin_fields_tmp_bytes": (_i64, [_i64]),
    "dbm_bin_fields_f64": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _vp, ctypes.c_int, _vp, ctypes.c_int, _vp, _vp,
                                          _vp, _vp, _vp]),
    "dbm_bin_fields3_f64": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _vp, ctypes.c_int, _vp, ctypes.c_int, _vp,
                                           ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "dbm_lbm_step": (ctypes.c_int, [ctypes.c_int, _vp, _vp, _i32, _i32, _i32, _vp, _f64, _i32, _vp, _vp]),
    "dbm_sim_create": (ctypes.c_int, [ctypes.POINTER(SimDesc), ctypes.POINTER(InstanceDesc), _i32, ctypes.POINTER(_vp)]),
    "dbm_sim_destroy": (ctypes.c_int, [_vp]),
    "dbm_sim_set_state": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i64, _vp]),
    "dbm_sim_set_state_sorted": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i64, _vp]),
    "dbm_sim_set_state_f32": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i64, ctypes.c_int32, _vp]),
    "dbm_sim_get_state_f32": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "dbm_sim_step": (ctypes.c_int, [_vp, _i32, _vp]),
    "dbm_sim_step_partial": (ctypes.c_int, [_vp, _i32, _vp]),
    "dbm_sim_profile_step": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float), _vp]),
    "dbm_sim_count": (ctypes.c_int, [_vp, ctypes.POINTER(_i64), _vp]),
    "dbm_sim_get_state": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "dbm_sim_status": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_uint32), _i32, _vp]),
    "dbm_sim_conservation": (ctypes.c_int, [_vp, _vp, _vp]),
    "dbm_sim_use_graphs": (ctypes.c_int, [_vp, _i32]),
    "dbm_sim_set_option": (ctypes.c_int, [_vp, _i32, _i32]),
    "dbm_sim_trace": (ctypes.c_int, [_vp, _i32, _vp, _i64, ctypes.POINTER(_i64), _vp]),
    "dbm_sim_device_bytes": (_i64, [_vp]),
    "dbm_sim_get_tiling": (ctypes.c_int, [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i32)]),
    "dbm_sim_get_brick_width": (ctypes.c_int, [_vp, ctypes.POINTER(_i32)]),
    "dbm_sim_set_tau": (ctypes.c_int, [_vp, _vp, _i32]),
    "dbm_sim_set_obstacle": (ctypes.c_int, [_vp, _i32, _vp, _f64]),
    "dbm_sim_set_inflow": (ctypes.c_int, [_vp, _i32, _vp, _i32]),
    "dbm_sim_snapshot": (ctypes.c_int, [_vp, _vp, _i64, ctypes.POINTER(_i64), _vp]),
    "dbm_sim_restore": (ctypes.c_int, [_vp, _vp, _i64, _vp]),
    "dbm_tape_create": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "dbm_tape_destroy": (ctypes.c_int, [_vp]),
    "dbm_tape_clear": (ctypes.c_int, [_vp]),
    "dbm_tape_step": (ctypes.c_int, [_vp, _vp]),
    "dbm_tape_length": (_i32, [_vp]),
    "dbm_tape_counts": (ctypes.c_int, [_vp, _i32, _vp]),
    "dbm_tape_backward": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp]),
    "dbm_tape_record": (ctypes.c_int, [_vp, _i32, _vp]),
    "dbm_tape_set_estimate": (ctypes.c_int, [_vp, _f64]),
    "dbm_tape_backward_all": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "dbm_tape_export": (ctypes.c_int, [_vp, _i32, _i32, _vp, _i64, ctypes.POINTER(_i64), _vp]),
}

EXPORTED = tuple(_SIGS)

_lib = None


def load(path: str | os.PathLike | None = None):
    """Load the library (once).  Raises DbmError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise DbmError(
            f"{p} is missing: build it with `python -m direbm_gb300.build` "
            "(there is no CPU fallback for the DiReBM kernels)"
        )
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str = "") -> None:
    if rc != DBM_OK:
        msg = _lib.dbm_last_error().decode() if _lib is not None else ""
        raise DbmError(f"{what or 'dbm call'} failed (status {rc}): {msg}")


def launch_count() -> int:
    return int(load().dbm_launch_count())
