"""The C-ABI library builds, loads and exports every symbol include/direbm_gb300.h declares.

No compute call is made here (no GPU in the CPU suite)."""

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    txt = (ROOT / "include" / "direbm_gb300.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dbm_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from direbm_gb300.build import build

    path = build()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = _declared()
    assert "dbm_sim_step" in names and "dbm_lbm_step" in names and "dbm_radix_sort_pairs_u32" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from direbm_gb300 import _lib

    assert set(_declared()) == set(_lib.EXPORTED)


def test_error_path_without_gpu(lib):
    """Argument validation runs before any CUDA call and reports through dbm_last_error."""
    lib.dbm_last_error.restype = ctypes.c_char_p
    lib.dbm_collide_f32.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_float, ctypes.c_void_p]
    rc = lib.dbm_collide_f32(None, ctypes.c_int64(-1), 0, ctypes.c_float(0.6), None)
    assert rc == 1
    assert b"bad arguments" in lib.dbm_last_error()
    lib.dbm_sim_create.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
    assert lib.dbm_sim_create(None, None, 0, None) == 1
    lib.dbm_radix_sort_tmp_bytes.restype = ctypes.c_int64
    lib.dbm_radix_sort_tmp_bytes.argtypes = [ctypes.c_int64, ctypes.c_int]
    assert lib.dbm_radix_sort_tmp_bytes(1000, 4) > 8000
    assert lib.dbm_radix_sort_tmp_bytes(1000, 3) == -1


def test_product_has_no_oracle_imports():
    """The product package never imports the CPU oracle (it is test infrastructure)."""
    for p in (ROOT / "direbm_gb300").rglob("*.py"):
        src = p.read_text()
        assert "import oracle" not in src and "from oracle" not in src, p
