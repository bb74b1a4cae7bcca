"""pytest plugin (test infrastructure): run the reference's own GPU tests against this library.

Loaded with ``-p tests._reference_swap`` in a separate pytest process.  It puts the reference's
CPU package (installed under baseline/_ref by oracle/install_reference.py) on the path, aliases
``direbm.warp`` and its submodules to ``direbm_gb300.warp`` -- the module swap a maintainer would
make -- and registers a minimal ``warp`` module for the two direct uses of ``wp.array`` /
``wp.vec2`` / ``wp.float32`` / ``wp.int32`` in the reference's tests/test_warp_propagation.py:18-24
(an array constructor returning this library's device array).  The test files themselves run
unchanged.
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
REF = ROOT / "baseline" / "_ref"
sys.path.insert(0, str(REF))
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import torch  # noqa: E402

import direbm_gb300.warp as _gw  # noqa: E402
from direbm_gb300.warp import lbm, physics, propagation, simulator  # noqa: E402,F401
from direbm_gb300.warp._arrays import DeviceArray, to_device  # noqa: E402

import direbm  # noqa: E402  (the reference's CPU package; its __init__ does not import warp)

for _sub in ("", ".lbm", ".physics", ".propagation", ".simulator"):
    sys.modules["direbm.warp" + _sub] = sys.modules["direbm_gb300.warp" + _sub]
direbm.warp = _gw

_wp = types.ModuleType("warp")
_wp.vec2, _wp.float32, _wp.int32 = "vec2", "float32", "int32"
_DT = {"vec2": torch.float32, "float32": torch.float32, "int32": torch.int32}


def _array(data, dtype=None, device=None):
    return DeviceArray(to_device(data, _DT.get(dtype, torch.float32), device or physics.default_device()))


_wp.array = _array
sys.modules["warp"] = _wp
