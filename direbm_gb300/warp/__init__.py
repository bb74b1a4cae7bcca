"""Drop-in replacement for the reference's ``direbm.warp`` package (direbm/warp/__init__.py:9-24).

Same names, arguments and return conventions; the kernels are the library's hand-written
sm_103a CUDA instead of Warp JIT kernels.  There is no CPU fallback.
"""

from .lbm import GpuHexLBM
from .physics import collide, default_device, equilibrium
from .propagation import create_control_points, disperse, refine_control_points, resample
from .simulator import GpuSimulator

__all__ = [
    "collide",
    "equilibrium",
    "default_device",
    "disperse",
    "create_control_points",
    "refine_control_points",
    "resample",
    "GpuSimulator",
    "GpuHexLBM",
]
