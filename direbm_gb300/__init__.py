"""direbm_gb300 -- the DiReBM step (berfandil/DiReBM) as hand-written sm_103a CUDA for GB300.

Layers:
  include/direbm_gb300.h       C ABI of libdirebm_gb300.so (csrc/*.cu)
  direbm_gb300._lib            ctypes binding
  direbm_gb300.sim             batched fused step (Simulation, Instance)
  direbm_gb300.lbm             batched hexagonal D2Q7 lattice Boltzmann
  direbm_gb300.warp            drop-in for the reference's direbm.warp API
"""

from . import lattices
from .lattices import D2Q7, D2Q9, D3Q13, D3Q19, equilibrium

__version__ = "0.1.0"

__all__ = ["lattices", "D2Q7", "D2Q9", "D3Q13", "D3Q19", "equilibrium", "Simulation", "Instance", "HexLBM"]


def __getattr__(name):
    # torch-dependent modules load on first use so `import direbm_gb300` stays light
    if name in ("Simulation", "Instance"):
        from . import sim

        return getattr(sim, name)
    if name == "HexLBM":
        from .lbm import HexLBM

        return HexLBM
    raise AttributeError(name)
