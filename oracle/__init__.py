"""CPU oracle for the DiReBM hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in numpy (FP64, plus exact-FP32 emulation where integer decisions depend
on FP32 rounding), the algorithms of berfandil/DiReBM that the CUDA library replaces:

- ``physics``   -- BGK recover / equilibrium / collide      (direbm/physics.py:16-55)
- ``lbm``       -- hexagonal D2Q7 lattice Boltzmann         (direbm/lbm.py:26-66)
- ``lattices``  -- D2Q7, D3Q13 (reference) + D2Q9, D3Q19    (direbm/lattices.py, constants.py)
- ``stages``    -- the GPU path's stage functions on explicit component arrays
                   (direbm/warp/propagation.py:21-246, direbm/warp/physics.py:31-62)
- ``grid_step`` -- the same step on the dense cell grid used by the fused CUDA pipeline
                   (direbm/warp/simulator.py:50-73 with periodic boxes and batching)
- ``fields``    -- macroscopic binning                      (direbm/fields.py:17-41)

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it,
and there only as the checker.  The product path (``direbm_gb300``) never imports it: if the CUDA
library is missing, the product raises instead of falling back to anything here.

Pinning: ``tests/test_oracle_golden.py`` checks every function here against golden vectors
generated from the reference's own CPU code (``tests/golden/make_golden.py``) and against the
reference tests' own numpy restatement of cell thinning (tests/test_warp_propagation.py:27-36).
"""
