"""Generate golden vectors from the reference's own CPU code (berfandil/DiReBM).

Run in a container where the reference checkout is available:

    python tests/golden/make_golden.py /path/to/DiReBM

It imports the reference's numpy package (``direbm``, ``direbm.lbm``, ``direbm.fields``,
``direbm.reference``) -- which needs no Warp -- then the reference's GPU package
(``direbm.warp``) with ``warp_emulator.py`` standing in for Warp (``warp_reference.npz``), and, for the two numpy helpers that live in the
reference's Warp test module (``_cell_thin_ref`` and ``_ring`` of tests/test_warp_propagation.py),
extracts just those function definitions with ``ast`` (the module itself imports Warp).  The
outputs are small ``.npz`` files next to this script; the tests load only those files, so the
reference checkout is not needed where the tests run.
"""

from __future__ import annotations

import ast
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _load_test_helpers(ref_root: Path) -> dict:
    src = (ref_root / "tests" / "test_warp_propagation.py").read_text()
    tree = ast.parse(src)
    keep = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in ("_cell_thin_ref", "_ring")]
    mod = ast.Module(body=keep, type_ignores=[])
    ns = {"np": np}
    exec(compile(mod, "reference_test_helpers", "exec"), ns)
    return ns


def main(ref_root: str) -> None:
    ref_root = Path(ref_root).resolve()
    sys.path.insert(0, str(ref_root))
    import direbm
    from direbm import bin_fields, collide, equilibrium
    from direbm.lattices import D2Q7, D3Q13, Lattice
    from direbm.lbm import HexLBM
    from direbm.reference import Moment, Simulator

    helpers = _load_test_helpers(ref_root)

    # -- physics (tests/test_warp_physics.py:13-37 seeds; plus D3Q13 and a harness-built D2Q9) ----
    d2q9 = Lattice(
        C=np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]], float),
        W=np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4),
        cs2=1.0 / 3.0,
        name="D2Q9",
    )
    out = {}
    for name, lat in (("D2Q7", D2Q7), ("D2Q9", d2q9), ("D3Q13", D3Q13)):
        rng = np.random.default_rng(0)
        rho = rng.uniform(0.5, 2.0, size=128)
        u = rng.uniform(-0.1, 0.1, size=(128, lat.D))
        out[f"{name}_eq_rho"] = rho
        out[f"{name}_eq_u"] = u
        out[f"{name}_eq"] = equilibrium(rho, u, lat)
        rng = np.random.default_rng(1)
        f = rng.uniform(0.01, 1.0, size=(256, lat.Q))
        out[f"{name}_col_f"] = f
        out[f"{name}_col"] = collide(f, 0.6, lat)
    np.savez_compressed(HERE / "physics.npz", **out)

    # -- hexagonal LBM (tests/test_warp_lbm.py:9-39, tests/test_lbm.py) ------------------------------
    out = {}
    lbm = HexLBM(21, 21, tau=0.6)
    lbm.set_pulse(1.5)
    out["pulse21_f0"] = lbm.f.copy()
    for _ in range(10):
        lbm.step()
    out["pulse21_f10"] = lbm.f.copy()
    lbm = HexLBM(25, 25, tau=0.7)
    lbm.set_pulse(2.0)
    out["pulse25_f0"] = lbm.f.copy()
    for _ in range(15):
        lbm.step()
    out["pulse25_f15"] = lbm.f.copy()
    np.savez_compressed(HERE / "lbm.npz", **out)

    # -- cell thinning KAT: the reference test's own numpy restatement (_cell_thin_ref) on the
    #    FP32 component clouds of its seeds (tests/test_warp_propagation.py:43-76) ---------------
    out = {}
    C32 = direbm.C.astype(np.float32)
    for seed, (n, lo, hi) in {0: (20, -5.0, 5.0), 1: (50, -5.0, 5.0), 2: (40, -3.0, 3.0)}.items():
        rng = np.random.default_rng(seed)
        pos_m = rng.uniform(lo, hi, size=(n, 2))
        f_m = rng.uniform(0.01, 1.0, size=(n, 7))
        pc = (pos_m.astype(np.float32)[:, None, :] + C32[None, :, :] * np.float32(1.0)).reshape(-1, 2)
        cp = helpers["_cell_thin_ref"](pc, 1.0 / 4.0)
        out[f"s{seed}_pos_m"] = pos_m
        out[f"s{seed}_f_m"] = f_m
        out[f"s{seed}_pos_c"] = pc
        out[f"s{seed}_cp"] = cp
    # ring fixtures (tests/test_warp_propagation.py:79-112)
    ring = helpers["_ring"]
    posA, dirA, valA = ring((0.0, 0.0), 0.2, [0, 1, 2, 3, 4, 5, 6], [0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7])
    posB, dirB, valB = ring((10.0, 0.0), 0.2, [0, 1, 2], [0.1, 0.2, 0.3])
    w = np.exp(valA)
    out["ringAB_pos"] = np.vstack([posA, posB])
    out["ringAB_dir"] = np.concatenate([dirA, dirB])
    out["ringAB_val"] = np.concatenate([valA, valB])
    out["ringAB_cp"] = np.array([[0.0, 0.0], [10.0, 0.0]])
    out["ringAB_expected"] = np.array([(w[:, None] * posA).sum(0) / w.sum(), [10.0, 0.0]])
    pos4, dir4, val4 = ring((0.0, 0.0), 0.2, [0, 1, 2, 3], [0.1, 0.3, 0.5, 0.7])
    pos5, dir5, val5 = ring((20.0, 0.0), 0.2, [0, 1, 2, 3, 4], [0.1, 0.3, 0.5, 0.7, 0.9])
    out["ring45_pos"] = np.vstack([pos4, pos5])
    out["ring45_dir"] = np.concatenate([dir4, dir5])
    out["ring45_val"] = np.concatenate([val4, val5])
    out["ring45_cp"] = np.array([[0.0, 0.0], [20.0, 0.0]])
    np.savez_compressed(HERE / "propagation.npz", **out)

    # -- macroscopic binning (tests/test_fields.py) ---------------------------------------------
    out = {}
    rng = np.random.default_rng(3)
    x = rng.uniform(-3.0, 4.0, size=(200, 2))
    f = rng.uniform(0.01, 0.5, size=(200, 7))
    rho, u, _ = bin_fields(x, f, -3, 4, h=1.0)
    out.update(x=x, f=f, rho=rho, u=u)
    np.savez_compressed(HERE / "fields.npz", **out)

    # -- reference CPU simulator: the 13x13 rest block + central pulse of
    #    tests/test_warp_simulator.py:10-63, 3 steps, binned density --------------------------------
    f_rest = equilibrium(np.float64(1.0), np.zeros(2))
    pos, fs = [], []
    for i in range(-6, 7):
        for j in range(-6, 7):
            pos.append([float(i), float(j)])
            fs.append(equilibrium(np.float64(1.5), np.zeros(2)) if (i == 0 and j == 0) else f_rest.copy())
    pos = np.array(pos)
    fs = np.stack(fs)
    sim = Simulator([Moment(f=fs[k].copy(), x=pos[k].copy()) for k in range(len(pos))], tau=0.6, rho_rest=1.0)
    for _ in range(3):
        sim.step()
    xv = np.array([m.x for m in sim.moments])
    fv = np.stack([m.f for m in sim.moments])
    rv, _, _ = bin_fields(xv, fv, -3, 3, h=1.0)
    np.savez_compressed(HERE / "simulator.npz", pos0=pos, f0=fs, x3=xv, f3=fv, rho3=rv)

    # -- soft-outer spawn point (direbm/reference/simulator.py:153-166) on seeded sets of nearby
    #    component directions, plus the balanced sets that spawn nothing --------------------------
    from direbm.reference.types import Component, ControlPoint

    sim = Simulator([], tau=0.6)  # D2Q7, soft_mode="spawn", dx = 1
    rng = np.random.default_rng(7)
    sets = [list(rng.integers(0, 7, size=int(rng.integers(1, 40)))) for _ in range(64)]
    sets += [[1, 2, 3, 4, 5, 6], [0, 0, 0], [1, 4], [2, 5, 0], [1], [6, 6, 6, 1]]
    L = max(len(x) for x in sets)
    labels = np.full((len(sets), L), -1, dtype=np.int64)
    p = rng.uniform(-5.0, 5.0, size=(len(sets), 2))
    spawn = np.full((len(sets), 2), np.nan)
    for j, lab in enumerate(sets):
        labels[j, : len(lab)] = lab
        cp = ControlPoint(x=p[j].copy(), f=np.zeros(7))
        cp.nu_near = [Component(f=0.0, i=int(i), x=np.zeros(2)) for i in lab]
        r = sim._soft_new_point(cp)
        if r is not None:
            spawn[j] = r
    np.savez_compressed(HERE / "soft_spawn.npz", labels=labels, p=p, spawn=spawn)

    warp_reference(helpers)
    print("golden vectors written to", HERE)


def warp_reference(helpers) -> None:
    """The reference's own GPU package (direbm/warp/*.py) run unchanged on the host through
    warp_emulator.py: its stages on the propagation seeds, 3 steps of its GpuSimulator on the 13 x 13
    pulse, its FP32 physics kernels and 10 steps of its GpuHexLBM.  Written to warp_reference.npz."""
    sys.path.insert(0, str(HERE))
    import warp_emulator

    warp_emulator.install()
    from direbm import equilibrium as eq64
    from direbm.constants import ALPHA, DX, KAPPA_HARD, W
    from direbm.warp import GpuHexLBM, GpuSimulator, collide, create_control_points, disperse, equilibrium, \
        refine_control_points, resample

    out = {}
    f_rest = (1.0 * W).astype(np.float32)
    out["stage_dx"], out["stage_cs"], out["stage_kappa_hard"] = DX, DX / ALPHA, KAPPA_HARD
    # the propagation test's seeds (tests/test_warp_propagation.py:43-76)
    for seed, (n, lo, hi) in {0: (20, -5.0, 5.0), 1: (50, -5.0, 5.0), 2: (40, -3.0, 3.0)}.items():
        rng = np.random.default_rng(seed)
        pos_m = rng.uniform(lo, hi, size=(n, 2))
        f_m = rng.uniform(0.01, 1.0, size=(n, 7))
        pos_c, val_c, dir_c = disperse(pos_m, f_m, DX)
        cp, P = create_control_points(pos_c, DX / ALPHA)
        cp_ref = refine_control_points(cp, pos_c, val_c, dir_c, DX, KAPPA_HARD)
        wf = __import__("warp").array(f_rest, dtype=__import__("warp").float32)
        opos, of = resample(pos_c, val_c, dir_c, cp_ref, DX, wf)
        k = f"s{seed}_"
        out[k + "pos_m"], out[k + "f_m"] = pos_m, f_m
        out[k + "pos_c"], out[k + "val_c"], out[k + "dir_c"] = pos_c.numpy(), val_c.numpy(), dir_c.numpy()
        out[k + "cp"], out[k + "cp_refined"] = cp.numpy(), cp_ref.numpy()
        out[k + "out_pos"], out[k + "out_f"] = opos.numpy(), of.numpy()
    # GpuSimulator: the 13 x 13 rest block with a central pulse (tests/test_warp_simulator.py:10-63)
    pos, fs = [], []
    for i in range(-6, 7):
        for j in range(-6, 7):
            pos.append([float(i), float(j)])
            fs.append(eq64(np.float64(1.5 if (i == 0 and j == 0) else 1.0), np.zeros(2)))
    pos, fs = np.array(pos), np.stack(fs)
    sim = GpuSimulator(pos, fs, tau=0.6, rho_rest=1.0)
    out["sim_pos0"], out["sim_f0"] = pos, fs
    for step in range(1, 4):
        sim.step()
        x, f = sim.moments()
        out[f"sim_x{step}"], out[f"sim_f{step}"] = x, f
    # GpuSimulator on a jittered block (no lattice-exact distances, so every radius test is
    # decided away from a tie): 12 x 12 points jittered by +-0.3, a small shear flow, 3 steps
    rng = np.random.default_rng(5)
    pos = (np.stack(np.meshgrid(np.arange(12.0), np.arange(12.0), indexing="xy"), -1).reshape(-1, 2)
           + rng.uniform(-0.3, 0.3, size=(144, 2)))
    u = np.stack([0.03 * np.sin(2 * np.pi * pos[:, 1] / 12.0), 0.02 * np.cos(2 * np.pi * pos[:, 0] / 12.0)], 1)
    fs = np.stack([eq64(np.float64(1.0), u[i]) for i in range(len(pos))])
    sim = GpuSimulator(pos, fs, tau=0.7, rho_rest=1.0)
    out["jit_pos0"], out["jit_f0"] = pos, fs
    for step in range(1, 4):
        sim.step()
        x, f = sim.moments()
        out[f"jit_x{step}"], out[f"jit_f{step}"] = x, f
    # FP32 physics kernels (tests/test_warp_physics.py seeds)
    rng = np.random.default_rng(0)
    rho = rng.uniform(0.5, 2.0, size=128)
    u = rng.uniform(-0.1, 0.1, size=(128, 2))
    out["phys_rho"], out["phys_u"], out["phys_eq"] = rho, u, equilibrium(rho, u)
    rng = np.random.default_rng(1)
    fcol = rng.uniform(0.01, 1.0, size=(256, 7))
    out["phys_f"], out["phys_col"] = fcol, collide(fcol, 0.6)
    # GpuHexLBM: 21 x 21 pulse, 10 steps (tests/test_warp_lbm.py)
    lbm = GpuHexLBM(21, 21, tau=0.6)
    lbm.set_pulse(1.5)
    out["lbm_f0"] = lbm.f.numpy()
    for _ in range(10):
        lbm.step()
    out["lbm_f10"] = lbm.f.numpy()
    np.savez_compressed(HERE / "warp_reference.npz", **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to a checkout of the reference>")
    main(sys.argv[1])
