"""The reference's own GPU-path tests (tests/test_warp_*.py), run against direbm_gb300.warp.

Each test keeps the reference test's inputs, seeds and assertions; where the restatement in
oracle/stages.py pins a value more tightly than the reference did (exact FP32 thinning, the
refine radius test), the tighter check is added.
"""

import numpy as np
import pytest

from oracle import stages
from oracle.fields import bin_fields
from oracle.lattices import D2Q7
from oracle.physics import collide, equilibrium, recover

pytestmark = pytest.mark.gpu


def _w():
    import direbm_gb300.warp as w

    return w


# ---- tests/test_warp_physics.py --------------------------------------------------------------

def test_warp_equilibrium_matches_reference():
    rng = np.random.default_rng(0)
    rho = rng.uniform(0.5, 2.0, size=128)
    u = rng.uniform(-0.1, 0.1, size=(128, 2))
    assert np.allclose(_w().equilibrium(rho, u), equilibrium(rho, u), rtol=1e-4, atol=1e-5)


def test_warp_collide_matches_reference():
    rng = np.random.default_rng(1)
    f = rng.uniform(0.01, 1.0, size=(256, 7))
    assert np.allclose(_w().collide(f, 0.6), collide(f, 0.6), rtol=1e-4, atol=1e-5)


def test_warp_collide_conserves_mass_and_momentum():
    rng = np.random.default_rng(2)
    f = rng.uniform(0.01, 1.0, size=(128, 7))
    rho0, u0 = recover(f)
    rho1, u1 = recover(_w().collide(f, 0.6))
    assert np.allclose(rho1, rho0, rtol=1e-5, atol=1e-5)
    assert np.allclose(rho1[:, None] * u1, rho0[:, None] * u0, atol=1e-5)


def test_runs_on_reported_device():
    assert _w().default_device() == "cuda:0"


# ---- tests/test_warp_propagation.py -----------------------------------------------------------

def _sorted_rows(a):
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def test_dispersion_matches_formula(golden):
    rng = np.random.default_rng(0)
    pos_m = rng.uniform(-5.0, 5.0, size=(20, 2))
    f_m = rng.uniform(0.01, 1.0, size=(20, 7))
    pos_c, val_c, dir_c = _w().disperse(pos_m, f_m, dx=1.0)
    expected = (pos_m[:, None, :] + D2Q7.C[None, :, :] * 1.0).reshape(-1, 2)
    assert np.allclose(pos_c.numpy(), expected, atol=1e-5)
    assert np.allclose(val_c.numpy(), f_m.reshape(-1), atol=1e-6)
    assert np.array_equal(dir_c.numpy(), np.tile(np.arange(7), 20))
    # exact FP32 formula
    np.testing.assert_array_equal(pos_c.numpy(), stages.disperse(pos_m, f_m, 1.0)[0])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_cell_thinning_matches_reference(golden, seed):
    g = golden("propagation")
    pos_c, _, _ = _w().disperse(g[f"s{seed}_pos_m"], g[f"s{seed}_f_m"], dx=1.0)
    np.testing.assert_array_equal(pos_c.numpy(), g[f"s{seed}_pos_c"])
    cp, p = _w().create_control_points(pos_c, 1.0 / 4.0)
    ref = g[f"s{seed}_cp"]
    assert p == len(ref)
    assert np.allclose(_sorted_rows(cp.numpy()), _sorted_rows(ref), atol=1e-4)
    # bit-exact against the FP32 sequential-centroid restatement, same (key) order
    cp_o, _, _, _ = stages.create_control_points(g[f"s{seed}_pos_c"], 0.25)
    np.testing.assert_array_equal(cp.numpy(), cp_o)


def test_thinning_reduces_count_and_is_bounded():
    rng = np.random.default_rng(2)
    pos_m = rng.uniform(-3.0, 3.0, size=(40, 2))
    f_m = rng.uniform(0.01, 1.0, size=(40, 7))
    pos_c, _, _ = _w().disperse(pos_m, f_m, dx=1.0)
    _, p = _w().create_control_points(pos_c, cs=1.0 / 4.0)
    assert 0 < p <= pos_c.shape[0]


def test_refine_hard_keeps_inner_moves(golden):
    g = golden("propagation")
    new = _w().refine_control_points(g["ringAB_cp"], g["ringAB_pos"], g["ringAB_val"], g["ringAB_dir"], dx=1.0,
                                     kappa_hard=4).numpy()
    assert np.allclose(new[0], g["ringAB_expected"][0], atol=1e-4)
    assert np.allclose(new[1], [10.0, 0.0], atol=1e-5)


def test_refine_kappa_threshold(golden):
    g = golden("propagation")
    new = _w().refine_control_points(g["ring45_cp"], g["ring45_pos"], g["ring45_val"], g["ring45_dir"], dx=1.0,
                                     kappa_hard=4).numpy()
    assert np.allclose(new[0], [0.0, 0.0], atol=1e-5)
    assert not np.allclose(new[1], [20.0, 0.0], atol=1e-3)


@pytest.mark.parametrize("seed", [3, 4])
def test_refine_and_resample_match_restatement(seed):
    rng = np.random.default_rng(seed)
    pos_m = rng.uniform(-6.0, 6.0, size=(300, 2))
    f_m = equilibrium(rng.uniform(0.3, 1.2, size=300), rng.uniform(-0.05, 0.05, size=(300, 2)))
    w = _w()
    pos_c, val_c, dir_c = w.disperse(pos_m, f_m, dx=1.0)
    cp, p = w.create_control_points(pos_c, 0.25)
    new = w.refine_control_points(cp, pos_c, val_c, dir_c, 1.0, 4).numpy()
    new_o, _ = stages.refine_control_points(cp.numpy(), pos_c.numpy(), val_c.numpy(), dir_c.numpy(), 1.0, 4)
    np.testing.assert_allclose(new, new_o, atol=2e-5)
    f_rest = equilibrium(np.float64(1.0), np.zeros(2))
    out_pos, out_f = w.resample(pos_c, val_c, dir_c, new, 1.0, f_rest)
    _, f_o, _ = stages.resample(pos_c.numpy(), val_c.numpy(), dir_c.numpy(), new, 1.0, f_rest)
    np.testing.assert_array_equal(out_pos.numpy(), new)
    np.testing.assert_allclose(out_f.numpy(), f_o, rtol=2e-5, atol=1e-6)


# ---- tests/test_warp_simulator.py ------------------------------------------------------------

def _rest_field(half, pulse_rho=None):
    f_rest = equilibrium(np.float64(1.0), np.zeros(2))
    pos, f = [], []
    for i in range(-half, half + 1):
        for j in range(-half, half + 1):
            fi = f_rest.copy()
            if pulse_rho is not None and i == 0 and j == 0:
                fi = equilibrium(np.float64(pulse_rho), np.zeros(2))
            pos.append([float(i), float(j)])
            f.append(fi)
    return np.array(pos), np.stack(f)


def test_gpu_rest_field_preserved():
    pos, f = _rest_field(6)
    sim = _w().GpuSimulator(pos, f, tau=0.6, rho_rest=1.0)
    for _ in range(4):
        sim.step()
    xp, fp = sim.moments()
    assert np.isfinite(fp).all()
    assert (fp.sum(axis=1) > 0).all()
    rho, _, _ = bin_fields(xp, fp, -3, 3, h=1.0)
    pop = rho > 0
    assert abs(rho[pop].mean() - 1.0) < 0.2


def test_gpu_pulse_spreads():
    pos = np.zeros((1, 2))
    f = equilibrium(np.float64(1.5), np.zeros(2))[None, :]
    sim = _w().GpuSimulator(pos, f, tau=0.6)
    for _ in range(5):
        sim.step()
    xp, fp = sim.moments()
    assert len(xp) > 1
    assert np.isfinite(fp).all()
    assert np.linalg.norm(xp, axis=1).max() > 3.0


def test_gpu_matches_v1_macroscopically(golden):
    g = golden("simulator")
    gpu = _w().GpuSimulator(g["pos0"], g["f0"], tau=0.6, rho_rest=1.0)
    for _ in range(3):
        gpu.step()
    xg, fg = gpu.moments()
    rg, _, _ = bin_fields(xg, fg, -3, 3, h=1.0)
    rv = g["rho3"]
    assert abs(rv[rv > 0].mean() - rg[rg > 0].mean()) < 0.15


def test_gpu_simulator_replans_unbounded_box():
    """A pulse spreading for 20 steps crosses several planning points without leaving the box."""
    pos = np.zeros((1, 2))
    f = equilibrium(np.float64(1.5), np.zeros(2))[None, :]
    sim = _w().GpuSimulator(pos, f, tau=0.6, replan_every=4)
    for _ in range(20):
        sim.step()
    xp, fp = sim.moments()
    assert np.isfinite(fp).all()
    assert np.linalg.norm(xp, axis=1).max() > 12.0


def test_gpu_simulator_replanned_run_equals_a_fixed_box_run():
    """Re-planning (device bounding box, state moved device to device) depends on nothing but the
    export/import it goes through: the unbounded run equals, bit for bit, a run in one fixed box
    that holds the whole spread and takes the same export/import at the same iterations (cells
    shift by whole cells; offsets and sums are cell-relative)."""
    pos = np.zeros((1, 2))
    f = equilibrium(np.float64(1.5), np.zeros(2))[None, :]
    for prec in ("fp32dev", "fp64"):
        moving = _w().GpuSimulator(pos, f, tau=0.6, replan_every=3, precision=prec)
        for _ in range(15):
            moving.step()
        moving.check()
        assert len(moving.replanned_at) >= 2
        fixed = _w().GpuSimulator(pos, f, tau=0.6, box=((-24.0, -24.0), (24.0, 24.0)), precision=prec)
        for i in range(15):
            if i in moving.replanned_at:
                _, p, ff = fixed.simulation.state()
                fixed.simulation.set_state(None, p, ff)
            fixed.step()
        a, b = moving.moments(), fixed.moments()
        np.testing.assert_array_equal(a[0], b[0], err_msg=prec)
        np.testing.assert_array_equal(a[1], b[1], err_msg=prec)


# ---- tests/test_warp_lbm.py -----------------------------------------------------------------

def test_gpu_lbm_matches_cpu(golden):
    g = golden("lbm")
    gpu = _w().GpuHexLBM(21, 21, tau=0.6)
    gpu.set_pulse(1.5)
    for _ in range(10):
        gpu.step()
    rg, _ = gpu.macroscopic()
    rc, _ = recover(g["pulse21_f10"])
    assert np.allclose(rc, rg, atol=1e-6, rtol=1e-6)  # reference asserted 1e-3


def test_gpu_lbm_rest_is_steady():
    gpu = _w().GpuHexLBM(15, 15, tau=0.6, rho0=1.0)
    r0, _ = gpu.macroscopic()
    for _ in range(20):
        gpu.step()
    r1, u1 = gpu.macroscopic()
    assert np.allclose(r1, r0, atol=1e-4)
    assert np.allclose(u1, 0.0, atol=1e-5)


def test_gpu_lbm_conserves_mass():
    gpu = _w().GpuHexLBM(25, 25, tau=0.7)
    gpu.set_pulse(2.0)
    m0 = float(gpu.f.numpy().sum())
    for _ in range(15):
        gpu.step()
    assert np.isclose(float(gpu.f.numpy().sum()), m0, rtol=1e-3)


def test_moments_are_the_state_rounded_to_float32():
    """moments() / pos_m / f_m read the state back as float32 computed on the device: positions
    are the float64 ones rounded once, f within one float32 ulp of the float64 f rounded (the
    FP32DEV store's rho W + dev summed in double-float)."""
    from direbm_gb300.lattices import D2Q7, equilibrium
    from direbm_gb300.warp import GpuSimulator

    rng = np.random.default_rng(5)
    pos = (np.stack(np.meshgrid(np.arange(14) + 0.5, np.arange(14) + 0.5), -1).reshape(-1, 2)
           + rng.uniform(-0.2, 0.2, (196, 2))).astype(np.float32)
    f = equilibrium(np.ones(196), 0.02 * rng.standard_normal((196, 2)), D2Q7).astype(np.float32)
    sim = GpuSimulator(pos, f, tau=0.7, dx=1.0)
    for _ in range(3):
        sim.step()
    p32, f32 = sim.moments()
    _, p64, f64 = sim.simulation.state_numpy()
    assert p32.dtype == np.float32 and f32.dtype == np.float32
    np.testing.assert_array_equal(p32, p64.astype(np.float32))
    spacing = np.spacing(np.abs(f64).astype(np.float32)).astype(np.float64)
    assert (np.abs(f32.astype(np.float64) - f64) <= spacing).all()
    np.testing.assert_array_equal(sim.pos_m.numpy(), p32)
    np.testing.assert_array_equal(sim.f_m.numpy(), f32)


# ---- against the reference's own Warp kernels (tests/golden/warp_reference.npz: direbm/warp/*.py
#      run unchanged on the host by tests/golden/warp_emulator.py, FP32 without contraction) ------

_W7 = np.array([0.5] + [1.0 / 12.0] * 6)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_warp_stages_match_the_reference_kernels(golden, seed):
    """disperse and the thinning bit for bit; refine to FP32 rounding of its weighted sums (hard_outer
    points kept exactly); resample to FP32 rounding, positions exact."""
    g = golden("warp_reference")
    k = f"s{seed}_"
    dx, cs, kh = float(g["stage_dx"]), float(g["stage_cs"]), int(g["stage_kappa_hard"])
    w = _w()
    pos_c, val_c, dir_c = w.disperse(g[k + "pos_m"], g[k + "f_m"], dx=dx)
    np.testing.assert_array_equal(pos_c.numpy(), g[k + "pos_c"])
    np.testing.assert_array_equal(val_c.numpy(), g[k + "val_c"])
    np.testing.assert_array_equal(dir_c.numpy(), g[k + "dir_c"])
    cp, p = w.create_control_points(pos_c, cs)
    np.testing.assert_array_equal(cp.numpy(), g[k + "cp"])
    new = w.refine_control_points(cp, pos_c, val_c, dir_c, dx, kh).numpy()
    ref = g[k + "cp_refined"]
    assert np.abs(new - ref).max() < 4e-6
    assert np.mean(new == ref) > 0.1  # the hard_outer points, kept bit for bit
    out_pos, out_f = w.resample(pos_c, val_c, dir_c, ref, dx, _W7)
    np.testing.assert_array_equal(out_pos.numpy(), g[k + "out_pos"])
    rf = g[k + "out_f"]
    assert np.abs(out_f.numpy() - rf).max() < 1e-6 * np.abs(rf).max()


def _nearest(xo, xr):
    d2 = ((xo[:, None, :] - xr[None, :, :]) ** 2).sum(-1)
    j = d2.argmin(1)
    return j, np.sqrt(d2[np.arange(len(xo)), j])


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
def test_gpu_simulator_matches_the_reference_gpu_simulator_on_the_pulse(golden, precision):
    """First step of the reference test's 13 x 13 pulse (a lattice, no tie left to rounding): every
    moment of this library's step equals the reference's to FP32 rounding."""
    g = golden("warp_reference")
    sim = _w().GpuSimulator(g["sim_pos0"], g["sim_f0"], tau=0.6, rho_rest=1.0, precision=precision)
    sim.step()
    xg, fg = (a.astype(np.float64) for a in sim.moments())
    xr, fr = g["sim_x1"].astype(np.float64), g["sim_f1"].astype(np.float64)
    assert len(xg) == len(xr)
    j, d = _nearest(xg, xr)
    assert len(np.unique(j)) == len(xr)
    assert d.max() < 5e-6
    assert np.abs(fg - fr[j]).max() < 2e-6 * np.abs(fr).max()


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("step", [1, 2, 3])
def test_gpu_simulator_matches_the_reference_step_by_step(golden, precision, step):
    """The jittered block: one step of this library from the reference's state against the
    reference's next state.
      - The moment counts are equal.
      - All but the tie-decided control points are in place to 1e-5. A tie is an inclusive radius
        test at exactly dx, common in D2Q7 at r = dx. The measured in-place share is 98.4-98.8 %
        for FP64 and 96.4 % for FP32DEV, whose cell-relative FP32 arithmetic decides more ties its
        own way.
      - The median moment's f agrees to 1e-5 in FP64. In FP32DEV it agrees to 2e-4: each moved
        point changes the weights of its neighbours' components.
      - The total mass agrees to 2 %, because the step's gap fill follows the moved points."""
    g = golden("warp_reference")
    x, f = (g["jit_pos0"], g["jit_f0"]) if step == 1 else (g[f"jit_x{step - 1}"], g[f"jit_f{step - 1}"])
    sim = _w().GpuSimulator(np.asarray(x, np.float64), np.asarray(f, np.float64), tau=0.7, rho_rest=1.0,
                            precision=precision)
    sim.step()
    xg, fg = (a.astype(np.float64) for a in sim.moments())
    xr, fr = g[f"jit_x{step}"].astype(np.float64), g[f"jit_f{step}"].astype(np.float64)
    assert len(xg) == len(xr)
    j, d = _nearest(xg, xr)
    assert np.mean(d < 1e-5) > (0.97 if precision == "fp64" else 0.95)
    assert np.median(np.abs(fg - fr[j]).max(1)) < (1e-5 if precision == "fp64" else 2e-4)
    assert abs(fg.sum() - fr.sum()) < 0.02 * fr.sum()


def test_warp_physics_and_lbm_match_the_reference_fp32_kernels(golden):
    g = golden("warp_reference")
    w = _w()
    np.testing.assert_allclose(w.equilibrium(g["phys_rho"], g["phys_u"]), g["phys_eq"], rtol=1e-6, atol=5e-7)
    np.testing.assert_allclose(w.collide(g["phys_f"], 0.6), g["phys_col"], rtol=1e-6, atol=5e-7)
    lbm = w.GpuHexLBM(21, 21, tau=0.6)
    lbm.set_pulse(1.5)
    np.testing.assert_allclose(lbm.f.numpy(), g["lbm_f0"], rtol=1e-7, atol=0)
    for _ in range(10):
        lbm.step()
    np.testing.assert_allclose(lbm.f.numpy(), g["lbm_f10"], rtol=1e-6, atol=1e-6)
