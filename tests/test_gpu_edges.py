"""Edge cases of the simulator on the GPU: empty and tiny states, an empty instance in a batch,
the capacity limit, a bounded box that material leaves, and bad arguments (all checked against the
oracle where a value exists)."""

import numpy as np
import pytest

from _cases import oracle_spec, periodic_tg
from oracle import grid_step

pytestmark = pytest.mark.gpu


def _sim(instances, precision="fp64", lattice="D2Q9", cap=0, **kw):
    from direbm_gb300.sim import Instance, Simulation

    return Simulation([Instance(**i) for i in instances], lattice=lattice, precision=precision, dx=1.0, r_res=1.5,
                      cell=1.0, moment_capacity=cap, **kw)


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
def test_empty_state_steps_to_empty(precision):
    sim = _sim([dict(dims=(16, 16))], precision)
    sim.set_state(None, np.zeros((0, 2)), np.zeros((0, 9)))
    assert sim.count() == 0
    sim.step(3)
    assert sim.count() == 0
    assert sim.status() == 0
    assert float(sim.conservation()[0, 0]) == 0.0


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
def test_single_moment_matches_oracle(precision):
    """One moment alone in a periodic box: thinning gives one control point per direction cell,
    the gap fill fills the rest of each control point's directions with the rest state."""
    from oracle.lattices import BY_NAME
    from oracle.physics import equilibrium

    x = np.array([[8.3, 7.6]])
    f = equilibrium(np.array([1.2]), np.array([[0.02, -0.01]]), BY_NAME["D2Q9"])
    inst = dict(dims=(16, 16), tau=0.7)
    sim = _sim([inst], precision)
    sim.set_state(None, x, f)
    sim.step(1)
    _, xg, fg = sim.state_numpy()
    spec = oracle_spec("D2Q9", [inst], 1.0, 1.5, 1.0)
    ref = grid_step.step(spec, grid_step.from_world(spec, np.zeros(1, np.int64), x, f))
    _, xo, fo = grid_step.to_world(spec, ref)
    assert len(xg) == len(xo) == 9
    tol = 1e-12 if precision == "fp64" else 1e-6
    np.testing.assert_allclose(xg, xo, rtol=0, atol=tol)
    np.testing.assert_allclose(fg, fo, rtol=0, atol=tol * np.abs(fo).max())


def test_empty_instance_in_a_batch_is_left_alone():
    x, f = periodic_tg(20, "D2Q9", seed=5)
    insts = [dict(dims=(20, 20)), dict(dims=(12, 12)), dict(dims=(20, 20), tau=0.8)]
    inst_of = np.concatenate([np.zeros(len(x), np.int32), np.full(len(x), 2, np.int32)])
    sim = _sim(insts, cap=2 * len(inst_of))
    sim.set_state(inst_of, np.concatenate([x, x]), np.concatenate([f, f]))
    sim.step(2)
    ig, _, _ = sim.state_numpy()
    assert (ig != 1).all()
    cons = sim.conservation().cpu().numpy()
    assert cons[1, 0] == 0.0 and cons[0, 0] > 0 and cons[2, 0] > 0


def test_capacity_is_enforced():
    from direbm_gb300._lib import DbmError

    x, f = periodic_tg(16, "D2Q9", seed=1)
    sim = _sim([dict(dims=(16, 16))], cap=0)  # capacity = cell count = 256 = len(x)
    sim.set_state(None, x, f)
    with pytest.raises(DbmError):
        sim.set_state(None, np.concatenate([x, x]), np.concatenate([f, f]))


def test_bounded_box_reports_material_leaving():
    from direbm_gb300._lib import ST_OUT_OF_BOX, DbmError

    x, f = periodic_tg(12, "D2Q9", seed=2)
    sim = _sim([dict(dims=(12, 12), periodic=False)])
    sim.set_state(None, x, f)
    sim.step(1)
    assert sim.status() & ST_OUT_OF_BOX
    with pytest.raises(DbmError):
        sim.check_status()


def test_bad_arguments_raise():
    from direbm_gb300._lib import DbmError

    with pytest.raises(DbmError):
        _sim([dict(dims=(4, 4))])  # periodic box narrower than one window
    with pytest.raises(DbmError):
        _sim([dict(dims=(16, 16), tau=0.5)])  # tau must exceed 1/2
    sim = _sim([dict(dims=(16, 16), periodic=False)])
    with pytest.raises(DbmError):
        sim.set_state(None, np.array([[20.0, 3.0]]), np.ones((1, 9)) / 9)  # outside its bounded box
    sim = _sim([dict(dims=(16, 16))])
    sim.set_state(None, np.array([[20.0, 3.0]]), np.ones((1, 9)) / 9)  # a periodic box wraps it
    _, xg, _ = sim.state_numpy()
    np.testing.assert_allclose(xg, [[4.0, 3.0]])
    with pytest.raises(DbmError):
        sim.set_tiling(12, False)  # must divide 256
    with pytest.raises(DbmError):
        sim.set_tau([0.4])


def test_state_into_caller_buffers_and_status_reads_on_busy_copy_streams():
    """state(out=...) writes the same rows as state() into the caller's (larger) buffers and checks
    them; count and status read correctly while a bulk copy runs on another stream."""
    import torch

    from direbm_gb300.sim import Instance, Simulation

    x, f = periodic_tg(24, "D2Q9", seed=5)
    sim = Simulation([Instance(dims=(24, 24), tau=0.7)], lattice="D2Q9", precision="fp32dev", r_res=1.5, cell=1.0)
    sim.set_state(None, x, f)
    sim.step(2)
    ref = [t.clone() for t in sim.state()]
    n = ref[0].shape[0]
    out = (torch.full((n + 7,), -1, dtype=torch.int32, device="cuda"),
           torch.full((n + 7, 2), -1.0, dtype=torch.float64, device="cuda"),
           torch.full((n + 7, 9), -1.0, dtype=torch.float64, device="cuda"))
    side = torch.cuda.Stream()
    big = torch.empty(64 << 20, dtype=torch.uint8).pin_memory()
    dbig = torch.empty(big.shape, dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(side):
        dbig.copy_(big, non_blocking=True)
    got = sim.state(out=out)
    assert sim.count() == n and sim.status() == 0
    torch.cuda.synchronize()
    for g, r, o in zip(got, ref, out):
        assert g.data_ptr() == o.data_ptr() and torch.equal(g, r)
        assert bool((o[n:] == -1).all())
    with pytest.raises(ValueError):
        sim.state(out=(out[0][: n - 1], out[1], out[2]))
    with pytest.raises(ValueError):
        sim.state(out=(out[0], out[1].float(), out[2]))


def test_pipelined_load_and_export_without_host_waits():
    """set_state(check=False) defers the bad-input check to status(), and state_into writes the
    same rows as state() into capacity-sized buffers without reading the count on the host."""
    import torch

    from direbm_gb300._lib import ST_BAD_INPUT, DbmError

    x, f = periodic_tg(24, "D2Q9", seed=6)
    sim = _sim([dict(dims=(24, 24), tau=0.7)], "fp32dev")
    sim.set_state(None, x, f, check=False)
    sim.step(2)
    C = sim.capacity
    out = (torch.full((C,), -1, dtype=torch.int32, device="cuda"),
           torch.full((C, 2), -1.0, dtype=torch.float64, device="cuda"),
           torch.full((C, 9), -1.0, dtype=torch.float64, device="cuda"))
    assert sim.state_into(out) is out
    ref = sim.state()
    n = sim.count()
    for o, r in zip(out, ref):
        assert torch.equal(o[:n], r)
    assert sim.status() == 0
    with pytest.raises(ValueError):
        sim.state_into((out[0][: C - 1], out[1], out[2]))
    # a moment outside its bounded box: no error at the load, the bit waits in the status word
    sim = _sim([dict(dims=(16, 16), periodic=False)])
    sim.set_state(None, np.array([[20.0, 3.0]]), np.ones((1, 9)) / 9, check=False)
    assert sim.status() & ST_BAD_INPUT
    with pytest.raises(DbmError):
        sim.check_status()
