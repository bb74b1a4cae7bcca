"""Launch configurations of the tiled kernels (tile width, persistent launches) and the autotuner:
every configuration gives the same bits, the autotuner picks one of its candidates, leaves the
state untouched and caches its choice."""

import numpy as np
import pytest
import torch

from tests._cases import bounded_box, periodic_tg, rest_pulse

pytestmark = pytest.mark.gpu


def _make(lattice, instances, dx, r_res, cell, precision, x, f, inst=None):
    from direbm_gb300.sim import Instance, Simulation

    insts = [Instance(dims=tuple(i["dims"]), origin=tuple(i.get("origin", (0,) * len(i["dims"]))),
                      periodic=i.get("periodic", True), tau=i.get("tau", 0.6)) for i in instances]
    sim = Simulation(insts, lattice=lattice, precision=precision, dx=dx, r_res=r_res, cell=cell,
                     moment_capacity=4 * len(x))
    sim.set_state(inst, x, f)
    return sim


def _cases():
    x, f = periodic_tg(48, "D2Q9", seed=2)
    yield "tg", ("D2Q9", [{"dims": (48, 48)}], 1.0, 1.5, 1.0, x, f, None)
    xp, fp = rest_pulse(6, "D2Q7", 1.5)
    dims, origin = bounded_box(xp, 0.25, 3.0)
    yield "pulse", ("D2Q7", [{"dims": dims, "origin": origin, "periodic": False, "tau": 0.7}], 1.0, 1.0, 0.25, xp, fp,
                    None)
    xa, fa = periodic_tg(20, "D2Q9", seed=3)
    xb, fb = periodic_tg(36, "D2Q9", seed=4)
    yield "two", ("D2Q9", [{"dims": (20, 20)}, {"dims": (36, 36), "tau": 0.9}], 1.0, 1.5, 1.0,
                  np.concatenate([xa, xb]), np.concatenate([fa, fb]),
                  np.concatenate([np.zeros(len(xa), np.int32), np.ones(len(xb), np.int32)]))


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("name,case", list(_cases()))
def test_every_launch_configuration_gives_the_same_bits(name, case, precision):
    sim = _make(*case[:5], precision, *case[5:])
    snap = sim.snapshot()
    ref = None
    for w in (8, 16, 32, 64, 128):
        for pers in (False, True):
            sim.set_tiling(w, pers)
            assert sim.tiling() == (w, pers)
            sim.restore(snap)
            sim.step(3)
            out = [t.cpu().numpy() for t in sim.state()]
            if ref is None:
                ref = out
            else:
                for a, b in zip(out, ref):
                    np.testing.assert_array_equal(a, b, err_msg=f"{name} {w} {pers}")


def test_autotuner_picks_a_candidate_keeps_the_state_and_caches(tmp_path, monkeypatch):
    from direbm_gb300 import autotune

    monkeypatch.setenv("DIREBM_GB300_TUNE_CACHE", str(tmp_path / "tiling.json"))
    _, case = next(_cases())
    sim = _make(*case[:5], "fp32dev", *case[5:])
    before = [t.cpu().numpy() for t in sim.state()]
    choice = autotune.autotune(sim, steps=2)
    assert (choice["tile_width"], choice["persistent"]) in autotune.CANDIDATES
    assert not choice["cached"] and len(choice["timings"]) == len(autotune.CANDIDATES)
    assert sim.tiling() == (choice["tile_width"], choice["persistent"])
    after = [t.cpu().numpy() for t in sim.state()]
    for a, b in zip(before, after):
        np.testing.assert_array_equal(a, b)
    sim.set_tiling(32, False)
    again = autotune.autotune(sim, steps=2)
    assert again["cached"] and sim.tiling() == (choice["tile_width"], choice["persistent"])


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
def test_every_brick_width_gives_the_same_bits(precision):
    """The untiled window kernels (3D here, and 2D with tiles off) give each block a brick of cells;
    every brick width yields the same bits, and the 3D autotuner picks one of its candidates."""
    from direbm_gb300 import autotune

    x, f = periodic_tg(12, "D3Q19", seed=6, u0=0.04)
    sim = _make("D3Q19", [{"dims": (12, 12, 12)}], 1.0, 1.5, 1.0, precision, x, f)
    snap = sim.snapshot()
    assert sim.brick_width() == 8
    ref = None
    for w in (4, 8, 16, 32):
        sim.set_brick_width(w)
        assert sim.brick_width() == w
        sim.restore(snap)
        sim.step(3)
        out = [t.cpu().numpy() for t in sim.state()]
        if ref is None:
            ref = out
        else:
            for a, b in zip(out, ref):
                np.testing.assert_array_equal(a, b, err_msg=f"brick {w}")
    sim.restore(snap)
    choice = autotune.autotune(sim, steps=1, use_cache=False)
    assert choice["brick_width"] in autotune.BRICK_CANDIDATES and sim.brick_width() == choice["brick_width"]
    x2, f2 = periodic_tg(40, "D2Q9", seed=7)
    sim2 = _make("D2Q9", [{"dims": (40, 40)}], 1.0, 1.5, 1.0, precision, x2, f2)
    sim2.lib.dbm_sim_set_option(sim2.handle, 2, 0)  # tiles off: the untiled kernels in 2D
    snap2 = sim2.snapshot()
    ref2 = None
    for w in (8, 16, 64):
        sim2.set_brick_width(w)
        sim2.restore(snap2)
        sim2.step(2)
        out = [t.cpu().numpy() for t in sim2.state()]
        if ref2 is None:
            ref2 = out
        else:
            for a, b in zip(out, ref2):
                np.testing.assert_array_equal(a, b, err_msg=f"2D brick {w}")
    with pytest.raises(Exception):
        sim2.set_brick_width(12)
