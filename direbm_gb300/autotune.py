"""Autotuner for the launch configuration of the window kernels.

In 3D the untiled window kernels give each block a brick of 256 cells; its width along x is the
choice there (``BRICK_CANDIDATES``), timed the same way.  The rest of this note is about 2D.

The thinning/refine, weights and gather kernels run one 256-thread block per tile of
w x 256/w cells and stage the tile plus a halo in shared memory; the halo share of the staged
region, the staging capacity and the row-segment lengths all depend on w, and the kernels can be
launched one block per tile or persistently (a few resident blocks per SM striding over the tile
list).  Every setting gives bit-identical results, so the choice is purely a speed question:
``autotune`` times a short run of the simulator's own step from one snapshot for each candidate
and keeps the fastest.  Choices are cached in a JSON file keyed by the GPU, the lattice, the
precision, the radius and displacement in cell units and the moment density, so a later run with
the same shape of problem skips the timing.
"""

from __future__ import annotations

import json
import os
from pathlib import Path

import torch

from .sim import Simulation

CANDIDATES = tuple((w, p) for w in (32, 16, 64, 8) for p in (False, True))
BRICK_CANDIDATES = (8, 4, 16, 32)  # 3D brick widths along x (8 x 8 x 4, 4 x 8 x 8, 16 x 4 x 4, 32 x 4 x 2)


def cache_file() -> Path:
    p = os.environ.get("DIREBM_GB300_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "direbm_gb300" / "tiling.json"


def problem_key(sim: Simulation, moments: int) -> str:
    dev = torch.cuda.get_device_name(sim.device)
    density = moments / max(sim.ncells, 1)
    return (f"{dev}|{sim.lattice.name}|{sim.precision}|R={sim.r_res / sim.cell:.4g}|cd={sim.dx / sim.cell:.4g}"
            f"|density={density:.2g}")


def _load(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def apply_cached(sim: Simulation) -> dict | None:
    """Apply a cached choice for this problem, if there is one; returns it."""
    entry = _load(cache_file()).get(problem_key(sim, sim.count()))
    if entry:
        if entry.get("brick_width"):
            sim.set_brick_width(entry["brick_width"])
        else:
            sim.set_tiling(entry["tile_width"], entry["persistent"])
    return entry


def _autotune_bricks(sim: Simulation, steps: int, key: str, use_cache: bool) -> dict:
    """3D: time each brick width of the untiled window kernels from one snapshot, keep the fastest."""
    snap = sim.snapshot()
    it = sim.iteration
    timings = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.device(sim.device):
        for w in BRICK_CANDIDATES:
            sim.set_brick_width(w)
            sim.restore(snap)
            sim.step(1)  # warm-up: captures this configuration's graphs
            sim.restore(snap)
            torch.cuda.synchronize()
            e0.record()
            sim.step(steps)
            e1.record()
            torch.cuda.synchronize()
            timings[f"brick{w}"] = e0.elapsed_time(e1) / steps
    w, ms = min(zip(BRICK_CANDIDATES, timings.values()), key=lambda cv: cv[1])
    sim.set_brick_width(w)
    sim.restore(snap, it)
    entry = {"tile_width": None, "persistent": None, "brick_width": int(w), "ms_per_step": float(ms),
             "timings": timings}
    if use_cache:
        path = cache_file()
        data = _load(path)
        data[key] = entry
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(data, indent=1, sort_keys=True))
        except OSError:
            pass
    return dict(entry, cached=False)


def autotune(sim: Simulation, steps: int = 2, candidates=CANDIDATES, use_cache: bool = True) -> dict:
    """Time ``steps`` steps of the loaded state under each (tile width, persistent) candidate (3D:
    each brick width), apply the fastest and return {tile_width, persistent, [brick_width,]
    ms_per_step, timings}.  The simulator's state and iteration count are left as they were."""
    moments = sim.count()
    key = problem_key(sim, moments)
    if use_cache:
        hit = apply_cached(sim)
        if hit:
            return dict(hit, cached=True)
    if sim.lattice.D != 2:
        return _autotune_bricks(sim, steps, key, use_cache)
    snap = sim.snapshot()
    it = sim.iteration
    timings = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.device(sim.device):
        for w, pers in candidates:
            sim.set_tiling(w, pers)
            sim.restore(snap)
            sim.step(1)  # warm-up: captures this configuration's graphs
            sim.restore(snap)
            torch.cuda.synchronize()
            e0.record()
            sim.step(steps)
            e1.record()
            torch.cuda.synchronize()
            timings[f"{w}x{256 // w}{'-persistent' if pers else ''}"] = e0.elapsed_time(e1) / steps
    best = min(zip(candidates, timings.values()), key=lambda cv: cv[1])
    (w, pers), ms = best
    sim.set_tiling(w, pers)
    sim.restore(snap, it)
    entry = {"tile_width": int(w), "persistent": bool(pers), "ms_per_step": float(ms), "timings": timings}
    if use_cache:
        path = cache_file()
        data = _load(path)
        data[key] = entry
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(data, indent=1, sort_keys=True))
        except OSError:
            pass
    return dict(entry, cached=False)
