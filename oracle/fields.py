"""Macroscopic binning restated (test oracle), direbm/fields.py:17-41.

The reference bins with the D2Q7 velocity table; ``lattice`` lets the same binning run on the
other 2D set.
"""

from __future__ import annotations

import numpy as np

from .lattices import D2Q7


def bin_fields(x, f, xmin, xmax, h, lattice=D2Q7):
    x = np.asarray(x, dtype=np.float64)
    f = np.asarray(f, dtype=np.float64)
    edges = np.arange(xmin, xmax + h, h)
    mass = f.sum(axis=1)
    mom = f @ lattice.C
    mg, _, _ = np.histogram2d(x[:, 0], x[:, 1], bins=[edges, edges], weights=mass)
    mx, _, _ = np.histogram2d(x[:, 0], x[:, 1], bins=[edges, edges], weights=mom[:, 0])
    my, _, _ = np.histogram2d(x[:, 0], x[:, 1], bins=[edges, edges], weights=mom[:, 1])
    mg, mx, my = mg.T, mx.T, my.T
    rho = mg / (h * h)
    safe = np.where(mg == 0.0, 1.0, mg)
    u = np.stack([mx / safe, my / safe], axis=-1)
    u[mg == 0.0] = 0.0
    return rho, u, (xmin, xmax, xmin, xmax)


def bin_fields3(x, f, xmin, xmax, h, lattice):
    """The same binning in 3D (test oracle; the reference has no 3D form): numpy histogramdd over
    (x, y, z) with mass and momentum weights, indexed [iz][iy][ix], density = mass / h^3."""
    x = np.asarray(x, dtype=np.float64)
    f = np.asarray(f, dtype=np.float64)
    edges = np.arange(xmin, xmax + h, h)
    mass = f.sum(axis=1)
    mom = f @ lattice.C
    grids = [np.histogramdd(x, bins=[edges] * 3, weights=w)[0].transpose(2, 1, 0)
             for w in (mass, mom[:, 0], mom[:, 1], mom[:, 2])]
    mg = grids[0]
    rho = mg / (h * h * h)
    safe = np.where(mg == 0.0, 1.0, mg)
    u = np.stack([g / safe for g in grids[1:]], axis=-1)
    u[mg == 0.0] = 0.0
    return rho, u, (xmin, xmax, xmin, xmax, xmin, xmax)
