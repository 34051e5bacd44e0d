"""Seeded synthetic initial phase fields for the stepper's workloads.

The reference builds phi0 from ~50 hard-coded tanh profiles
(fluidbase.cpp:539-703, e.g. init_ellipse :1862-1878) or loads it from a raw
``.out`` file (ninit = 7, fluidbase.cpp:560-567).  The workloads here use one
family, seeded ellipsoids:

    phi0 = tanh(d / (sqrt(2) eps)),  d = (1 - |((x-x0)/a, (y-y0)/b, (z-z0)/c)|) * min(a, b, c)

on the reference's grid x_i = i L / n - L / 2 (fluidbase.cpp:156-161); a
union of two ellipsoids takes the max of their d values.
"""
from __future__ import annotations

import math

import numpy as np

TWO_PI = 2.0 * math.pi


def grid(n: int, L: float = TWO_PI) -> np.ndarray:
    return np.arange(n) * L / n - L / 2.0


def eps_rule(epssize: int, nx: int, lenx: float = 1.0) -> float:
    """eps of fluidbase.cpp:68-108 for a box of lenx * 2 pi."""
    xlen = lenx * TWO_PI
    h2 = 2 * xlen / 2.0 / nx
    table = {1: 2.5 * (math.sqrt(2.0) * xlen / 2.0 / nx), 2: 2.5 * h2, 3: 1.5 * h2, 4: 1.25 * h2, 5: h2,
             6: 0.7 * h2, 7: 4.0 * h2, 8: 2.5 * (math.sqrt(2.0) * xlen / 2.0 / nx) * 1.22}
    if epssize in table:
        return table[epssize]
    return epssize / 100.0 * h2 if epssize > 10 else 2.0 * h2


def ellipsoid(nx: int, nz: int, eps: float, axes, centre=(0.0, 0.0, 0.0), second=None,
              L: float = TWO_PI) -> np.ndarray:
    x = grid(nx, L)
    z = grid(nz, L)

    def dist(ax, c0):
        a, b, c = ax
        X = (x[None, None, :] - c0[0]) / a
        Y = (x[None, :, None] - c0[1]) / b
        Z = (z[:, None, None] - c0[2]) / c
        return (1.0 - np.sqrt(X * X + Y * Y + Z * Z)) * min(a, b, c)

    d = dist(axes, centre)
    if second is not None:
        d = np.maximum(d, dist(second[0], second[1]))
    return np.tanh(d / (math.sqrt(2.0) * eps))


def seeded_axes(rng: np.random.Generator):
    """a, b ~ U[1.2, 2.0], c ~ U[0.5, 1.2]."""
    return (float(rng.uniform(1.2, 2.0)), float(rng.uniform(1.2, 2.0)), float(rng.uniform(0.5, 1.2)))


def seeded_ellipsoid(nx: int, nz: int, eps: float, seed: int) -> np.ndarray:
    return ellipsoid(nx, nz, eps, seeded_axes(np.random.default_rng(seed)))


def seeded_pair(nx: int, nz: int, eps: float, seed: int) -> np.ndarray:
    """Two overlapping seeded ellipsoids with centres in [-0.8, 0.8]^3."""
    rng = np.random.default_rng(seed)
    ax = seeded_axes(rng)
    c1 = tuple(float(v) for v in rng.uniform(-0.8, 0.8, 3))
    ax2 = seeded_axes(rng)
    c2 = tuple(float(v) for v in rng.uniform(-0.8, 0.8, 3))
    return ellipsoid(nx, nz, eps, ax, centre=c1, second=(ax2, c2))
