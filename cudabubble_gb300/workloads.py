"""Seeded synthetic workloads of the benchmark configurations.

* batched (config 4): 64 vesicles with grids drawn uniformly from
  {32, 48, 64, 96, 128}^3, ellipsoid axes as in config 2, the volume target
  alpha scaled by U[0.6, 0.95] (beta from t = 0), ETD-RK2 with per-instance
  adaptive dt;
* served (config 5): Poisson arrivals at a given rate, grids from
  {32, 64, 96, 128, 192, 256}^3 with weights 30/25/20/15/7/3 %, each request a
  relaxation to |dE/E| < rel_tol with a step cap.

There is no public dataset behind these: every input is generated here from
a numpy PCG64 stream with the stated seed.
"""
from __future__ import annotations

import math

import numpy as np

from . import capi, shapes

BATCH_SIZES = (32, 48, 64, 96, 128)
SERVE_SIZES = (32, 64, 96, 128, 192, 256)
SERVE_WEIGHTS = (0.30, 0.25, 0.20, 0.15, 0.07, 0.03)
EPSSIZE = 150
TWO_PI = 2.0 * math.pi


def _axes(rng):
    return (rng.uniform(1.2, 2.0), rng.uniform(1.2, 2.0), rng.uniform(0.5, 1.2))


def batched(count: int = 64, seed: int = 4, precision: int = capi.CB_FP32):
    """(params list, phi0 list) of the batched workload.  alpha is the volume
    of phi0 times U[0.6, 0.95]; beta is phi0's area, computed with a
    throw-away FP64 handle per instance."""
    rng = np.random.default_rng(seed)
    plist, phis = [], []
    for _ in range(count):
        n = int(rng.choice(BATCH_SIZES))
        ax = _axes(rng)
        scale = rng.uniform(0.6, 0.95)
        eps = shapes.eps_rule(EPSSIZE, n)
        phi = shapes.ellipsoid(n, n, eps, ax)
        probe = capi.Stepper(capi.default_params(nx=n, ny=n, nz=n, epssize=EPSSIZE, method=capi.CB_ETD2,
                                                 precision=capi.CB_FP64))
        probe.set_phi(phi)
        s = probe.scalars()
        probe.close()
        plist.append(capi.default_params(nx=n, ny=n, nz=n, epssize=EPSSIZE, method=capi.CB_ETD2,
                                         precision=precision, time_step=1e-6, fixed_time_step=0.0,
                                         alpha=s["V"] * scale, beta=s["S"]))
        phis.append(phi)
    return plist, phis


def served(rate_hz: float = 200.0, duration_s: float = 2.0, seed: int = 5, rel_tol: float = 1e-8,
           max_steps: int = 200, precision: int = capi.CB_FP32):
    """cb_request list of a Poisson arrival trace over `duration_s` seconds."""
    rng = np.random.default_rng(seed)
    reqs, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= duration_s:
            break
        n = int(rng.choice(SERVE_SIZES, p=SERVE_WEIGHTS))
        rq = capi.cb_request()
        rq.params = capi.default_params(nx=n, ny=n, nz=n, epssize=EPSSIZE, method=capi.CB_ETD2,
                                        precision=precision, time_step=1e-6, fixed_time_step=0.0, rel_tol=rel_tol)
        rq.axes[:] = list(_axes(rng))
        rq.centre[:] = [0.0, 0.0, 0.0]
        rq.axes2[:] = [0.0, 0.0, 0.0]
        rq.centre2[:] = [0.0, 0.0, 0.0]
        rq.arrival_s = t
        rq.max_steps = max_steps
        reqs.append(rq)
    return reqs
