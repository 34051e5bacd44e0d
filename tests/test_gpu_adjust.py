"""The shape adjustment (belastic::shape_adjust, belastic.cpp:174-284) on the GPU.

Checked against the reference's own run of it (the adjust32 / adjust48 golden
cases made by tests/golden/make_golden.py through oracle/ref_harness) and
against the oracle's restatement, whose accept / reject decisions the FP64
form must reproduce one for one.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np
import pytest

from cudabubble_gb300 import capi
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _case(name):
    man = json.load(open(os.path.join(GOLDEN, "manifest.json")))
    if name not in man["cases"]:
        pytest.skip(f"golden case {name} not generated")
    return man["cases"][name]


def _setup(case, precision=capi.CB_FP64, method=capi.CB_ETD2, beta=-1.0):
    nx, nz = case["nx"], case["nz"]
    eps = O.eps_from_epssize(case["epssize"], 2 * math.pi, nx)
    phi0 = O.ellipsoid_phi0(nx, nz, eps * case["width"], (1.6, 1.6, 0.8))
    p = capi.default_params(nx=nx, ny=nx, nz=nz, eps=eps, method=method, precision=precision, M1=1e4, M2=1e4,
                            alpha=-1.0 if beta <= 0 else 20.0, beta=beta, time_step=1e-6)
    st = capi.Stepper(p)
    st.set_phi(phi0)
    return st, phi0, eps


# (case, max |phi - phi_ref|, relative energy tolerance): the spread between
# independent FP64 implementations after the adjustment, which keeps dt at the
# explicit-Euler stability limit where the unstable high-|k| modes amplify
# rounding step after step (the oracle and the reference differ by 1.1e-10 in
# phi after the 86 steps of adjust32 and by 1.2e-8 after the 820 of adjust48)
ADJUST = [("adjust32", 5e-10, 1e-10), ("adjust48", 5e-8, 1e-7)]


@pytest.mark.parametrize("name,phi_tol,e_tol", ADJUST)
@pytest.mark.parametrize("method", [capi.CB_ETD2, capi.CB_EULER])
def test_fp64_matches_reference(name, phi_tol, e_tol, method):
    case = _case(name)
    st, _, _ = _setup(case, capi.CB_FP64, method)
    a = st.shape_adjust()
    assert a["status"] == capi.CB_DONE_CONVERGED
    assert a["E_start"] == pytest.approx(case["scalars"]["E0"], rel=1e-12)
    assert a["E_end"] == pytest.approx(case["scalars"]["E"], rel=e_tol)
    err = np.abs(st.get_phi() - np.load(os.path.join(GOLDEN, name + ".npz"))["phi_adjust"]).max()
    assert err < phi_tol, err
    st.close()


@pytest.mark.parametrize("name", ["adjust32", "adjust48"])
def test_fp64_decisions_match_oracle(name):
    case = _case(name)
    st, phi0, eps = _setup(case)
    a = st.shape_adjust()
    b = O.Belastic(O.Params(nx=case["nx"], nz=case["nz"], eps=eps), phi0.copy())
    why, accepted, attempts, tcur = b.shape_adjust()
    assert why == "converged"
    assert (a["steps"], a["attempts"]) == (accepted, attempts)
    assert a["attempts"] > a["steps"]  # the case rejects some attempts
    assert a["t"] == tcur  # the same sequence of FP64 dt values, summed in the same order
    st.close()


@pytest.mark.parametrize("name", ["adjust32", "adjust48"])
def test_fp32_form_tracks_reference(name):
    """The FP32 form follows another accept / reject path.  The adjustment keeps
    dt at the explicit-Euler stability limit, where rejections turn on the
    high-|k| modes' rounding, and its convergence checks fall at times set by
    the dt sequence (int(t/dt) a multiple of int(1e-4/dt)), so it stops at
    another check: measured 90 against 86 steps at 32^3 and 501 against 820 at
    48^3.  It relaxes along the same path and never past the reference's end."""
    case = _case(name)
    st, _, _ = _setup(case, capi.CB_FP32)
    a = st.shape_adjust()
    assert a["status"] == capi.CB_DONE_CONVERGED
    assert a["E_start"] == pytest.approx(case["scalars"]["E0"], rel=1e-6)
    assert min(case["checks"]) * 0.99 <= a["E_end"] < a["E_start"]
    st.close()


@pytest.mark.parametrize("precision", [capi.CB_FP64, capi.CB_FP32])
def test_loop_state_after_adjustment(precision):
    """dt, time and counters of the loop are kept; alpha, beta come from the
    adjusted state (beta <= 0) or stay as given; the loop then runs as from a
    fresh handle set to the adjusted field."""
    case = _case("adjust32")
    st, _, _ = _setup(case, precision)
    s0 = st.scalars()
    st.shape_adjust()
    s1 = st.scalars()
    assert (s1["dt"], s1["t"], s1["steps"], s1["attempts"]) == (s0["dt"], s0["t"], s0["steps"], s0["attempts"])
    assert (s1["alpha"], s1["beta"]) == (s1["V"], s1["S"])
    assert s1["E"] == pytest.approx(s1["E_el"], rel=1e-14)  # on target: no penalty
    phi = st.get_phi()
    p2 = capi.default_params(nx=case["nx"], ny=case["nx"], nz=case["nz"], eps=st.params.eps, method=capi.CB_ETD2,
                             precision=precision, M1=1e4, M2=1e4, alpha=-1.0, beta=-1.0, time_step=1e-6)
    fresh = capi.Stepper(p2)
    fresh.set_phi(phi)
    r1, r2 = st.run(30), fresh.run(30)
    assert r1["steps"] == r2["steps"] == 30
    e1, e2 = st.scalars()["E"], fresh.scalars()["E"]
    assert e1 == pytest.approx(e2, rel=1e-10 if precision == capi.CB_FP64 else 1e-5)
    st.close()
    fresh.close()
    # given targets stay
    st, _, _ = _setup(case, precision, beta=30.0)
    st.shape_adjust()
    s2 = st.scalars()
    assert (s2["alpha"], s2["beta"]) == (20.0, 30.0)
    st.close()


def test_max_steps_bound():
    case = _case("adjust48")
    st, _, _ = _setup(case)
    a = st.shape_adjust(max_steps=25)
    assert a["status"] == capi.CB_DONE_TARGET and a["steps"] == 25
    st.close()
