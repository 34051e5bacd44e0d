"""Spontaneous curvature C != 0 in the plain FP64 form, against the oracle.

The reference stubs it (phasefield.cpp:183-250; its curvature field is NULL,
fluidbase.cpp:150), so parity is with the oracle's restatement of the
commented-out formulas, whose g_C tests/test_oracle.py checks as the variational
derivative of E_el.  In the ETD loops the curvature terms g_C - g0 enter the
nonlinear part whole (no counterpart in the reference, whose nld ignores C).
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pair(capi, n, method, C, fixed, M=1e4):
    eps = O.eps_from_epssize(200, 2 * math.pi, n)
    phi0 = O.ellipsoid_phi0(n, n, eps, (1.6, 1.6, 0.8))
    m = {"euler": capi.CB_EULER, "etd2": capi.CB_ETD2, "etd4": capi.CB_ETD4}[method]
    p = capi.default_params(nx=n, ny=n, nz=n, eps=eps, method=m, precision=capi.CB_FP64, M1=M, M2=M,
                            time_step=1e-6, fixed_time_step=fixed, spont_c=C, accurate_coefficients=1)
    st = capi.Stepper(p)
    st.set_phi(phi0)
    op = O.Params(nx=n, nz=n, eps=eps, M1=M, M2=M, time_step=1e-6, fixed_time_step=fixed, C=C,
                  accurate_coefficients=True, etd4_reference_combine=True)
    if method == "euler":
        op.grow_factor, op.dt_cap, op.cap_probe = 1.4, 1e300, 0.0
    return st, O.Belastic(op, phi0)


@pytest.mark.parametrize("method,fixed,nsteps", [("euler", 1e-7, 40), ("euler", 0.0, 30), ("etd2", 0.0, 30),
                                                 ("etd4", 2e-6, 10)])
@pytest.mark.parametrize("C", [0.8, -0.5])
def test_fp64_curvature_matches_oracle(cblib, method, fixed, nsteps, C):
    from cudabubble_gb300 import capi
    st, b = _pair(capi, 32, method, C, fixed)
    r = st.run(nsteps)
    assert r["steps"] == nsteps
    why = b.run_static(nsteps) if method == "euler" else b.run_static_fEIF(nsteps, method)
    assert why == "max_steps"
    s = st.scalars()
    assert s["rejects"] == b.rejects
    err = np.abs(st.get_phi() - b.pd.d).max()
    assert err < 1e-10, err
    assert s["E"] == pytest.approx(b.getstaticenergy(b.pd), rel=1e-10)
    assert s["E_el"] == pytest.approx(b.pd.elastic_eng(), rel=1e-10)
    st.close()


def test_curvature_changes_the_energy_and_zero_is_the_reference(cblib):
    from cudabubble_gb300 import capi
    a, _ = _pair(capi, 32, "etd2", 0.0, 1e-6)
    c, _ = _pair(capi, 32, "etd2", 0.8, 1e-6)
    assert a.scalars()["E_el"] != c.scalars()["E_el"]
    a.run(5)
    c.run(5)
    assert np.abs(a.get_phi() - c.get_phi()).max() > 1e-6
    a.close()
    c.close()


def test_fp32_form_rejects_curvature(cblib):
    from cudabubble_gb300 import capi
    p = capi.default_params(nx=32, ny=32, nz=32, precision=capi.CB_FP32, spont_c=0.5)
    with pytest.raises(capi.CBError) as ei:
        capi.Stepper(p)
    assert ei.value.code == capi.CB_EUNSUPPORTED
