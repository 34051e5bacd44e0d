"""Spontaneous curvature C != 0: the plain FP64 form against the oracle, and the FP32
form against the FP64 form.

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


# method, fixed dt, steps
FP32_CASES = [("euler", 1e-7, 40), ("euler", 0.0, 30), ("etd2", 0.0, 30), ("etd4", 2e-6, 10)]


@pytest.mark.parametrize("method,fixed,nsteps", FP32_CASES, ids=[f"{c[0]}-{'fixed' if c[1] else 'adapt'}"
                                                                 for c in FP32_CASES])
@pytest.mark.parametrize("n", [32, 64], ids=["one-CTA-planes", "cluster-planes"])
@pytest.mark.parametrize("C", [0.8, -0.5])
def test_fp32_curvature_matches_fp64(cblib, method, fixed, nsteps, n, C):
    """The FP32 form with curvature (its fused passes carry the third field q) against
    the plain FP64 form on the same steps: the same accepted and rejected attempts, and
    the relative energy within the benchmark spec's 1e-6.  32^2 planes run on one CTA per
    plane, 64^2 planes on two-CTA clusters."""
    from cudabubble_gb300 import capi
    st64, _ = _pair(capi, n, method, C, fixed)
    eps = O.eps_from_epssize(200, 2 * math.pi, n)
    m = {"euler": capi.CB_EULER, "etd2": capi.CB_ETD2, "etd4": capi.CB_ETD4}[method]
    p = capi.default_params(nx=n, ny=n, nz=n, eps=eps, method=m, precision=capi.CB_FP32, M1=1e4, M2=1e4,
                            time_step=1e-6, fixed_time_step=fixed, spont_c=C, accurate_coefficients=1)
    st32 = capi.Stepper(p)
    st32.set_phi(O.ellipsoid_phi0(n, n, eps, (1.6, 1.6, 0.8)))
    s0_32, s0_64 = st32.scalars(), st64.scalars()
    assert s0_32["E_el"] == pytest.approx(s0_64["E_el"], rel=1e-7)
    st64.run(nsteps)
    st32.run(nsteps)
    a, b = st32.scalars(), st64.scalars()
    assert a["steps"] == b["steps"] == nsteps
    assert a["rejects"] == b["rejects"]
    rel = abs(a["E"] - b["E"]) / abs(b["E"])
    print(f"FP32 curvature {method} n={n} C={C}: rel E {rel:.2e}, "
          f"rel V {abs(a['V'] - b['V']) / b['V']:.2e}, rel S {abs(a['S'] - b['S']) / b['S']:.2e}")
    assert rel <= 1e-6, rel
    assert np.abs(st32.get_phi() - st64.get_phi()).max() < 1e-4
    st32.close()
    st64.close()


def test_fp32_curvature_refuses_the_split_passes(cblib):
    """The split y/x plane passes carry no third field: FP32 with C != 0 on them (forced,
    or 256^2 planes, which need them) is refused before any allocation."""
    from cudabubble_gb300 import capi
    for kw in (dict(nx=32, ny=32, nz=32, xy_split=capi.XYP_SPLIT), dict(nx=256, ny=256, nz=32)):
        p = capi.default_params(precision=capi.CB_FP32, spont_c=0.5, method=capi.CB_ETD2, **kw)
        with pytest.raises(capi.CBError) as ei:
            capi.Stepper(p)
        assert ei.value.code == capi.CB_EUNSUPPORTED


def test_fp32_curvature_in_a_batch(cblib):
    """Curvature is part of a batch's size-class key: instances with and without it, of
    one grid, advance together and each ends as it does alone."""
    from cudabubble_gb300 import capi
    n = 32
    eps = O.eps_from_epssize(200, 2 * math.pi, n)
    phi0 = O.ellipsoid_phi0(n, n, eps, (1.6, 1.6, 0.8))
    plist = [capi.default_params(nx=n, ny=n, nz=n, eps=eps, method=capi.CB_ETD2, precision=capi.CB_FP32,
                                 time_step=1e-6, spont_c=C) for C in (0.8, 0.0, -0.5)]
    b = capi.Batch(plist)
    for i in range(len(plist)):
        b.set_phi(i, phi0)
    b.run(10)
    for i, p in enumerate(plist):
        st = capi.Stepper(p)
        st.set_phi(phi0)
        st.run(10)
        assert np.array_equal(st.get_phi(), b.get_phi(i)), i
        assert st.scalars()["E"] == b.scalars(i)["E"]
        st.close()
    b.close()
