"""GPU stepper against the reference's own FP64 cuFFT outputs (tests/golden,
made by tests/golden/make_golden.py from the unmodified reference build),
through the C ABI.

Bars: the plain FP64 form reproduces the reference to max|phi - phi_ref| <=
1e-10 (fields to 1e-11 of their magnitude).  The FP32 form (FP32 FFT and
pointwise, FP64 reductions, the state's real-space field in double-float) is
held to per-case relative energy bounds a few times above the measured
errors, and makes the reference's accept / reject decisions (the same
rejection count at every checked step).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def man():
    return json.load(open(os.path.join(GOLDEN, "manifest.json")))


def _params(capi, case, method, prec, **kw):
    m = {"euler": capi.CB_EULER, "etd2": capi.CB_ETD2, "etd4": capi.CB_ETD4}[method]
    return capi.default_params(nx=case["nx"], ny=case["nx"], nz=case["nz"], epssize=case["epssize"], method=m,
                               precision=prec, M1=case.get("M", 1e4), M2=case.get("M", 1e4), **kw)


def _rel(a, ref):
    return np.abs(a - ref).max() / np.abs(ref).max()


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("name", ["f16", "f24", "f32x16"])
def test_fields_vs_reference(cblib, man, name, prec):
    from cudabubble_gb300 import capi
    case = man["cases"][name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    sc = case["scalars"]
    dt = case["dt"]
    tol = 1e-11 if prec == 0 else 2e-5
    t4 = 1e-10 if prec == 0 else 3e-3  # fourth-derivative fields: see test_gpu_fields
    st = capi.Stepper(_params(capi, case, "etd2", prec, time_step=dt, fixed_time_step=dt))
    st.set_phi(g["phi0"])
    fields = {"fd": capi.CB_FIELD_FD, "lap": capi.CB_FIELD_LAP, "f": capi.CB_FIELD_F, "g0": capi.CB_FIELD_G0,
              "nld": capi.CB_FIELD_NLD, "dx": capi.CB_FIELD_DX, "dy": capi.CB_FIELD_DY, "dz": capi.CB_FIELD_DZ,
              "s": capi.CB_FIELD_S, "nld_hat": capi.CB_FIELD_NLD_HAT}
    for k, w in fields.items():
        err = _rel(st.field(w), g[k])
        lim = t4 if k in ("g0", "nld", "nld_hat") else (5 * tol if k in ("lap", "f", "s") else tol)
        assert err <= lim, (k, err)
    s = st.scalars()
    stol = 1e-12 if prec == 0 else 1e-6
    for k in ("V", "S", "E_el", "E"):
        assert abs(s[k] - sc[k]) <= stol * abs(sc[k]), (k, s[k], sc[k])
    st.ETD2RK()
    assert np.abs(st.get_phi() - g["etd2_1"]).max() <= (1e-12 if prec == 0 else 2e-6)
    st.close()
    st = capi.Stepper(_params(capi, case, "euler", prec, time_step=dt, fixed_time_step=dt))
    st.set_phi(g["phi0"])
    assert _rel(st.field(capi.CB_FIELD_RHS), g["rhs_euler"]) <= t4
    st.euler_step()
    assert np.abs(st.get_phi() - g["euler1"]).max() <= (1e-13 if prec == 0 else 2e-6)
    st.close()
    # ETD-RK4 in the reference-exact closed forms: bounded by their conditioning
    st = capi.Stepper(_params(capi, case, "etd4", prec, time_step=dt, fixed_time_step=dt, accurate_coefficients=0))
    st.set_phi(g["phi0"])
    st.ETD4RK()
    assert np.abs(st.get_phi() - g["etd4_1"]).max() <= 2e-5
    st.close()


# name, FP64 max|phi - phi_ref|, FP32 relative energy bound.  Measured FP32 errors on
# GB300: euler32 1.3e-9, euler32_adapt 4.7e-9, etd2_32 1.9e-10, etd2_48 5.0e-9,
# c1_euler64 3.4e-9, each with the reference's rejection count
TRAJ = [("euler32", 1e-12, 2e-8), ("euler32_adapt", 1e-10, 5e-8), ("etd2_32", 1e-10, 2e-8),
        ("etd2_48", 1e-10, 5e-8), ("c1_euler64", 1e-10, 5e-8)]


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("name,tol64,relE32", TRAJ, ids=[t[0] for t in TRAJ])
def test_trajectory_vs_reference(cblib, man, name, tol64, relE32, prec):
    from cudabubble_gb300 import capi
    case = man["cases"][name]
    snaps = np.load(os.path.join(GOLDEN, name + ".npz"))
    st = capi.Stepper(_params(capi, case, case["method"], prec, time_step=case["time_step"],
                              fixed_time_step=case["fixed"]))
    st.set_phi(snaps["phi_000000"])
    last = case["steps"][-1]
    st.run(last["step"])
    s = st.scalars()
    assert s["steps"] == last["step"]
    if prec == 0:
        assert s["rejects"] == case["end"]["rejects"]
        assert s["dt"] == pytest.approx(last["dt"], rel=1e-15)
        err = np.abs(st.get_phi() - snaps["phi_%06d" % last["step"]]).max()
        assert err <= tol64, err
        assert s["E"] == pytest.approx(last["E"], rel=1e-11)
    else:
        rel = abs(s["E"] - last["E"]) / abs(last["E"])
        print(f"{name} FP32: rejects {s['rejects']} (reference {case['end']['rejects']}), rel E error {rel:.2e}")
        assert rel <= relE32, (s["E"], last["E"])
        assert s["rejects"] == case["end"]["rejects"]
    st.close()


def test_config2_fp32_energy_error_vs_reference(cblib, man):
    """Workload config 2: 128^3 ETD-RK2, adaptive dt from 1e-6, 1000 steps,
    against the reference's FP64 cuFFT trajectory.  The FP32 form makes the
    reference's accept / reject decisions step for step under its strict rule
    (248 rejections, all on the same steps).  Measured on GB300: relative
    energy error <= 4.0e-8 at every checkpoint and 1.6e-8 at step 1000.  Bar:
    2e-7 at every checkpoint (the benchmark spec's is 1e-6 at step 1000),
    rejections equal throughout."""
    from cudabubble_gb300 import capi, shapes
    case = man["cases"]["c2_etd2_128"]
    phi0 = shapes.seeded_ellipsoid(128, 128, shapes.eps_rule(150, 128), 2)
    st = capi.Stepper(_params(capi, case, "etd2", capi.CB_FP32, time_step=1e-6, fixed_time_step=0.0))
    st.set_phi(phi0)
    ref = {s["step"]: s for s in case["steps"]}
    errs = {}
    for k in (1, 10, 20, 30, 100, 150, 300, 500, 700, 1000):
        st.run(k - st.scalars()["steps"])
        s = st.scalars()
        errs[k] = abs(s["E"] - ref[k]["E"]) / abs(ref[k]["E"])
        assert s["rejects"] == ref[k]["rejects"], (k, s["rejects"], ref[k]["rejects"])
    print("config 2 FP32 rel E error vs reference:", {k: f"{v:.2e}" for k, v in errs.items()})
    assert max(errs.values()) <= 2e-7, errs
    st.close()
