"""The split plane path (a y-column pass and an x-row pass in place of the
single-CTA xy pass), through the C ABI.

* forced on small grids, it reproduces the single-CTA path: fields, scalars
  and stepped trajectories agree to rounding (FP64 1e-12, FP32 1e-6 of the
  energy);
* it carries the grids a plane does not fit one CTA for: the plain FP64 form
  at 128^3 follows the reference's own FP64 cuFFT trajectory of workload
  config 2 (128^3 ETD-RK2, adaptive dt from 1e-6): same accept/reject
  sequence and dt, energy to 1e-10, for the first 200 steps (near the dt
  stability limit the adaptive loop amplifies 1e-16 rounding differences
  between cuFFT and these transforms to ~1e-11 of the energy);
* 192^3 and 256^3 step in both precisions and agree with each other.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _stepper(capi, n, nz, method, prec, split, **kw):
    m = {"euler": capi.CB_EULER, "etd2": capi.CB_ETD2, "etd4": capi.CB_ETD4}[method]
    p = capi.default_params(nx=n, ny=n, nz=nz, epssize=150, method=m, precision=prec, xy_split=split, **kw)
    return capi.Stepper(p)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("n,nz", [(32, 32), (48, 24), (64, 64)])
def test_split_matches_single_cta(cblib, n, nz, prec):
    from cudabubble_gb300 import capi, shapes
    eps = shapes.eps_rule(150, n)
    phi0 = shapes.seeded_ellipsoid(n, nz, eps, 5)
    tol = 1e-12 if prec == 0 else 1e-6
    ftol = 1e-11 if prec == 0 else 2e-5
    res = {}
    for split in (0, 1):
        st = _stepper(capi, n, nz, "etd2", prec, split, time_step=1e-6, fixed_time_step=0.0)
        st.set_phi(phi0)
        s0 = st.scalars()
        flds = {w: st.field(w) for w in (capi.CB_FIELD_PHI, capi.CB_FIELD_LAP, capi.CB_FIELD_F, capi.CB_FIELD_NLD_HAT)}
        st.run(30)
        res[split] = (s0, flds, st.scalars(), st.get_phi())
        st.close()
    (a0, af, a1, ap), (b0, bf, b1, bp) = res[0], res[1]
    for k in ("V", "S", "E_el", "E"):
        assert abs(a0[k] - b0[k]) <= tol * abs(a0[k]), (k, a0[k], b0[k])
    for w in af:
        scale = np.abs(af[w]).max()
        assert np.abs(af[w] - bf[w]).max() <= ftol * scale, w
    if prec == 0:
        assert a1["rejects"] == b1["rejects"] and a1["dt"] == b1["dt"]
        assert np.abs(ap - bp).max() <= 1e-10
    assert abs(a1["E"] - b1["E"]) <= (1e-11 if prec == 0 else 1e-5) * abs(a1["E"])


@pytest.mark.parametrize("method", ["euler", "etd4"])
def test_split_other_methods(cblib, method):
    from cudabubble_gb300 import capi, shapes
    n = 32
    eps = shapes.eps_rule(150, n)
    phi0 = shapes.seeded_ellipsoid(n, n, eps, 7)
    ts = 1e-7 if method == "euler" else 1e-6
    out = []
    for split in (0, 1):
        st = _stepper(capi, n, n, method, capi.CB_FP64, split, time_step=ts, fixed_time_step=ts,
                      accurate_coefficients=1)
        st.set_phi(phi0)
        st.run(10)
        out.append((st.scalars()["E"], st.get_phi()))
        st.close()
    assert abs(out[0][0] - out[1][0]) <= 1e-11 * abs(out[0][0])
    assert np.abs(out[0][1] - out[1][1]).max() <= 1e-10


def test_fp64_128_config2_vs_reference(cblib):
    from cudabubble_gb300 import capi, shapes
    man = json.load(open(os.path.join(GOLDEN, "manifest.json")))
    case = man["cases"]["c2_etd2_128"]
    ref = {s["step"]: s for s in case["steps"]}
    phi0 = shapes.seeded_ellipsoid(128, 128, shapes.eps_rule(150, 128), 2)
    st = _stepper(capi, 128, 128, "etd2", capi.CB_FP64, 0, time_step=1e-6, fixed_time_step=0.0)
    st.set_phi(phi0)
    for k in (1, 10, 50, 100, 200):
        st.run(k - st.scalars()["steps"])
        s = st.scalars()
        assert s["steps"] == k
        assert s["rejects"] == ref[k]["rejects"], (k, s["rejects"], ref[k]["rejects"])
        assert s["dt"] == pytest.approx(ref[k]["dt"], rel=1e-15)
        assert s["E"] == pytest.approx(ref[k]["E"], rel=1e-10), (k, s["E"], ref[k]["E"])
    st.close()


@pytest.mark.parametrize("n", [192, 256])
def test_large_grids_both_precisions(cblib, n):
    from cudabubble_gb300 import capi, shapes
    eps = shapes.eps_rule(150, n)
    phi0 = shapes.seeded_ellipsoid(n, n, eps, 2)
    E = {}
    for prec in (0, 1):
        st = _stepper(capi, n, n, "etd2", prec, 0, time_step=1e-6, fixed_time_step=1e-6)
        st.set_phi(phi0)
        e0 = st.scalars()["E"]
        st.run(3)
        s = st.scalars()
        assert s["steps"] == 3 and np.isfinite(s["E"])
        E[prec] = (e0, s["E"])
        st.close()
    assert abs(E[1][0] - E[0][0]) <= 1e-6 * abs(E[0][0])
    assert abs(E[1][1] - E[0][1]) <= 1e-5 * abs(E[0][1])
