"""The xy-path autotuner (cb_autotune) and the explicit path codes of
cb_params.xy_split.  No counterpart in the reference, which has one path.

One GPU run stopped with an illegal memory access inside the tuner's timing of the batched
pool's classes, and reading the code has not found the cause.  The tuner is therefore kept
out of every default path, and its tests run only when asked for (CB_TEST_AUTOTUNE=1); the
explicit path codes, which the tuner chooses among, are tested always."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

tuner = pytest.mark.skipif(os.environ.get("CB_TEST_AUTOTUNE") != "1",
                           reason="the xy-path tuner runs only when asked for (CB_TEST_AUTOTUNE=1)")


def _stepper(capi, n, nz, prec, path, method="etd2"):
    from cudabubble_gb300 import shapes
    eps = shapes.eps_rule(150, n)
    m = {"etd2": capi.CB_ETD2, "etd4": capi.CB_ETD4, "euler": capi.CB_EULER}[method]
    p = capi.default_params(nx=n, ny=n, nz=nz, eps=eps, method=m, precision=prec, M1=1e4, M2=1e4,
                            time_step=1e-6, fixed_time_step=0.0, xy_split=path)
    st = capi.Stepper(p)
    st.set_phi(shapes.seeded_ellipsoid(n, nz, eps, 3))
    return st


@tuner
@pytest.mark.parametrize("n,prec", [(64, 1), (128, 1), (64, 0)])
def test_autotune_keeps_the_state_and_picks_a_timed_path(cblib, n, prec):
    from cudabubble_gb300 import capi
    st = _stepper(capi, n, n, prec, capi.XYP_AUTO)
    st.run(5)
    before = st.scalars()
    r = st.autotune(8)
    after = st.scalars()
    for k in ("E", "V", "S", "dt", "t", "steps", "rejects"):
        assert after[k] == before[k], k
    assert r["path"] in r["timed"] and all(v > 0 for v in r["timed"].values())
    if prec == 1:
        assert capi.XYP_CLUSTER in r["timed"] and capi.XYP_SINGLE in r["timed"]
    st.close()
    # a handle tuned before its first step runs exactly as one created on the chosen path
    # (the paths sum in different orders, so the comparison starts from the same phi0)
    st = _stepper(capi, n, n, prec, capi.XYP_AUTO)
    r = st.autotune(8)
    other = _stepper(capi, n, n, prec, r["path"])
    st.run(25)
    other.run(25)
    assert np.array_equal(st.get_phi(), other.get_phi())
    st.close()
    other.close()


def test_cluster_pass_at_192_matches_the_split_passes(cblib):
    """192^2 planes: the two-CTA cluster fused pass (one CTA per SM, ~157 KB of shared
    memory each) against the split y/x passes, FP32 form."""
    from cudabubble_gb300 import capi
    res = {}
    for path in (capi.XYP_CLUSTER, capi.XYP_SPLIT):
        st = _stepper(capi, 192, 32, capi.CB_FP32, path)
        st.run(15)
        res[path] = (st.scalars(), st.get_phi())
        st.close()
    (a, pa), (b, pb) = res[capi.XYP_CLUSTER], res[capi.XYP_SPLIT]
    assert a["rejects"] == b["rejects"] and a["dt"] == b["dt"]
    assert a["E"] == pytest.approx(b["E"], rel=1e-7)
    assert np.abs(pa - pb).max() < 1e-5


@tuner
def test_autotune_at_192_times_cluster_and_split(cblib):
    from cudabubble_gb300 import capi
    st = _stepper(capi, 192, 32, capi.CB_FP32, capi.XYP_AUTO)
    r = st.autotune(4)
    assert set(r["timed"]) == {capi.XYP_CLUSTER, capi.XYP_SPLIT}
    st.run(3)
    st.close()


def test_bad_path_code(cblib):
    from cudabubble_gb300 import capi
    p = capi.default_params(nx=32, ny=32, nz=32, xy_split=7)
    with pytest.raises(capi.CBError) as ei:
        capi.Stepper(p)
    assert ei.value.code == capi.CB_EINVAL
