"""Failure detection through the C ABI, with every failure made on the host.

- A non-finite phi: the reference stops its loops when phi turns non-finite
  (belastic.cpp:421, :733).  Here a NaN planted into phi0 on the host gives
  CB_ENONFINITE from cb_run and the single step bodies, with the exit reason
  CB_DONE_NONFINITE, in both precisions; the handle stays usable afterwards.
- A bounded run: cb_set_launch_limit caps the attempts one cb_run may launch.  A
  run that reaches the cap returns CB_ETIMEOUT between two attempts, and a further
  run continues the same trajectory: its result equals an uninterrupted run's bit
  for bit (every kernel reduces in a fixed order).
No GPU fault, trap or hang is involved: the failing values come from the host, and
the bounded wait is a host-side count of graph launches.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _phi0(n, es=150, seed=2):
    from cudabubble_gb300 import shapes
    return shapes.seeded_ellipsoid(n, n, shapes.eps_rule(es, n), seed)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("method", ["etd2", "etd4", "euler"])
def test_nan_in_phi0_ends_the_loop(cblib, prec, method):
    from cudabubble_gb300 import capi
    m = {"euler": capi.CB_EULER, "etd2": capi.CB_ETD2, "etd4": capi.CB_ETD4}[method]
    n = 32
    phi = _phi0(n)
    phi[n // 2, n // 2, n // 2] = np.nan  # the point the reference's test reads
    dt = 1e-7 if method == "euler" else 1e-6
    st = capi.Stepper(capi.default_params(nx=n, ny=n, nz=n, epssize=150, method=m, precision=prec, time_step=dt))
    st.set_phi(phi)
    r = st.run(10)
    s = st.scalars()
    assert r["rc"] == capi.CB_ENONFINITE
    assert s["status"] == capi.CB_DONE_NONFINITE
    assert s["steps"] == 0
    # the single step body reports it too
    with pytest.raises(capi.CBError) as e:
        {"euler": st.euler_step, "etd2": st.ETD2RK, "etd4": st.ETD4RK}[method]()
    assert e.value.code == capi.CB_ENONFINITE
    # a finite state makes the handle step again
    st.set_phi(_phi0(n))
    r = st.run(3)
    assert r["rc"] == capi.CB_OK and st.scalars()["steps"] == 3
    st.close()


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
def test_launch_limit_times_out_and_resumes(cblib, prec):
    from cudabubble_gb300 import capi
    n, steps = 32, 40
    p = capi.default_params(nx=n, ny=n, nz=n, epssize=150, method=capi.CB_ETD2, precision=prec, time_step=1e-6)
    phi0 = _phi0(n)
    ref = capi.Stepper(p)
    ref.set_phi(phi0)
    assert ref.run(steps)["rc"] == capi.CB_OK
    phi_ref, s_ref = ref.get_phi(), ref.scalars()
    ref.close()

    st = capi.Stepper(p)
    st.set_phi(phi0)
    st.set_launch_limit(5)
    with pytest.raises(capi.CBError) as e:
        st.run(steps)
    assert e.value.code == capi.CB_ETIMEOUT
    s = st.scalars()
    assert s["attempts"] == 5 and 0 < s["steps"] < steps
    # continue, still bounded, until the target is reached
    left, calls = steps - s["steps"], 0
    while left > 0:
        calls += 1
        try:
            st.run(left)
        except capi.CBError as err:
            assert err.code == capi.CB_ETIMEOUT
        left = steps - st.scalars()["steps"]
        assert calls < 100
    st.set_launch_limit(0)
    s = st.scalars()
    assert s["steps"] == steps and s["rejects"] == s_ref["rejects"]
    assert s["E"] == s_ref["E"] and s["dt"] == s_ref["dt"]
    assert np.array_equal(st.get_phi(), phi_ref)
    st.close()


def test_nan_instance_in_a_batch_leaves_the_others_alone(cblib):
    """One instance of a batch starts from a phi with a NaN: it alone ends with
    CB_DONE_NONFINITE, and every other instance ends exactly as it does alone."""
    from cudabubble_gb300 import capi
    sizes = [32, 32, 48]
    plist = [capi.default_params(nx=n, ny=n, nz=n, epssize=150, method=capi.CB_ETD2, precision=capi.CB_FP32,
                                 time_step=1e-6) for n in sizes]
    phis = [_phi0(n, seed=2 + i) for i, n in enumerate(sizes)]
    bad = phis[1].copy()
    bad[16, 16, 16] = np.nan
    b = capi.Batch(plist)
    for i, ph in enumerate(phis):
        b.set_phi(i, bad if i == 1 else ph)
    b.run(8)
    assert b.scalars(1)["status"] == capi.CB_DONE_NONFINITE
    for i in (0, 2):
        st = capi.Stepper(plist[i])
        st.set_phi(phis[i])
        st.run(8)
        assert np.array_equal(st.get_phi(), b.get_phi(i)), i
        assert b.scalars(i)["status"] == capi.CB_DONE_TARGET
        st.close()
    b.close()


def test_served_request_that_blows_up_ends_alone(cblib):
    """A request whose shape is not a number (its phi0 is NaN everywhere) ends with
    CB_DONE_NONFINITE at its first attempt; the requests beside it finish as usual."""
    from cudabubble_gb300 import capi
    reqs = []
    for i, ax in enumerate(([1.6, 1.4, 0.9], [float("nan"), 1.4, 0.9], [1.5, 1.5, 1.0])):
        rq = capi.cb_request()
        rq.params = capi.default_params(nx=32, ny=32, nz=32, epssize=150, method=capi.CB_ETD2,
                                        precision=capi.CB_FP32, time_step=1e-6, rel_tol=1e-6)
        rq.axes[:] = ax
        rq.arrival_s = 0.001 * i
        rq.max_steps = 200
        reqs.append(rq)
    res, stats, _ = capi.serve_trace(reqs, 10 ** 10, max_slots_per_class=4, quantum=2)
    assert stats["completed"] == 3
    assert res[1]["status"] == capi.CB_DONE_NONFINITE and res[1]["steps"] == 0
    for i in (0, 2):
        assert res[i]["status"] in (capi.CB_DONE_TARGET, capi.CB_DONE_CONVERGED)
        assert res[i]["steps"] > 0
