"""Batched and served modes on the GPU, through the C ABI.

Every instance keeps its own buffers, dt, accept/reject state and
fixed-order FP64 reductions, so a vesicle's trajectory must be bitwise the
same alone, in a batch of uneven grids, and in the continuous-batching
server's mix.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(capi, n, method, prec=1, **kw):
    m = {"euler": capi.CB_EULER, "etd2": capi.CB_ETD2, "etd4": capi.CB_ETD4}[method]
    base = dict(nx=n, ny=n, nz=n, epssize=150, method=m, precision=prec, time_step=1e-6, fixed_time_step=0.0,
                M1=1e4, M2=1e4)
    base.update(kw)
    return capi.default_params(**base)


MIX = [(16, "etd2", 3), (24, "etd2", 4), (32, "etd2", 5), (32, "etd4", 6), (48, "etd2", 7), (32, "euler", 8),
       (64, "etd2", 9)]


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
def test_batch_matches_single_instances(cblib, prec):
    from cudabubble_gb300 import capi, shapes
    mix = [m for m in MIX if not (prec == 0 and m[0] > 96)]
    plist, phis = [], []
    for n, method, seed in mix:
        kw = {"time_step": 1e-7} if method == "euler" else {}
        plist.append(_params(capi, n, method, prec, **kw))
        phis.append(shapes.seeded_ellipsoid(n, n, shapes.eps_rule(150, n), seed))
    b = capi.Batch(plist)
    for i, phi in enumerate(phis):
        b.set_phi(i, phi)
    r = b.run(12)
    assert r["steps"] == 12 * len(mix)
    for i, (p, phi) in enumerate(zip(plist, phis)):
        st = capi.Stepper(p)
        st.set_phi(phi)
        st.run(12)
        a, s = b.get_phi(i), st.get_phi()
        assert np.array_equal(a, s), (mix[i], np.abs(a - s).max())
        sa, ss = b.scalars(i), st.scalars()
        assert (sa["steps"], sa["rejects"], sa["dt"], sa["E"]) == (ss["steps"], ss["rejects"], ss["dt"], ss["E"])
        st.close()
    # a second run continues every instance from where it stopped
    b.run(3)
    assert all(b.scalars(i)["steps"] == 15 for i in range(len(mix)))
    b.close()


def _request(capi, n, seed, arrival, method="etd2", rel_tol=1e-5, max_steps=150):
    rng = np.random.default_rng(seed)
    rq = capi.cb_request()
    rq.params = _params(capi, n, method, 1, rel_tol=rel_tol)
    rq.axes[:] = [rng.uniform(1.2, 2.0), rng.uniform(1.2, 2.0), rng.uniform(0.5, 1.2)]
    rq.centre[:] = [0.0, 0.0, 0.0]
    rq.axes2[:] = [0.0, 0.0, 0.0]
    rq.arrival_s = arrival
    rq.max_steps = max_steps
    return rq


def test_server_results_same_alone_and_in_mix(cblib):
    from cudabubble_gb300 import capi
    sizes = [16, 32, 24, 48, 16, 32, 64, 24, 32, 16]
    reqs = [_request(capi, n, 100 + i, 0.02 * i) for i, n in enumerate(sizes)]
    one = capi.cb_instance_bytes if hasattr(capi, "cb_instance_bytes") else None
    b64 = cblib.cb_instance_bytes(reqs[6].params)
    # budget below the whole trace so admission has to queue
    budget = int(2.5 * b64)
    want = {i: (n, n, n) for i, n in enumerate(sizes)}
    res, stats, phis = capi.serve_trace(reqs, budget, max_slots_per_class=3, quantum=2, phi_out=want)
    assert stats["completed"] == len(sizes)
    assert stats["peak_bytes"] <= budget
    for i, r in enumerate(res):
        assert r["status"] in (1, 5), r  # max_steps (not converged) or converged
        assert r["finished_s"] >= r["admitted_s"] >= r["arrival_s"] - 1e-9
        alone, _, ph = capi.serve_trace([reqs[i]], budget, max_slots_per_class=3, quantum=2,
                                        phi_out={0: want[i]})
        assert (alone[0]["steps"], alone[0]["E"]) == (r["steps"], r["E"]), i
        assert np.array_equal(ph[0], phis[i]), i


def test_server_cancellation_frees_the_slot_and_budget(cblib):
    """A client cancels one running request and one queued request.  The budget holds
    one 32^3 instance at a time, so the requests behind the running one wait for its
    memory: it is retired with CB_DONE_CANCELLED after its class's current batch, its
    bytes go back, and the next request is admitted and finishes as it would alone."""
    from cudabubble_gb300 import capi
    r0 = _request(capi, 32, 200, 0.000)
    r1 = _request(capi, 32, 201, 0.001, rel_tol=0.0, max_steps=10 ** 7)  # runs until cancelled
    r1.cancel_ms = 200
    r2 = _request(capi, 32, 202, 0.002)
    r3 = _request(capi, 32, 203, 0.003)  # cancelled while it waits in the queue
    r3.cancel_ms = 50
    reqs = [r0, r1, r2, r3]
    budget = int(1.5 * cblib.cb_instance_bytes(r0.params))
    res, stats, _ = capi.serve_trace(reqs, budget, max_slots_per_class=4, quantum=2)
    assert stats["completed"] == 4
    assert stats["peak_bytes"] <= budget
    assert res[0]["status"] in (capi.CB_DONE_TARGET, capi.CB_DONE_CONVERGED)
    assert res[1]["status"] == capi.CB_DONE_CANCELLED
    assert res[1]["admitted_s"] > 0 and res[1]["steps"] > 0
    assert res[1]["finished_s"] >= 0.201 - 1e-3
    assert res[3]["status"] == capi.CB_DONE_CANCELLED
    assert res[3]["admitted_s"] == 0.0 and res[3]["steps"] == 0
    assert 0.053 - 1e-3 <= res[3]["finished_s"] < res[1]["finished_s"]
    # the request behind the cancelled one got its memory and ran to its own end
    assert res[2]["admitted_s"] >= res[1]["finished_s"] - 1e-3
    assert res[2]["status"] in (capi.CB_DONE_TARGET, capi.CB_DONE_CONVERGED)
    alone, _, _ = capi.serve_trace([r2], budget, max_slots_per_class=4, quantum=2)
    assert (alone[0]["steps"], alone[0]["E"]) == (res[2]["steps"], res[2]["E"])


def test_server_passes_over_a_full_class(cblib):
    """A full class does not hold up requests of other classes behind it."""
    from cudabubble_gb300 import capi
    big = [_request(capi, 48, 300 + i, 0.0, rel_tol=0.0, max_steps=400) for i in range(2)]
    small = _request(capi, 16, 310, 0.001, max_steps=50)
    res, stats, _ = capi.serve_trace(big + [small], 10 ** 10, max_slots_per_class=1, quantum=2)
    assert stats["completed"] == 3
    # the second 48^3 request waits for the first one's slot; the 16^3 one does not
    assert res[1]["admitted_s"] >= res[0]["finished_s"] - 1e-3
    assert res[2]["admitted_s"] < res[0]["finished_s"]
    assert res[2]["finished_s"] < res[1]["finished_s"]
