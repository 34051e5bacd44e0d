"""The persistent batched attempt (CB_BATCH_PERSISTENT) on the GPU, through the C ABI.

One kernel walks the work list of every instance's attempt.  Its z tiles and small
planes run on thread groups of the one-pass kernels' shapes, so against the per-class
graph of the default mode an instance's trajectory is the same bits, except on 64^2
planes, which it runs on 512-thread CTAs (256 in the graph): there the sums differ in
summation order only, the decisions are the same and the energies agree to round-off.
Within the persistent mode an instance's trajectory is bitwise the same alone and in any
mix.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIX = [(32, 3), (48, 4), (64, 5), (96, 6), (32, 7), (64, 8), (128, 9)]


def _params(capi, n, **kw):
    base = dict(nx=n, ny=n, nz=n, epssize=150, method=capi.CB_ETD2, precision=capi.CB_FP32, time_step=1e-6,
                fixed_time_step=0.0, M1=1e4, M2=1e4)
    base.update(kw)
    return capi.default_params(**base)


def _default_z_tile():
    """The library was built with the one-pass z tile the persistent kernel's groups use
    (16 columns on 256 threads: the default schedule)."""
    from cudabubble_gb300 import build
    d = dict(x[2:].split("=", 1) for x in build.defines() if "=" in x)
    return d.get("CB_Z_TX", "16") == "16" and d.get("CB_Z_NT", "256") == "256"


def _batch(capi, shapes, mix, persistent, steps):
    plist = [_params(capi, n) for n, _ in mix]
    phis = [shapes.seeded_ellipsoid(n, n, shapes.eps_rule(150, n), seed) for n, seed in mix]
    b = capi.Batch(plist, persistent=persistent)
    for i, phi in enumerate(phis):
        b.set_phi(i, phi)
    r = b.run(steps)
    return b, r


def test_persistent_matches_the_per_class_graph(cblib):
    from cudabubble_gb300 import capi, shapes
    g, rg = _batch(capi, shapes, MIX, False, 15)
    m, rm = _batch(capi, shapes, MIX, True, 15)
    assert rg["steps"] == rm["steps"] == 15 * len(MIX)
    assert rm["attempts"] == rg["attempts"]
    worst = {"E": 0.0, "V": 0.0, "S": 0.0, "phi": 0.0}
    same_shapes = _default_z_tile()
    for i, (n, _) in enumerate(MIX):
        sg, sm = g.scalars(i), m.scalars(i)
        assert (sm["steps"], sm["rejects"], sm["dt"]) == (sg["steps"], sg["rejects"], sg["dt"]), (n, sg, sm)
        if n != 64 and same_shapes:  # the same bodies on the same shapes: the same bits
            assert sm["E"] == sg["E"] and np.array_equal(m.get_phi(i), g.get_phi(i)), n
        for k in ("E", "V", "S"):
            worst[k] = max(worst[k], abs(sm[k] - sg[k]) / abs(sg[k]))
        worst["phi"] = max(worst["phi"], float(np.abs(m.get_phi(i) - g.get_phi(i)).max()))
    print("persistent vs per-class graph, worst relative E, V, S and max |d phi|:", worst)
    # summation order only: far inside the FP32 form's own error against FP64 (~1e-8 on E)
    assert worst["E"] < 1e-7 and worst["V"] < 1e-8 and worst["S"] < 1e-7, worst
    assert worst["phi"] < 1e-5, worst
    # a second run continues every instance from where it stopped
    m.run(3)
    assert all(m.scalars(i)["steps"] == 18 for i in range(len(MIX)))
    g.close()
    m.close()


@pytest.mark.parametrize("kw", [dict(fixed_time_step=2e-6, accurate_coefficients=1),
                                dict(fixed_time_step=2e-6, M1=0.0, M2=0.0)],
                         ids=["fixed-dt-corrected-accurate", "fixed-dt-no-penalty"])
def test_persistent_fixed_dt_loops(cblib, kw):
    """The fixed-dt loops (with the alpha/beta correction's redo of a step, and without
    penalties) through the persistent kernel against the per-class graph."""
    from cudabubble_gb300 import capi, shapes
    mix = [(32, 11), (64, 12), (48, 13)]
    out = []
    for persistent in (False, True):
        plist = [_params(capi, n, **kw) for n, _ in mix]
        b = capi.Batch(plist, persistent=persistent)
        for i, (n, seed) in enumerate(mix):
            b.set_phi(i, shapes.seeded_ellipsoid(n, n, shapes.eps_rule(150, n), seed))
        b.run(8)
        out.append([b.scalars(i) for i in range(len(mix))])
        b.close()
    for (n, _), sg, sm in zip(mix, *out):
        assert (sm["steps"], sm["rejects"], sm["attempts"], sm["dt"]) == (sg["steps"], sg["rejects"], sg["attempts"],
                                                                          sg["dt"]), n
        assert abs(sm["E"] - sg["E"]) <= 1e-7 * abs(sg["E"]), (n, sm["E"], sg["E"])


def test_persistent_same_alone_and_in_mix(cblib):
    """The 64^3 instance (seed 5) alone and among six others: the same bits."""
    from cudabubble_gb300 import capi, shapes
    a, _ = _batch(capi, shapes, [(64, 5)], True, 12)
    m, _ = _batch(capi, shapes, MIX, True, 12)
    assert np.array_equal(a.get_phi(0), m.get_phi(2))
    sa, sm = a.scalars(0), m.scalars(2)
    assert (sa["steps"], sa["rejects"], sa["dt"], sa["E"]) == (sm["steps"], sm["rejects"], sm["dt"], sm["E"])
    a.close()
    m.close()


@pytest.mark.parametrize("what", ["fp64", "etd4", "n192", "curvature", "split"])
def test_persistent_refuses_what_it_is_not_built_for(cblib, what):
    from cudabubble_gb300 import capi
    kw = {"fp64": dict(precision=capi.CB_FP64), "etd4": dict(method=capi.CB_ETD4), "n192": dict(nx=192, ny=192, nz=32),
          "curvature": dict(spont_c=0.5), "split": dict(xy_split=capi.XYP_SPLIT)}[what]
    p = _params(capi, 32, **kw)
    with pytest.raises(capi.CBError) as ei:
        capi.Batch([p, _params(capi, 32)] if what != "fp64" else [p], persistent=True)
    assert ei.value.code == capi.CB_EUNSUPPORTED
