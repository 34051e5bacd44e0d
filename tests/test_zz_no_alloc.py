"""cb_intf_noalloc (partial sums in a fixed device array, no allocation) against
the stepper's own reductions, through the C ABI.  Collected last so it runs
both after the other GPU tests and, alone, in a fresh process."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _intf(lib, d_u, shape, addition, multiply, volume, d_val):
    nz, ny, nx = shape
    rc = lib.cb_intf_noalloc(C.c_void_p(d_u.data_ptr()), nx, ny, nz, addition, multiply, volume,
                             C.c_void_p(d_val.data_ptr()), None)
    assert rc == 0, lib.cb_last_error()


def test_intf_noalloc_matches_stepper(cblib):
    torch = pytest.importorskip("torch")
    from cudabubble_gb300 import capi, shapes
    n, nz = 64, 48
    eps = shapes.eps_rule(150, n)
    phi = shapes.seeded_ellipsoid(n, nz, eps, 3)
    st = capi.Stepper(capi.default_params(nx=n, ny=n, nz=nz, epssize=150, method=capi.CB_ETD2,
                                          precision=capi.CB_FP64, time_step=1e-6, fixed_time_step=1e-6))
    st.set_phi(phi)
    sc = st.scalars()
    s_field = st.field(capi.CB_FIELD_S)
    st.close()
    L3 = (2 * math.pi) ** 3
    d_phi = torch.from_numpy(phi).cuda()
    d_s = torch.from_numpy(np.ascontiguousarray(s_field)).cuda()
    d_val = torch.zeros(2, dtype=torch.float64, device="cuda")
    for _ in range(2):  # two calls in a row: the scratch counter must be back at zero
        d_val.zero_()
        _intf(cblib, d_phi, phi.shape, 1.0, 0.5, L3, d_val[0:1])
        _intf(cblib, d_s, s_field.shape, 0.0, 3.0 / (2.0 * math.sqrt(2.0)), L3, d_val[1:2])
        torch.cuda.synchronize()
        V, S = d_val.cpu().numpy()
        assert V == pytest.approx(sc["V"], rel=1e-12, abs=1e-12)
        assert S == pytest.approx(sc["S"], rel=1e-10)


def test_intf_noalloc_rejects_oversize(cblib):
    torch = pytest.importorskip("torch")
    d = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = cblib.cb_intf_noalloc(C.c_void_p(d.data_ptr()), 1, 1, 4097, 0.0, 1.0, 1.0, C.c_void_p(d.data_ptr()), None)
    assert rc != 0
    assert b"4096" in cblib.cb_last_error()
