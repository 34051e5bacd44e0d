"""ctypes binding of ``include/cbstep.h`` (libcbstep.so).

The library is loaded from the package's ``lib/`` directory; importing this
module never falls back to anything else: if the shared library is missing
or does not export the declared symbols, the import fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# CB_LIB names another build of the library (the schedule tuner times candidate builds
# in child processes this way)
LIB_PATH = os.environ.get("CB_LIB") or os.path.join(_HERE, "lib", "libcbstep.so")

CB_OK, CB_EINVAL, CB_ENOMEM, CB_ECUDA, CB_ENONFINITE, CB_ENOTCONVERGED, CB_ETIMEOUT, CB_EDTUNDERFLOW, \
    CB_EUNSUPPORTED = 0, -1, -2, -3, -4, -5, -6, -7, -8
CB_EULER, CB_ETD2, CB_ETD4 = 0, 1, 2
CB_FP64, CB_FP32 = 0, 1
(CB_FIELD_PHI, CB_FIELD_FD, CB_FIELD_LAP, CB_FIELD_F, CB_FIELD_G0, CB_FIELD_NLD, CB_FIELD_DX, CB_FIELD_DY,
 CB_FIELD_DZ, CB_FIELD_S, CB_FIELD_NLD_HAT, CB_FIELD_RHS) = range(12)
XYP_AUTO, XYP_SPLIT, XYP_SINGLE, XYP_CLUSTER = range(4)
(CB_RUNNING, CB_DONE_TARGET, CB_DONE_DT_UNDERFLOW, CB_DONE_SMALL_ENERGY, CB_DONE_NONFINITE, CB_DONE_CONVERGED,
 CB_DONE_TMAX, CB_DONE_CANCELLED) = range(8)
STATUS_NAMES = {0: "running", 1: "target", 2: "dt_underflow", 3: "small_energy", 4: "nonfinite", 5: "converged",
                6: "tmax"}
ERROR_NAMES = {CB_EINVAL: "CB_EINVAL", CB_ENOMEM: "CB_ENOMEM", CB_ECUDA: "CB_ECUDA", CB_ENONFINITE: "CB_ENONFINITE",
               CB_ENOTCONVERGED: "CB_ENOTCONVERGED", CB_ETIMEOUT: "CB_ETIMEOUT",
               CB_EDTUNDERFLOW: "CB_EDTUNDERFLOW", CB_EUNSUPPORTED: "CB_EUNSUPPORTED"}


class cb_params(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("lenx", C.c_double), ("epssize", C.c_int),
                ("eps", C.c_double), ("eta", C.c_double), ("ga", C.c_double), ("alpha", C.c_double),
                ("beta", C.c_double), ("M1", C.c_double), ("M2", C.c_double), ("time_step", C.c_double),
                ("fixed_time_step", C.c_double), ("tmax", C.c_double), ("method", C.c_int),
                ("precision", C.c_int), ("grow_every", C.c_int), ("grow_factor", C.c_double),
                ("dt_cap", C.c_double), ("cap_probe", C.c_double), ("etd4_textbook", C.c_int),
                ("accurate_coefficients", C.c_int), ("rel_tol", C.c_double), ("xy_split", C.c_int),
                ("pad0", C.c_int), ("reject_tol", C.c_double), ("spont_c", C.c_double)]


class cb_scalars(C.Structure):
    _fields_ = [("V", C.c_double), ("S", C.c_double), ("E_el", C.c_double), ("E", C.c_double),
                ("lamb1", C.c_double), ("lamb2", C.c_double), ("alpha", C.c_double), ("beta", C.c_double),
                ("dt", C.c_double), ("t", C.c_double), ("lserror", C.c_double), ("steps", C.c_int),
                ("attempts", C.c_int), ("rejects", C.c_int), ("status", C.c_int), ("E_attempt", C.c_double)]


class cb_run_stats(C.Structure):
    _fields_ = [("steps", C.c_int), ("attempts", C.c_int), ("status", C.c_int), ("graph_launches", C.c_int),
                ("device_ms", C.c_double)]


class cb_adjust_stats(C.Structure):
    _fields_ = [("steps", C.c_int), ("attempts", C.c_int), ("status", C.c_int), ("graph_launches", C.c_int),
                ("t", C.c_double), ("E_start", C.c_double), ("E_end", C.c_double), ("device_ms", C.c_double)]


class cb_tune_result(C.Structure):
    _fields_ = [("path", C.c_int), ("npaths", C.c_int), ("paths", C.c_int * 3), ("ms_per_attempt", C.c_double * 3)]


class cb_request(C.Structure):
    _fields_ = [("params", cb_params), ("axes", C.c_double * 3), ("centre", C.c_double * 3),
                ("axes2", C.c_double * 3), ("centre2", C.c_double * 3), ("arrival_s", C.c_double),
                ("max_steps", C.c_int), ("cancel_ms", C.c_int)]


class cb_result(C.Structure):
    _fields_ = [("arrival_s", C.c_double), ("admitted_s", C.c_double), ("finished_s", C.c_double),
                ("latency_s", C.c_double), ("E", C.c_double), ("V", C.c_double), ("S", C.c_double),
                ("steps", C.c_int), ("attempts", C.c_int), ("status", C.c_int), ("pad", C.c_int),
                ("bytes", C.c_longlong)]


class cb_serve_stats(C.Structure):
    _fields_ = [("wall_s", C.c_double), ("point_steps", C.c_double), ("completed", C.c_int),
                ("graph_launches", C.c_int), ("peak_bytes", C.c_longlong)]


# every symbol include/cbstep.h declares, with its ctypes signature
_P = C.POINTER
SIGNATURES = {
    "cb_params_default": (None, [_P(cb_params)]),
    "cb_params_from_ini_line": (C.c_int, [C.c_char_p, _P(cb_params)]),
    "cb_params_eps": (C.c_double, [_P(cb_params)]),
    "cb_instance_bytes": (C.c_longlong, [_P(cb_params)]),
    "cb_supported": (C.c_int, [_P(cb_params)]),
    "cb_create": (C.c_int, [_P(cb_params), _P(C.c_void_p)]),
    "cb_destroy": (C.c_int, [C.c_void_p]),
    "cb_set_phi": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "cb_get_phi": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "cb_scalars_get": (C.c_int, [C.c_void_p, _P(cb_scalars)]),
    "cb_getstaticenergy": (C.c_double, [C.c_void_p]),
    "cb_ETD2RK": (C.c_int, [C.c_void_p]),
    "cb_ETD4RK": (C.c_int, [C.c_void_p]),
    "cb_euler_step": (C.c_int, [C.c_void_p]),
    "cb_run": (C.c_int, [C.c_void_p, C.c_int, _P(cb_run_stats)]),
    "cb_field": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "cb_set_dt": (C.c_int, [C.c_void_p, C.c_double]),
    "cb_set_loop_state": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double]),
    "cb_shape_adjust": (C.c_int, [C.c_void_p, C.c_int, _P(cb_adjust_stats)]),
    "cb_autotune": (C.c_int, [C.c_void_p, C.c_int, _P(cb_tune_result)]),
    "cb_synchronize": (C.c_int, [C.c_void_p]),
    "cb_set_launch_limit": (C.c_int, [C.c_void_p, C.c_longlong]),
    "cb_handle_bytes": (C.c_longlong, [C.c_void_p]),
    "cb_run_timed": (C.c_int, [C.c_void_p, C.c_int, C.c_longlong, _P(C.c_double), _P(C.c_int)]),
    "cb_profile_kernels": (C.c_int, [C.c_void_p, C.c_int, C.c_longlong, _P(C.c_double), _P(C.c_int)]),
    "cb_batch_create": (C.c_int, [_P(cb_params), C.c_int, _P(C.c_void_p)]),
    "cb_batch_create_ex": (C.c_int, [_P(cb_params), C.c_int, C.c_int, _P(C.c_void_p)]),
    "cb_batch_destroy": (C.c_int, [C.c_void_p]),
    "cb_batch_set_phi": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "cb_batch_get_phi": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "cb_batch_scalars": (C.c_int, [C.c_void_p, C.c_int, _P(cb_scalars)]),
    "cb_batch_run": (C.c_int, [C.c_void_p, C.c_int, _P(cb_run_stats)]),
    "cb_batch_run_timed": (C.c_int, [C.c_void_p, C.c_int, C.c_longlong, _P(C.c_double), _P(cb_run_stats)]),
    "cb_serve_trace": (C.c_int, [_P(cb_request), C.c_int, C.c_longlong, C.c_int, C.c_int, _P(cb_result),
                                 _P(C.c_void_p), _P(cb_serve_stats)]),
    "cb_intf_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                  C.c_void_p, C.c_void_p]),
    "cb_last_error": (C.c_char_p, []),
    "cb_version": (C.c_char_p, []),
}


class CBError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path: str = LIB_PATH) -> C.CDLL:
    if not os.path.exists(path):
        raise ImportError(f"libcbstep.so not built at {path}; run cudabubble_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError when a declared symbol is missing
        fn.restype = res
        fn.argtypes = args
    return lib


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = load()
    return _lib


def check(rc: int):
    if rc != CB_OK:
        raise CBError(rc, lib().cb_last_error().decode())
    return rc


def default_params(**kw) -> cb_params:
    p = cb_params()
    lib().cb_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def params_from_ini(line: str) -> cb_params:
    p = cb_params()
    check(lib().cb_params_from_ini_line(line.encode(), C.byref(p)))
    return p


def tune_xy_paths(params_list, phi_for, attempts: int = 6) -> dict:
    """Autotune the xy path once per (grid, method, precision) class of `params_list`
    and write the choice into each member's ``xy_split`` (members set to 0 only).
    ``phi_for(p)`` gives a representative initial field for a class; each class is
    timed on a temporary stepper (``cb_autotune``).  Returns {class key: path}."""
    chosen = {}
    for p in params_list:
        key = (p.nx, p.nz, p.method, p.precision)
        if p.xy_split != XYP_AUTO:
            continue
        if key not in chosen:
            st = Stepper(p)
            try:
                st.set_phi(phi_for(p))
                chosen[key] = st.autotune(attempts)["path"]
            finally:
                st.close()
        p.xy_split = chosen[key]
    return chosen


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Stepper:
    """One stepper instance (``cb_handle``)."""

    def __init__(self, params: cb_params):
        self.params = params
        h = C.c_void_p()
        check(lib().cb_create(C.byref(params), C.byref(h)))
        self.h = h
        self.shape = (params.nz, params.nx, params.nx)
        self.cshape = (params.nz, params.nx, params.nx // 2 + 1)

    def close(self):
        if self.h:
            lib().cb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_phi(self, phi: np.ndarray):
        a = np.ascontiguousarray(phi, dtype=np.float64)
        assert a.shape == self.shape, (a.shape, self.shape)
        check(lib().cb_set_phi(self.h, _dptr(a), 0))

    def get_phi(self, out: np.ndarray | None = None) -> np.ndarray:
        """phi in the .out layout; into `out` (C-contiguous float64, e.g. a pinned buffer)
        when given."""
        if out is None:
            out = np.empty(self.shape, np.float64)
        assert out.shape == self.shape and out.dtype == np.float64 and out.flags["C_CONTIGUOUS"]
        check(lib().cb_get_phi(self.h, _dptr(out), 0))
        return out

    def scalars(self) -> dict:
        s = cb_scalars()
        check(lib().cb_scalars_get(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in cb_scalars._fields_}

    def field(self, which: int) -> np.ndarray:
        if which in (CB_FIELD_FD, CB_FIELD_NLD_HAT):
            out = np.empty(self.cshape, np.complex128)
        else:
            out = np.empty(self.shape, np.float64)
        check(lib().cb_field(self.h, which, _dptr(out), 0))
        return out

    def ETD2RK(self):
        check(lib().cb_ETD2RK(self.h))

    def ETD4RK(self):
        check(lib().cb_ETD4RK(self.h))

    def euler_step(self):
        check(lib().cb_euler_step(self.h))

    def set_dt(self, dt: float):
        check(lib().cb_set_dt(self.h, dt))

    def set_loop_state(self, t: float, dt: float, alpha: float, beta: float):
        """Resume a run: accepted time, dt and volume / area targets (after set_phi)."""
        check(lib().cb_set_loop_state(self.h, t, dt, alpha, beta))

    def autotune(self, attempts: int = 20) -> dict:
        """Time each xy path this handle can run and keep the fastest."""
        r = cb_tune_result()
        check(lib().cb_autotune(self.h, attempts, C.byref(r)))
        return {"path": r.path, "timed": {r.paths[i]: r.ms_per_attempt[i] for i in range(r.npaths)}}

    def shape_adjust(self, max_steps: int = 0) -> dict:
        """belastic::shape_adjust (belastic.cpp:174-284) on the current state."""
        st = cb_adjust_stats()
        check(lib().cb_shape_adjust(self.h, max_steps, C.byref(st)))
        return {k: getattr(st, k) for k, _ in cb_adjust_stats._fields_}

    def run_timed(self, nsteps: int, flush_bytes: int = 0) -> dict:
        ms = C.c_double(0.0)
        att = C.c_int(0)
        rc = lib().cb_run_timed(self.h, nsteps, flush_bytes, C.byref(ms), C.byref(att))
        if rc not in (CB_OK, CB_ENONFINITE, CB_EDTUNDERFLOW):
            check(rc)
        return {"device_ms": ms.value, "attempts": att.value, "rc": rc}

    KERNEL_KINDS = ("xy_nonlin", "xy_reduce_s", "xy_reduce_full", "z_stage", "decide_coef", "xy_fused")

    def profile_kernels(self, nattempts: int, flush_bytes: int = 0) -> dict:
        ms = (C.c_double * len(self.KERNEL_KINDS))()
        cnt = (C.c_int * len(self.KERNEL_KINDS))()
        check(lib().cb_profile_kernels(self.h, nattempts, flush_bytes, ms, cnt))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(self.KERNEL_KINDS)}

    def set_launch_limit(self, n: int):
        """Bound the attempts one run / run_timed / shape_adjust call may launch (0: none);
        a call that reaches it raises CB_ETIMEOUT and leaves the state at its last accepted step."""
        check(lib().cb_set_launch_limit(self.h, C.c_longlong(n)))

    def nbytes(self) -> int:
        return int(lib().cb_handle_bytes(self.h))

    def run(self, nsteps: int) -> dict:
        st = cb_run_stats()
        rc = lib().cb_run(self.h, nsteps, C.byref(st))
        res = {k: getattr(st, k) for k, _ in cb_run_stats._fields_}
        res["rc"] = rc
        if rc not in (CB_OK, CB_ENONFINITE, CB_EDTUNDERFLOW):
            check(rc)
        return res


CB_BATCH_PERSISTENT = 1


class Batch:
    """Many vesicles of uneven grids advanced together (``cb_batch``).
    ``persistent``: one persistent kernel per attempt of every instance
    (``CB_BATCH_PERSISTENT``) instead of a launch per pass and grid size."""

    def __init__(self, params_list, persistent: bool = False):
        arr = (cb_params * len(params_list))(*params_list)
        h = C.c_void_p()
        flags = CB_BATCH_PERSISTENT if persistent else 0
        check(lib().cb_batch_create_ex(arr, len(params_list), flags, C.byref(h)))
        self.h = h
        self.shapes = [(p.nz, p.nx, p.nx) for p in params_list]

    def close(self):
        if self.h:
            lib().cb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self.shapes)

    def set_phi(self, i: int, phi: np.ndarray):
        a = np.ascontiguousarray(phi, dtype=np.float64)
        assert a.shape == self.shapes[i]
        check(lib().cb_batch_set_phi(self.h, i, _dptr(a), 0))

    def get_phi(self, i: int) -> np.ndarray:
        out = np.empty(self.shapes[i], np.float64)
        check(lib().cb_batch_get_phi(self.h, i, _dptr(out), 0))
        return out

    def scalars(self, i: int) -> dict:
        s = cb_scalars()
        check(lib().cb_batch_scalars(self.h, i, C.byref(s)))
        return {k: getattr(s, k) for k, _ in cb_scalars._fields_}

    def run(self, nsteps: int) -> dict:
        st = cb_run_stats()
        check(lib().cb_batch_run(self.h, nsteps, C.byref(st)))
        return {k: getattr(st, k) for k, _ in cb_run_stats._fields_}

    def run_timed(self, nsteps: int, flush_bytes: int) -> dict:
        st = cb_run_stats()
        ms = C.c_double(0)
        check(lib().cb_batch_run_timed(self.h, nsteps, flush_bytes, C.byref(ms), C.byref(st)))
        r = {k: getattr(st, k) for k, _ in cb_run_stats._fields_}
        r["device_ms"] = ms.value
        return r


def serve_trace(requests, hbm_budget_bytes: int, max_slots_per_class: int = 64, quantum: int = 4,
                phi_out: dict | None = None):
    """Replay an arrival trace through the continuous-batching server.
    ``requests``: list of :class:`cb_request`; ``phi_out``: {index: shape} of
    requests whose final phi to return.  Returns (results, stats, phis)."""
    n = len(requests)
    reqs = (cb_request * n)(*requests)
    res = (cb_result * n)()
    st = cb_serve_stats()
    phis = {}
    ptrs = None
    if phi_out:
        ptrs = (C.c_void_p * n)()
        for i, shape in phi_out.items():
            phis[i] = np.empty(shape, np.float64)
            ptrs[i] = phis[i].ctypes.data
    check(lib().cb_serve_trace(reqs, n, hbm_budget_bytes, max_slots_per_class, quantum, res, ptrs, C.byref(st)))
    results = [{k: getattr(r, k) for k, _ in cb_result._fields_} for r in res]
    stats = {k: getattr(st, k) for k, _ in cb_serve_stats._fields_}
    return results, stats, phis
