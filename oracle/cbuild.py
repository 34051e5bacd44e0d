"""Builds oracle/lib/libcstep.so, the plain-C FP64 port of the reference step
(oracle/cstep.c) used as the timed CPU baseline.  TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cstep.c")
LIB = os.path.join(HERE, "lib", "libcstep.so")


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", SRC, "-o", LIB + ".tmp", "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("gcc failed:\n" + r.stdout)
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


class CStep:
    """ctypes face of oracle/cstep.c."""

    def __init__(self, nx: int, nz: int, eps: float, xlen: float = 2 * np.pi, eta: float = 1.0, ga: float = 1.0,
                 M1: float = 1e4, M2: float = 1e4, threads: int = 0):
        self.lib = C.CDLL(build())
        L = self.lib
        L.cs_create.restype = C.c_void_p
        L.cs_create.argtypes = [C.c_int, C.c_int] + [C.c_double] * 6
        for n in ("cs_destroy",):
            getattr(L, n).argtypes = [C.c_void_p]
        L.cs_set_phi.argtypes = [C.c_void_p, C.c_void_p]
        L.cs_get_phi.argtypes = [C.c_void_p, C.c_void_p]
        L.cs_scalars.argtypes = [C.c_void_p, C.c_void_p]
        L.cs_r2c.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.cs_c2r.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.cs_run.restype = C.c_int
        L.cs_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                             C.POINTER(C.c_int)]
        L.cs_threads.restype = C.c_int
        L.cs_set_threads.argtypes = [C.c_int]
        if threads:
            L.cs_set_threads(threads)
        self.threads = L.cs_threads()
        self.shape = (nz, nx, nx)
        self.h = L.cs_create(nx, nz, xlen, eps, eta, ga, M1, M2)
        if not self.h:
            raise ValueError(f"unsupported grid {nx}x{nx}x{nz}")

    def close(self):
        if self.h:
            self.lib.cs_destroy(self.h)
            self.h = None

    def set_phi(self, phi):
        a = np.ascontiguousarray(phi, np.float64)
        self.lib.cs_set_phi(self.h, a.ctypes.data_as(C.c_void_p))

    def get_phi(self):
        out = np.empty(self.shape, np.float64)
        self.lib.cs_get_phi(self.h, out.ctypes.data_as(C.c_void_p))
        return out

    def scalars(self) -> dict:
        out = np.zeros(9)
        self.lib.cs_scalars(self.h, out.ctypes.data_as(C.c_void_p))
        return dict(V=out[0], S=out[1], E_el=out[2], E=out[3], alpha=out[4], beta=out[5], dt=out[6],
                    steps=int(out[7]), rejects=int(out[8]))

    def r2c(self, u):
        nz, ny, nx = self.shape
        out = np.empty((nz, ny, nx // 2 + 1), np.complex128)
        a = np.ascontiguousarray(u, np.float64)
        self.lib.cs_r2c(self.h, a.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p))
        return out

    def c2r(self, s):
        out = np.empty(self.shape, np.float64)
        a = np.ascontiguousarray(s, np.complex128)
        self.lib.cs_c2r(self.h, a.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p))
        return out

    def run(self, method: str, nsteps: int, time_step: float, fixed: float, alpha: float = -1.0,
            beta: float = -1.0, textbook: bool = False) -> str:
        why = C.c_int(0)
        m = {"euler": 0, "etd2": 1, "etd4": 2}[method]
        self.lib.cs_run(self.h, m, nsteps, time_step, fixed, alpha, beta, int(textbook), C.byref(why))
        return ["max_steps", "dt_underflow", "small_energy", "blowup", "converged"][why.value]
