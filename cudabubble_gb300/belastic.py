"""Python face of the stepper, shaped like the reference's ``belastic`` /
``phasefield`` classes (belastic.h:9-35, phasefield.h:11-37) so callers and
tests read like the reference's time loop.  Everything runs through the C ABI
of ``include/cbstep.h``; there is no Python or CPU compute path.
"""
from __future__ import annotations

import numpy as np

from . import capi
from .capi import (CB_ETD2, CB_ETD4, CB_EULER, CB_FIELD_DX, CB_FIELD_DY, CB_FIELD_DZ, CB_FIELD_F, CB_FIELD_FD,
                   CB_FIELD_G0, CB_FIELD_LAP, CB_FIELD_NLD, CB_FIELD_NLD_HAT, CB_FIELD_PHI, CB_FIELD_RHS, CB_FIELD_S,
                   CB_FP32, CB_FP64)


class Belastic:
    """One vesicle relaxation.  ``params`` is a :class:`capi.cb_params`, or
    build one from an ini first line with ``Belastic.from_ini``."""

    def __init__(self, params: capi.cb_params, phi0: np.ndarray):
        self.params = params
        self.st = capi.Stepper(params)
        self.st.set_phi(phi0)

    @classmethod
    def from_ini(cls, line: str, phi0: np.ndarray, **overrides):
        p = capi.params_from_ini(line)
        for k, v in overrides.items():
            setattr(p, k, v)
        return cls(p, phi0)

    def close(self):
        self.st.close()

    # ---- step bodies (belastic.cpp:491-552, :382)
    def ETD2RK(self):
        self.st.ETD2RK()

    def ETD4RK(self):
        self.st.ETD4RK()

    def euler_step(self):
        """``get_sum_fgqterm`` then ``time_diff_solve_phi(nld, -dt*ga)``."""
        self.st.euler_step()

    # ---- loops (belastic.cpp:286-470 / :554-786)
    def shape_adjust(self, max_steps: int = 0) -> dict:
        """Unconstrained pre-relaxation (belastic.cpp:174-284); both loops call it
        first when the run starts at t = 0 with a nonzero shape flag."""
        return self.st.shape_adjust(max_steps)

    def run_static(self, nsteps: int) -> dict:
        assert self.params.method == CB_EULER
        return self.st.run(nsteps)

    def run_static_fEIF(self, nsteps: int) -> dict:
        assert self.params.method in (CB_ETD2, CB_ETD4)
        return self.st.run(nsteps)

    # ---- scalars (phasefield.cpp:283-325, belastic.cpp:68-86)
    def scalars(self) -> dict:
        return self.st.scalars()

    def getstaticenergy(self) -> float:
        return self.st.scalars()["E"]

    def vol(self) -> float:
        return self.st.scalars()["V"]

    def surface(self) -> float:
        return self.st.scalars()["S"]

    def elastic_eng(self) -> float:
        return self.st.scalars()["E_el"]

    @property
    def time_step(self) -> float:
        return self.st.scalars()["dt"]

    @time_step.setter
    def time_step(self, dt: float):
        self.st.set_dt(dt)

    # ---- phasefield getters (phasefield.cpp:125-308)
    def d(self) -> np.ndarray:
        return self.st.get_phi()

    def fd(self) -> np.ndarray:
        return self.st.field(CB_FIELD_FD)

    def lap(self) -> np.ndarray:
        return self.st.field(CB_FIELD_LAP)

    def f(self) -> np.ndarray:
        return self.st.field(CB_FIELD_F)

    def g0(self) -> np.ndarray:
        return self.st.field(CB_FIELD_G0)

    def nld(self) -> np.ndarray:
        return self.st.field(CB_FIELD_NLD)

    def gradient(self):
        return tuple(self.st.field(w) for w in (CB_FIELD_DX, CB_FIELD_DY, CB_FIELD_DZ))

    def s(self) -> np.ndarray:
        return self.st.field(CB_FIELD_S)

    def get_nld_term(self) -> np.ndarray:
        """N-hat of the current state (belastic.cpp:473-489), ETD handles."""
        return self.st.field(CB_FIELD_NLD_HAT)

    def get_sum_fgqterm(self) -> np.ndarray:
        """Euler right-hand side (belastic.cpp:52-64), Euler handles."""
        return self.st.field(CB_FIELD_RHS)


__all__ = ["Belastic", "CB_EULER", "CB_ETD2", "CB_ETD4", "CB_FP32", "CB_FP64"]
