"""A reference-compatible time-loop driver on the GB300 stepper.

  python -m cudabubble_gb300.driver [index] [--results DIR] [--output-seconds S]
                                    [--max-steps K]

It follows the reference's executable (``main.cpp``, ``belastic`` constructor
and ``belastic::run_static_fEIF``, ``belastic.cpp:554-786``):

* reads the first line of ``<results>/ini<index>.dat`` (the 34-field
  contract, ``fluidbase.cpp:33-35``; a 35th and 36th field may select the
  method and the precision), works in ``<results>/<ifold>/`` and copies the
  ini file there;
* starts from ``d<nx>x<ny>x<nz>.out`` when ninit is 7 and otherwise from the
  workload ellipsoid (a = b = 1.6, c = 0.8), standing in for the reference's
  hard-coded shapes, which are outside this stepper's scope;
* resumes from ``<nx>x<ny>x<nz>.info`` (time, dt, alpha, beta) when present,
  and otherwise runs the shape adjustment first when the ini's shape flag
  (field 8) is nonzero (``belastic.cpp:558-560``);
* writes the reference's outputs at the start, every ``--output-seconds`` of
  wall time (20 s as ``belastic.cpp:759``) and at exit: the ``vol_sur``,
  ``lamb``, ``error``, ``time_step``, ``alpha_beta`` and ``energy`` logs,
  the ``d`` field (``.out`` plus text slices), the ``.info`` file, and the
  messages of ``output<nx>x<ny>x<nz>.txt``;
* stops on the loop's exits (dt below 1e-23, energy below 1e-3, blow-up),
  when ``ini<index>.dat`` names another folder (the reference's
  ``check_folder``, tested every 16 steps), or after ``--max-steps`` (not in
  the reference).
"""
from __future__ import annotations

import argparse
import math
import os
import shutil
import sys
import time

import numpy as np

from . import capi, checkpoint, shapes


class Run:
    def __init__(self, results: str, index: int, output_seconds: float = 20.0):
        self.results = results
        self.index = index
        self.output_seconds = output_seconds
        self.ini = os.path.join(results, f"ini{index}.dat")
        with open(self.ini) as f:
            self.line = f.readline()
        fields = self.line.split()
        self.ifold = int(fields[0])
        self.ninit = int(fields[11]) if len(fields) > 11 else 0
        self.b_shape = int(fields[7]) if len(fields) > 7 else 0
        self.params = capi.params_from_ini(self.line)
        p = self.params
        self.shape = (p.nz, p.ny, p.nx)
        self.folder = os.path.join(results, str(self.ifold)) + os.sep
        os.makedirs(self.folder, exist_ok=True)
        self.say(self.folder)
        self.say("\n")
        shutil.copyfile(self.ini, os.path.join(self.folder, f"ini{index}.dat"))
        self.alpha3 = 0.0

    # ---- fluidbase::output(const char*) (fluidbase.cpp:204-222)
    def say(self, s: str) -> None:
        with open(os.path.join(self.folder, f"output{checkpoint.tag(self.shape)}.txt"), "a") as f:
            f.write(s)
        sys.stdout.write(s)
        sys.stdout.flush()

    def check_folder(self) -> bool:
        """fluidbase.cpp:2885-2903: stop when the ini file names another folder."""
        try:
            with open(self.ini) as f:
                ifold = int(f.readline().split()[0])
        except (OSError, ValueError, IndexError):
            return False
        if ifold != self.ifold:
            self.say("User terminate!\n")
            return True
        return False

    def initial_phi(self) -> np.ndarray:
        p = self.params
        if self.ninit == 7:
            phi = checkpoint.read_out(self.folder, "d", self.shape, 0.0)
            if phi is None:
                self.say(f"Can not load file {checkpoint.out_path(self.folder, 'd', self.shape, 0.0)}! set as zeros\n")
                phi = np.zeros(self.shape)
            self.say("Loading initial shape from file; ")
            return phi
        eps = capi.lib().cb_params_eps(capi.C.byref(p))
        return shapes.ellipsoid(p.nx, p.nz, eps, (1.6, 1.6, 0.8))

    def lserror(self, st, sc) -> float:
        """belastic::geterror (belastic.cpp:136-143): LSerror of the Euler
        right-hand side lambda1/2 + lambda2 f + eta g0 at the current state."""
        p = self.params
        f = st.field(capi.CB_FIELD_F)
        g0 = st.field(capi.CB_FIELD_G0)
        rhs = 0.5 * sc["lamb1"] + sc["lamb2"] * f + p.eta * g0
        L3 = (2.0 * math.pi * p.lenx) ** 3
        return float(np.mean(rhs * rhs)) * L3

    def outputall(self, st) -> None:
        """belastic::outputall (belastic.cpp:147-171) and outputenergy (:88-113)."""
        p = self.params
        sc = st.scalars()
        t = sc["t"]
        v, s = sc["V"], sc["S"]
        err = self.lserror(st, sc)
        eng1 = p.eta * sc["E_el"]
        eng4 = 0.5 * p.M1 * (v - sc["alpha"]) ** 2
        eng5 = 0.5 * p.M2 * (s - sc["beta"]) ** 2
        eng = eng1 + eng4 + eng5
        ck = checkpoint
        ck.append_log(self.folder, "energy", self.shape, t, eng1, eng4, eng5, eng)
        ck.append_log(self.folder, "vol_sur", self.shape, t, v, s)
        ck.append_log(self.folder, "lamb", self.shape, t, sc["lamb1"], sc["lamb2"])
        ck.append_log(self.folder, "error", self.shape, t, err)
        ck.append_log(self.folder, "time_step", self.shape, t, sc["dt"])
        ck.append_log(self.folder, "alpha_beta", self.shape, t, sc["alpha"], sc["beta"])
        ck.write_info(self.folder, self.shape, {"time_current": t, "time_step": sc["dt"], "alpha": sc["alpha"],
                                                "beta": sc["beta"], "alpha3": self.alpha3})
        d = st.get_phi()
        ck.write_out(self.folder, "d", d, t)
        ck.write_slices(self.folder, "d", d, t)
        self.say(f"current time is {t:12.8f}\n")
        self.say(f"vol: {v:12.7f} surf: {s:12.7f} eng: {eng:12.10f} Error: {err:12.10f} "
                 f"Time_step: {sc['dt']:e}\n")

    def shape_adjust(self, st) -> None:
        """belastic::shape_adjust's messages (belastic.cpp:197-283) around the
        device loop; the energies of its intermediate checks are not reported."""
        self.say("Start Shape Adjusting......\n")
        r = st.shape_adjust()
        self.say(f"Start energy is {r['E_start']:12.8f}\n")
        self.say(f"energy is {r['E_end']:12.8f}\n")
        if r["status"] == capi.CB_DONE_DT_UNDERFLOW:
            self.say("time_step in shape adjust < 1e-13, get exit.\n")
        self.say("Shape Adjust Ended successfully\n")

    def run(self, max_steps: int = 0) -> int:
        p = self.params
        info = checkpoint.read_info(self.folder, self.shape)
        if info is None:
            self.say("Starting a new experiment.... start time is 0.\n")
        else:
            self.say("Continue the existing experiment....")
            self.say(f"Set start time to be {info['time_current']:12.8f}.\n")
            self.alpha3 = info["alpha3"]
        st = capi.Stepper(p)
        st.set_phi(self.initial_phi())
        if info is None and self.b_shape != 0:  # belastic.cpp:558-560 (a new run only)
            self.shape_adjust(st)
        if info is not None:
            alpha, beta = info["alpha"], info["beta"]
            if beta <= 0.0:  # belastic.cpp:588-591: targets from the state
                sc = st.scalars()
                alpha, beta = sc["V"], sc["S"]
            st.set_loop_state(info["time_current"], info["time_step"], alpha, beta)
        sc = st.scalars()
        dt = sc["dt"]
        self.say(f"grid(xyz): {p.nx}x{p.ny}x{p.nz}, timestep = {dt:e}\n")
        if p.fixed_time_step > 0:
            self.say(f"FIXED timestep = {dt:e}    ")
        else:
            self.say("Adjustment time_steps; ")
        eps = capi.lib().cb_params_eps(capi.C.byref(p))
        self.say(f"eps = {eps:9.6f}, ga = {p.ga:9.6f}, eta = {p.eta:9.6f}, tmax = {p.tmax:9.6f}\n")
        self.say(f"alpha = {sc['alpha']:9.6f}, beta = {sc['beta']:9.6f}, M1 = {p.M1:8.2f}, M2 = {p.M2:8.2f}\n")
        self.say("********* Start STATIC Running ***********\n")
        if info is None:
            self.say(f"Preserving volume and surface. (Initial volume = {sc['alpha']:12.8f}, "
                     f"surface = {sc['beta']:12.8f}\n")
            self.outputall(st)
        last = time.monotonic()
        steps = 0
        status = capi.CB_RUNNING
        while True:
            chunk = 16 if not max_steps else min(16, max_steps - steps)
            if chunk <= 0:
                break
            r = st.run(chunk)
            steps += r["steps"]
            status = r["status"]
            if status == capi.CB_DONE_DT_UNDERFLOW:
                self.say("time_step < 1e-23, get exit.\n")
                self.outputall(st)
                break
            if status == capi.CB_DONE_SMALL_ENERGY:
                self.say("Energy is too small < 1e-3, get exit.\n")
                self.outputall(st)
                break
            if status == capi.CB_DONE_NONFINITE:
                sc = st.scalars()
                self.say(f"Static Director Blow up! Blow up at time {sc['t']:12.8f}, {steps} steps\n")
                break
            if status == capi.CB_DONE_TMAX:
                self.say("Too long time running, get exit.\n")
                self.outputall(st)
                break
            if time.monotonic() - last >= self.output_seconds:
                self.outputall(st)
                last = time.monotonic()
            if self.check_folder():
                break
        if status in (capi.CB_DONE_TARGET, capi.CB_RUNNING) and max_steps:
            self.outputall(st)
        self.say("********* End Running ***********\n\n\n")
        st.close()
        return steps


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("index", nargs="?", type=int, default=0)
    ap.add_argument("--results", default="./results/")
    ap.add_argument("--output-seconds", type=float, default=20.0)
    ap.add_argument("--max-steps", type=int, default=0)
    a = ap.parse_args(argv)
    print("Elastic bending energy program!")
    Run(a.results, max(a.index, 0), a.output_seconds).run(a.max_steps)
    return 1  # main.cpp returns 1


if __name__ == "__main__":
    sys.exit(0 if main() else 1)
