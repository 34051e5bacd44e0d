"""Generates the golden vectors that pin the oracle to the reference.

The reference (mrazizadeh/CudaBubble) ships no tests, fixtures or golden data,
so its own FP64 cuFFT path is run, step by step, through
``oracle/ref_harness`` (built by ``oracle/ref_harness/build_ref.sh``) on a GPU
host, from seeded initial fields made here.  Two sub-commands:

  python tests/golden/make_golden.py run  --out <rawdir>   # on a GPU host
  python tests/golden/make_golden.py pack --raw <rawdir>   # anywhere

``pack`` writes the small ``tests/golden/*.npz`` / ``*.json`` fixtures the
tests read.  Seeds: configs 1..5 of the workload table use seeds 1..5.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle.oracle import ellipsoid_phi0, eps_from_epssize  # noqa: E402

REFSTEP = os.path.join(ROOT, "oracle", "_ref", "refstep")
TWO_PI = 2.0 * math.pi


def seeded_axes(rng):
    """Axes a, b ~ U[1.2, 2.0], c ~ U[0.5, 1.2] (workload configs 2, 4, 5)."""
    return (float(rng.uniform(1.2, 2.0)), float(rng.uniform(1.2, 2.0)), float(rng.uniform(0.5, 1.2)))


def phi0_for(case: dict) -> np.ndarray:
    nx, nz, es = case["nx"], case["nz"], case["epssize"]
    eps = eps_from_epssize(es, TWO_PI, nx)
    shape = case.get("shape", "fixed")
    if shape == "fixed":
        return ellipsoid_phi0(nx, nz, eps, (1.6, 1.6, 0.8))
    if shape == "wide":  # a profile wider than the equilibrium tanh: its energy starts high
        return ellipsoid_phi0(nx, nz, eps * case["width"], (1.6, 1.6, 0.8))
    rng = np.random.default_rng(case["seed"])
    ax = seeded_axes(rng)
    if shape == "seeded":
        return ellipsoid_phi0(nx, nz, eps, ax)
    # two overlapping ellipsoids, centres in [-0.8, 0.8]^3 (config 3)
    c1 = tuple(float(v) for v in rng.uniform(-0.8, 0.8, 3))
    ax2 = seeded_axes(rng)
    c2 = tuple(float(v) for v in rng.uniform(-0.8, 0.8, 3))
    return ellipsoid_phi0(nx, nz, eps, ax, centre=c1, second=(ax2, c2))


# fields: every derived quantity of one state + one step of each method
FIELD_CASES = [
    dict(name="f16", nx=16, nz=16, epssize=200, dt=1e-6, shape="fixed"),
    dict(name="f24", nx=24, nz=24, epssize=150, dt=2e-6, shape="seeded", seed=11),
    dict(name="f32x16", nx=32, nz=16, epssize=150, dt=1e-6, shape="seeded", seed=12),
]
# trajectories through the restated loops (snap_every 0 = scalars only)
RUN_CASES = [
    dict(name="euler32", method="euler", nx=32, nz=32, epssize=200, time_step=1e-7, fixed=1e-7,
         M=1e4, nsteps=100, snap=50, shape="fixed"),
    dict(name="euler32_adapt", method="euler", nx=32, nz=32, epssize=200, time_step=1e-7, fixed=0.0,
         M=1e4, nsteps=60, snap=60, shape="fixed"),
    dict(name="etd2_32", method="etd2", nx=32, nz=32, epssize=150, time_step=1e-6, fixed=0.0,
         M=1e4, nsteps=100, snap=50, shape="seeded", seed=2),
    dict(name="etd4_32", method="etd4", nx=32, nz=32, epssize=150, time_step=1e-6, fixed=1e-6,
         M=1e4, nsteps=20, snap=20, shape="seeded", seed=3),
    dict(name="etd4_32_adapt", method="etd4", nx=32, nz=32, epssize=150, time_step=1e-6, fixed=0.0,
         M=1e4, nsteps=40, snap=40, shape="seeded", seed=3),
    dict(name="etd2_48", method="etd2", nx=48, nz=48, epssize=150, time_step=1e-6, fixed=0.0,
         M=1e4, nsteps=60, snap=60, shape="seeded", seed=2),
    # workload config 1: 64^3 forward Euler, dt 1e-7, 1000 steps
    dict(name="c1_euler64", method="euler", nx=64, nz=64, epssize=200, time_step=1e-7, fixed=1e-7,
         M=1e4, nsteps=1000, snap=1000, shape="fixed"),
    # workload config 2 (FP64 reference form): 128^3 ETD-RK2 adaptive from 1e-6, 1000 steps
    dict(name="c2_etd2_128", method="etd2", nx=128, nz=128, epssize=150, time_step=1e-6, fixed=0.0,
         M=1e4, nsteps=1000, snap=0, shape="seeded", seed=2),
    # workload config 3: 256^3 ETD-RK4 fixed dt 5e-6 with the alpha/beta correction
    dict(name="c3_etd4_256", method="etd4", nx=256, nz=256, epssize=150, time_step=5e-6, fixed=5e-6,
         M=1e4, nsteps=20, snap=0, shape="two", seed=3),
]

# the unconstrained pre-relaxation belastic::shape_adjust (belastic.cpp:174-284), run
# once by the reference itself; the wide profiles start above its 100 eta exit energy
ADJUST_CASES = [
    dict(name="adjust32", nx=32, nz=32, epssize=200, shape="wide", width=2.0),
    dict(name="adjust48", nx=48, nz=48, epssize=150, shape="wide", width=3.0),
]


def cmd_run(out: str, only: list[str] | None):
    os.makedirs(out, exist_ok=True)
    # the reference writes its ini, phi0 copy and logs into a work tree; keep
    # that (and large phi0 files) out of the result directory
    work = os.path.join(tempfile.mkdtemp(prefix="cbref_"), "w")
    for case in FIELD_CASES + RUN_CASES + ADJUST_CASES:
        if only and case["name"] not in only:
            continue
        d = os.path.join(out, case["name"])
        os.makedirs(d, exist_ok=True)
        phi = phi0_for(case)
        small = case["nx"] <= 64
        p0 = os.path.join(d if small else os.path.dirname(work), case["name"] + "_phi0.bin")
        phi.astype(np.float64).tofile(p0)
        if case in FIELD_CASES:
            args = [REFSTEP, "fields", work + "_" + case["name"], str(case["nx"]), str(case["nz"]),
                    str(case["epssize"]), repr(case["dt"]), p0, d]
        elif case in ADJUST_CASES:
            args = [REFSTEP, "adjust", work + "_" + case["name"], str(case["nx"]), str(case["nz"]),
                    str(case["epssize"]), p0, d]
        else:
            args = [REFSTEP, "run", work + "_" + case["name"], case["method"], str(case["nx"]),
                    str(case["nz"]), str(case["epssize"]), repr(case["time_step"]), repr(case["fixed"]),
                    repr(case["M"]), repr(case["M"]), str(case["nsteps"]), p0, d, str(case["snap"])]
        t0 = time.time()
        r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        with open(os.path.join(d, "log.txt"), "w") as f:
            f.write(r.stdout)
        print(f"{case['name']}: rc={r.returncode} {time.time() - t0:.1f}s", flush=True)
        if r.returncode != 0:
            raise SystemExit(f"refstep failed on {case['name']}")


def _read(path, dtype, shape):
    return np.fromfile(path, dtype=dtype).reshape(shape)


def cmd_pack(raw: str, dest: str):
    manifest = {"generator": "tests/golden/make_golden.py", "reference": "mrazizadeh/CudaBubble (FP64 cuFFT build)",
                "cases": {}}
    old = os.path.join(dest, "manifest.json")
    if os.path.exists(old):  # a partial run (--only) updates its own cases and keeps the rest
        with open(old) as f:
            manifest["cases"] = json.load(f).get("cases", {})
    for case in FIELD_CASES:
        d = os.path.join(raw, case["name"])
        if not os.path.isdir(d):
            continue
        nx, nz = case["nx"], case["nz"]
        shp, shc = (nz, nx, nx), (nz, nx, nx // 2 + 1)
        arrs = {"phi0": _read(os.path.join(d, case["name"] + "_phi0.bin"), np.float64, shp)}
        for k in ["lap", "f", "g0", "nld", "dx", "dy", "dz", "s", "rhs_euler", "euler1", "etd2_1", "etd4_1"]:
            arrs[k] = _read(os.path.join(d, k + ".bin"), np.float64, shp)
        for k in ["fd", "nld_hat"]:
            arrs[k] = _read(os.path.join(d, k + ".bin"), np.complex128, shc)
        arrs["Het"] = _read(os.path.join(d, "Het.bin"), np.float64, shc)
        np.savez_compressed(os.path.join(dest, case["name"] + ".npz"), **arrs)
        with open(os.path.join(d, "scalars.json")) as f:
            sc = json.load(f)
        manifest["cases"][case["name"]] = dict(case, scalars=sc)
    for case in RUN_CASES:
        d = os.path.join(raw, case["name"])
        if not os.path.isdir(d):
            continue
        nx, nz = case["nx"], case["nz"]
        lines = [json.loads(s) for s in open(os.path.join(d, "steps.jsonl"))]
        steps = [l for l in lines if "step" in l]
        end = [l for l in lines if "end" in l][0]
        entry = dict(case, end=end, steps=steps)
        snaps = {}
        if case["snap"] > 0 and nx <= 64:
            for fn in sorted(os.listdir(d)):
                if fn.startswith("phi_") and fn.endswith(".bin"):
                    snaps[fn[:-4]] = _read(os.path.join(d, fn), np.float64, (nz, nx, nx))
        if snaps:
            np.savez_compressed(os.path.join(dest, case["name"] + ".npz"), **snaps)
            entry["snapshots"] = sorted(snaps)
        manifest["cases"][case["name"]] = entry
    for case in ADJUST_CASES:
        d = os.path.join(raw, case["name"])
        if not os.path.isdir(d):
            continue
        nx, nz = case["nx"], case["nz"]
        phi = _read(os.path.join(d, "phi_adjust.bin"), np.float64, (nz, nx, nx))
        np.savez_compressed(os.path.join(dest, case["name"] + ".npz"), phi_adjust=phi)
        with open(os.path.join(d, "scalars.json")) as f:
            sc = json.load(f)
        # the reference's own messages: "energy is %12.8f" at each convergence check
        checks = [float(l.split()[-1]) for l in open(os.path.join(d, "log.txt")) if l.startswith("energy is")]
        manifest["cases"][case["name"]] = dict(case, scalars=sc, checks=checks)
    with open(os.path.join(dest, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("packed", sorted(manifest["cases"]))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run")
    r.add_argument("--out", required=True)
    r.add_argument("--only", nargs="*")
    pk = sub.add_parser("pack")
    pk.add_argument("--raw", required=True)
    pk.add_argument("--dest", default=HERE)
    a = ap.parse_args()
    if a.cmd == "run":
        cmd_run(a.out, a.only)
    else:
        cmd_pack(a.raw, a.dest)
