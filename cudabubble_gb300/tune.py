"""Schedule tuner: picks the stepper's build-time launch schedules by timing them.

The schedules are compile-time constants of the kernels, so each candidate is a separate
build of the library, timed in a process of its own:

- the z pass tile: columns and threads per CTA (CB_Z_TX, CB_Z_NT);
- the split of the 128- and 96-point line transforms into two register phases
  (16 x 8 or 8 x 16; 16 x 6 or 12 x 8);
- the FP32 form's fused plane pass: two-CTA clusters or one CTA per plane.

A coordinate search starts from the default schedule and, knob by knob, keeps the
candidate with the lowest weighted device time per attempt of the FP32 ETD-RK2 loop on
the given grid sizes (seeded ellipsoids, the L2 flushed between attempts).  Candidates
whose energies leave the default's by more than 1e-5 are refused, and a knob moves off
its current option only for a gain of at least --min-gain (1 %: run-to-run spread, and
a line split changes the FP32 rounding).  With --write the
winner goes to cudabubble_gb300/schedule.txt, which build.py compiles with from then
on (CB_NVCC_DEFINES overrides it).

    python -m cudabubble_gb300.tune [--sizes 128] [--weights 1] [--steps 120] [--write]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys

from . import build as B

KNOBS = [
    ("z pass tile (columns x threads)", [("-DCB_Z_TX=16", "-DCB_Z_NT=256"), ("-DCB_Z_TX=8", "-DCB_Z_NT=128"),
                                         ("-DCB_Z_TX=32", "-DCB_Z_NT=512")]),
    ("128-point line split", [(), ("-DCB_PLAN128_8X16",)]),
    ("96-point line split", [(), ("-DCB_PLAN96_12X8",)]),
    ("FP32 fused plane pass", [(), ("-DCB_XY_CLUSTER=0",)]),
]


def _child(sizes, steps):
    """Time the FP32 ETD-RK2 loop on each size with the library CB_LIB names."""
    from . import capi, shapes
    out = {}
    for n in sizes:
        p = capi.default_params(nx=n, ny=n, nz=n, epssize=150, method=capi.CB_ETD2, precision=capi.CB_FP32,
                                time_step=1e-6, fixed_time_step=0.0, M1=1e4, M2=1e4)
        st = capi.Stepper(p)
        phi = shapes.seeded_ellipsoid(n, n, shapes.eps_rule(150, n), 2)
        st.set_phi(phi)
        st.run(10)
        st.set_phi(phi)
        r = st.run_timed(steps, 256 << 20)
        s = st.scalars()
        out[str(n)] = {"ms_per_attempt": r["device_ms"] / max(r["attempts"], 1), "E": s["E"],
                       "steps": s["steps"], "rejects": s["rejects"]}
        st.close()
    print(json.dumps(out))


def _measure(defs, sizes, steps):
    tag = hashlib.sha1(" ".join(defs).encode()).hexdigest()[:10]
    base = os.path.join(B.ROOT, "_build", "tune", tag)
    lib = os.path.join(base, "libcbstep.so")
    env = dict(os.environ, CB_NVCC_DEFINES=" ".join(defs))
    if not os.path.exists(lib):
        r = subprocess.run([sys.executable, "-c", "import sys; from cudabubble_gb300 import build as B; "
                            f"B.build_to({lib!r}, {os.path.join(base, 'obj')!r})"],
                           cwd=B.ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build of {defs} failed:\n{r.stdout[-2000:]}")
    env["CB_LIB"] = lib
    r = subprocess.run([sys.executable, "-m", "cudabubble_gb300.tune", "--child", "--sizes",
                        ",".join(map(str, sizes)), "--steps", str(steps)],
                       cwd=B.ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"timing of {defs} failed:\n{r.stdout[-2000:]}")
    return json.loads(r.stdout.strip().splitlines()[-1])


def tune(sizes, weights, steps, write=False, log=print, min_gain=0.01):
    choice = [opts[0] for _, opts in KNOBS]
    flat = lambda ch: [d for opt in ch for d in opt]
    cache = {}

    def cost(ch):
        key = tuple(flat(ch))
        if key not in cache:
            res = _measure(list(key), sizes, steps)
            cache[key] = (sum(w * res[str(n)]["ms_per_attempt"] for n, w in zip(sizes, weights)), res)
        return cache[key]

    ref_cost, ref = cost(choice)
    table = [(" ".join(flat(choice)) or "(defaults)", ref_cost)]
    log(f"default schedule: {ref_cost:.4f} ms per weighted attempt")
    for i, (name, opts) in enumerate(KNOBS):
        best = choice[i]
        best_cost = cost(choice)[0]
        for opt in opts:
            if opt == choice[i]:
                continue
            trial = list(choice)
            trial[i] = opt
            c, res = cost(trial)
            drift = max(abs(res[str(n)]["E"] - ref[str(n)]["E"]) / abs(ref[str(n)]["E"]) for n in sizes)
            table.append((" ".join(flat(trial)) or "(defaults)", c))
            log(f"  {name}: {' '.join(opt) or 'default'} -> {c:.4f} ms (energy drift {drift:.1e})")
            if drift <= 1e-5 and c < best_cost and c < cost(choice)[0] * (1.0 - min_gain):
                best, best_cost = opt, c
        choice[i] = best
        log(f"{name}: keep {' '.join(best) or 'default'}")
    final = flat(choice)
    if write:
        with open(B.SCHEDULE, "w") as f:
            f.write("# launch schedules chosen by cudabubble_gb300/tune.py (FP32 ETD-RK2 loop, sizes "
                    f"{sizes}, weights {weights}); build.py compiles with these defines\n")
            for d in final:
                f.write(d + "\n")
            f.write("# ms per weighted attempt of each schedule timed:\n")
            for k, c in sorted(table, key=lambda t: t[1]):
                f.write(f"#   {c:.4f}  {k}\n")
    return final, table


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="128")
    ap.add_argument("--weights", default="")
    ap.add_argument("--steps", type=int, default=120)
    ap.add_argument("--write", action="store_true")
    ap.add_argument("--min-gain", type=float, default=0.01)
    ap.add_argument("--child", action="store_true")
    a = ap.parse_args()
    sizes = [int(x) for x in a.sizes.split(",")]
    if a.child:
        _child(sizes, a.steps)
        return
    weights = [float(x) for x in a.weights.split(",")] if a.weights else [1.0] * len(sizes)
    final, table = tune(sizes, weights, a.steps, a.write, min_gain=a.min_gain)
    print(json.dumps({"schedule": final, "timed": [{"defines": k, "ms": c} for k, c in table]}))


if __name__ == "__main__":
    main()
