"""Benchmark of the GB300 stepper on CudaBubble's headline workload.

Workload (one "step" = one accepted step of the hot path): a 128^3 periodic
grid, seeded ellipsoid phi0 (axes a, b ~ U[1.2, 2], c ~ U[0.5, 1.2], seed 2),
eps = 1.5 h, M1 = M2 = 1e4, ETD-RK2 with the reference's adaptive dt starting
at 1e-6 (halve on energy rise, double every 4 accepted steps, cap 1e-3),
FP32 FFTs / pointwise math with FP64 reductions.  The timed steps are steps
1..K from phi0 (warm-up runs first on the same workload, then phi0 is
reloaded).  Every attempt (accepted or rejected) is timed with CUDA events on
the stepper's stream and L2 is flushed (256 MiB memset) between attempts,
outside the timed events.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--no-cpu-baseline] [--no-extra] [--only batched|batched_persistent|served]

--impl reference times the reference algorithm's CPU form (oracle/cstep.c,
the plain FP64 C port with OpenMP on every host core) on the same workload.

Besides the headline line's keys, the JSON carries (unless --no-extra):
  plain_fp64  the plain FP64 form of this stepper on the same workload (the
              "vs plain FP64" of the metric), and the FP32 form's speed-up;
  batched     workload config 4: 64 vesicles of grids drawn from
              {32,48,64,96,128}^3 advanced together (cb_batch_*), a launch per
              pass and grid size in one CUDA graph per attempt;
  batched_persistent  the same workload through one persistent kernel per attempt
              (CB_BATCH_PERSISTENT);
  served      workload config 5: the first 0.2 s of a Poisson trace at 200 req/s
              of relaxations to |dE/E| < 1e-8 on grids {32..256}^3 through the
              continuous-batching server (cb_serve_trace), run to completion, with
              p50/p99 latency overall and per grid size;
  ref_cufft   the reference's own FP64 cuFFT build (oracle/_ref/refstep, built by
              build() from the staged sources) on the same workload and GPU;
and (unless --no-cpu-baseline) cpu_baseline: the C port on the host cores, OpenMP and
single-threaded.  The JSON line's `config` is the workload's identity and is the same
in the --impl reference line; run details are under `run`.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# 32 hardware work queues for the process's streams (read when the CUDA context is made):
# with the default 8, the served and batched workloads' per-class streams share queues
# with each other and with the streams earlier workloads made, and a small class's
# launches wait behind a large class's in the same queue
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

N_GRID = 128
EPSSIZE = 150
SEED = 2
DT0 = 1e-6
METRIC = "grid-pts·steps/s vs plain FP64 at rel-E≤1e-6; served p50/p99 latency"
UNIT = "grid-pt·steps/s"
FLUSH_BYTES = 256 << 20
WORKLOAD = ("C2: 128^3 periodic [-pi,pi]^3, seeded ellipsoid phi0 (seed 2), eps=1.5h, M1=M2=1e4, "
            "ETD-RK2, adaptive dt from 1e-6 (halve on energy rise, x2 every 4 steps, cap 1e-3), steps 1..K from phi0")


def workload_config() -> dict:
    """The workload's identity, the same in both arms' JSON lines (run details such as
    attempts or the xy path go to `run`)."""
    return {"workload": WORKLOAD, "grid": [N_GRID] * 3, "method": "ETD-RK2", "points": N_GRID ** 3,
            "l2": "GPU arm: flushed between attempts (256 MiB memset, outside timed events)"}


def phi0():
    from cudabubble_gb300 import shapes
    return shapes.seeded_ellipsoid(N_GRID, N_GRID, shapes.eps_rule(EPSSIZE, N_GRID), SEED)


def golden_energy(step: int):
    """The reference's own FP64 cuFFT energy at `step` for this workload, if recorded."""
    path = os.path.join(ROOT, "tests", "golden", "manifest.json")
    try:
        man = json.load(open(path))
        for s in man["cases"]["c2_etd2_128"]["steps"]:
            if s["step"] == step:
                return s["E"]
    except (OSError, KeyError, ValueError):
        pass
    return None


class Clocks:
    """Samples nvidia-smi every 200 ms while active."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference_run(nsteps: int, warmup: int, threads: int = 0):
    """The reference algorithm on the host cores (oracle/cstep.c, FP64, OpenMP)."""
    from oracle.cbuild import CStep
    from cudabubble_gb300 import shapes
    eps = shapes.eps_rule(EPSSIZE, N_GRID)
    p0 = phi0()
    cs = CStep(N_GRID, N_GRID, eps, threads=threads)
    if warmup:
        cs.set_phi(p0)
        cs.run("etd2", warmup, DT0, 0.0)
    cs.set_phi(p0)
    t0 = time.perf_counter()
    why = cs.run("etd2", nsteps, DT0, 0.0)
    dt = time.perf_counter() - t0
    sc = cs.scalars()
    cs.close()
    return dict(seconds=dt, steps=sc["steps"], why=why, threads=cs.threads, E=sc["E"])


def cpu_c1_run(nsteps: int, threads: int):
    """Config 1 on the host cores: 64^3, axes (1.6, 1.6, 0.8), eps = 2h, forward Euler at
    fixed dt 1e-7, M1 = M2 = 1e4 (oracle/cstep.c, FP64)."""
    from oracle.cbuild import CStep
    from cudabubble_gb300 import shapes
    n = 64
    eps = shapes.eps_rule(200, n)
    p0 = shapes.ellipsoid(n, n, eps, (1.6, 1.6, 0.8))
    cs = CStep(n, n, eps, threads=threads)
    cs.set_phi(p0)
    t0 = time.perf_counter()
    cs.run("euler", nsteps, 1e-7, 1e-7)
    dt = time.perf_counter() - t0
    sc = cs.scalars()
    cs.close()
    return dict(seconds=dt, steps=sc["steps"], threads=cs.threads)


def cpu_baseline():
    """Bounded samples on the host cores (oracle/cstep.c, the plain FP64 C port of the
    reference step).  The workload (config 2): steps 1..20 (the GPU arm's K) with OpenMP on
    every host thread, median of 5 runs, and steps 1..4 on one thread, median of 3.
    Config 1 (64^3 Euler): 100 steps with OpenMP, median of 5, and 20 steps on one thread,
    median of 3.  About 35 s of CPU work in all."""
    def median(fn, nsteps, runs, threads):
        rs = sorted((fn(nsteps, threads) for _ in range(runs)), key=lambda r: r["seconds"])
        return rs[len(rs) // 2]
    allt = os.cpu_count() or 0
    omp = median(lambda k, t: cpu_reference_run(k, 0, t), 20, 5, allt)
    one = median(lambda k, t: cpu_reference_run(k, 0, t), 4, 3, 1)
    c1 = median(cpu_c1_run, 100, 5, allt)
    c1s = median(cpu_c1_run, 20, 3, 1)
    v = N_GRID ** 3 * omp["steps"] / omp["seconds"]
    v1 = N_GRID ** 3 * one["steps"] / one["seconds"]
    return {"value": v, "unit": UNIT, "cores": omp["threads"], "kind": "port",
            "sample": f"steps 1..{omp['steps']} of the workload on the host (oracle/cstep.c, FP64, OpenMP on "
                      f"{omp['threads']} threads), median of 5 runs, {omp['seconds']:.2f} s each",
            "single_thread": {"value": v1, "unit": UNIT, "cores": 1,
                              "sample": f"steps 1..{one['steps']}, one thread, median of 3 runs, "
                                        f"{one['seconds']:.2f} s each"},
            "config1": {"value": 64 ** 3 * c1["steps"] / c1["seconds"], "unit": UNIT, "cores": c1["threads"],
                        "sample": f"config 1 (64^3, Euler, fixed dt 1e-7), {c1['steps']} steps, OpenMP on "
                                  f"{c1['threads']} threads, median of 5 runs, {c1['seconds']:.2f} s each",
                        "single_thread": {"value": 64 ** 3 * c1s["steps"] / c1s["seconds"], "unit": UNIT,
                                          "cores": 1,
                                          "sample": f"{c1s['steps']} steps, one thread, median of 3 runs, "
                                                    f"{c1s['seconds']:.2f} s each"}}}


def ref_cufft(steps: int):
    """The reference's own FP64 cuFFT stepper (the unmodified sources built by
    oracle/ref_harness/build_ref.sh, driven step by step by its harness) on the same
    workload and GPU: CUDA-event time per accepted step, summed over steps 1..K."""
    exe = os.path.join(ROOT, "oracle", "_ref", "refstep")
    if not os.path.exists(exe):
        return {"unavailable": "oracle/_ref/refstep not built (no staged reference sources)"}
    import tempfile
    d = tempfile.mkdtemp(prefix="cb_refcufft_")
    p0 = os.path.join(d, "phi0.bin")
    phi0().astype(np.float64).tofile(p0)
    out = os.path.join(d, "out")
    os.makedirs(out)
    args = [exe, "run", os.path.join(d, "w"), "etd2", str(N_GRID), str(N_GRID), str(EPSSIZE), repr(DT0), "0.0",
            "10000.0", "10000.0", str(steps), p0, out, "0"]
    t0 = time.perf_counter()
    r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    wall = time.perf_counter() - t0
    if r.returncode != 0:
        return {"unavailable": f"refstep exited {r.returncode}: {r.stdout[-200:]}"}
    recs = [json.loads(l) for l in open(os.path.join(out, "steps.jsonl")) if l.strip()]
    st = [x for x in recs if "step" in x and x["step"] > 0]
    ms = sum(x["ms"] for x in st)
    ref_E = golden_energy(st[-1]["step"]) if st else None
    return {"value": N_GRID ** 3 * len(st) / (ms / 1e3), "unit": UNIT, "steps": len(st),
            "ms_per_step": ms / max(len(st), 1), "rejects": st[-1]["rejects"] if st else None,
            "rel_E_vs_golden": abs(st[-1]["E"] - ref_E) / abs(ref_E) if ref_E else None, "wall_s": wall,
            "what": "reference FP64 cuFFT build (Calc.cu, belastic.cpp) via oracle/ref_harness, CUDA events "
                    "around each accepted step (its blocking scalar reads included), same GPU, steps 1..K"}


def algorithmic_bytes(n: int, fsize: int, att: int, rej: int):
    """Bytes each kernel kind must move over `att` attempts with `rej` retries
    (a retry skips the stage-1 nonlinear pass and reuses the stored N_u).
    F = one half-spectrum field of complex FP32 (8 B per mode); the stepped
    state fields (phi-hat, candidate, a-hat) are double-float pairs, 2F, and so
    is the real-space u (n^3 points of 8 B, counted as 2F)."""
    F = n * n * (n // 2 + 1) * 2 * fsize
    return {
        # per stage: read P0, P2, u_state (2F); write G'', w; the candidate also writes its u (2F)
        "xy_fused": att * (2 * 6 * F + 2 * F),
        # S2: read A, B, a-hat(2F), phi(2F), N_u; write phi'(2F), P0, P2 = 11F
        # S1 fresh: read G'', w, phi(2F); write N_u, a-hat(2F), P0, P2   = 9F
        # S1 retry: read N_u, phi(2F); write a-hat(2F), P0, P2           = 7F
        "z_stage": att * 11 * F + (att - rej) * 9 * F + rej * 7 * F,
    }, F


# launches of one ETD-RK2 attempt of the FP32 form: prologue + coefficient fill,
# z S1, xy FUSED (work), z S2, xy FUSED (candidate), decide
LAUNCHES_PER_ATTEMPT = 6

# served workload: the first 0.2 s of the config-5 trace (42 requests, every grid size)
SERVE_TRACE_S = 0.2
SERVE_MAX_STEPS = 60000


def plain_fp64(steps: int):
    """The plain FP64 form of this stepper on the headline workload (same
    timing and L2 flushing as the FP32 line)."""
    from cudabubble_gb300 import capi
    p = capi.default_params(nx=N_GRID, ny=N_GRID, nz=N_GRID, epssize=EPSSIZE, method=capi.CB_ETD2,
                            precision=capi.CB_FP64, time_step=DT0, fixed_time_step=0.0, M1=1e4, M2=1e4)
    st = capi.Stepper(p)
    st.set_phi(phi0())
    st.run(3)
    st.set_phi(phi0())
    r = st.run_timed(steps, FLUSH_BYTES)
    sc = st.scalars()
    st.close()
    ms = r["device_ms"]
    ref_E = golden_energy(sc["steps"])
    return {"value": N_GRID ** 3 * sc["steps"] / (ms / 1e3), "unit": UNIT, "steps": sc["steps"],
            "attempts": r["attempts"], "ms_per_step": ms / max(sc["steps"], 1),
            "rel_E_error_vs_reference": abs(sc["E"] - ref_E) / abs(ref_E) if ref_E else None,
            "what": "CB_FP64 (FP64 transforms, split y/x plane passes at 128^2), same workload, steps 1..K"}


# cb_params.xy_split codes
PATH_NAMES = ["auto", "split", "single", "cluster"]


def schedule_defines():
    """The build-time launch schedule the library was compiled with (z tile, thread counts,
    line splits): the schedule tuner's choice in cudabubble_gb300/schedule.txt, or
    CB_NVCC_DEFINES."""
    from cudabubble_gb300 import build
    return " ".join(build.defines()) or "defaults"


def batched(steps: int, tune: bool = False, persistent: bool = False):
    """Workload config 4 through cb_batch (FP32 form); with `tune`, the xy path of each
    size class is chosen by cb_autotune first, else by the size rule; `persistent`: one
    persistent kernel per attempt of every instance (CB_BATCH_PERSISTENT)."""
    from cudabubble_gb300 import capi, workloads
    plist, phis = workloads.batched()
    tuned = {}
    if tune:
        first = {}
        for p, ph in zip(plist, phis):
            first.setdefault((p.nx, p.nz, p.method, p.precision), ph)
        tuned = capi.tune_xy_paths(plist, lambda p: first[(p.nx, p.nz, p.method, p.precision)])
    b = capi.Batch(plist, persistent=persistent)
    for i, ph in enumerate(phis):
        b.set_phi(i, ph)
    b.run(3)
    for i, ph in enumerate(phis):
        b.set_phi(i, ph)
    r = b.run_timed(steps, FLUSH_BYTES)
    pts = sum(p.nx * p.ny * p.nz * b.scalars(i)["steps"] for i, p in enumerate(plist))
    b.close()
    return {"value": pts / (r["device_ms"] / 1e3), "unit": UNIT, "instances": len(plist),
            "grid_points": int(sum(p.nx * p.ny * p.nz for p in plist)), "steps_per_instance": steps,
            "xy_paths": {f"{k[0]}x{k[0]}x{k[1]}": PATH_NAMES[v] for k, v in tuned.items()} or "size rule",
            "schedule": schedule_defines(),
            "attempts": r["attempts"], "device_ms": r["device_ms"],
            "what": "config 4: 64 vesicles, grids U{32,48,64,96,128}^3 (seed 4), alpha x U[0.6,0.95], ETD-RK2 "
                    "per-instance adaptive dt, FP32 form; "
                    + ("one persistent kernel per attempt walking a work list of (instance, pass, tile) units"
                       if persistent else "one CUDA graph per attempt over all size classes, a launch per pass "
                       "and class") + "; "
                    + ("xy path per size class chosen by cb_autotune" if tune else "xy path by the size rule")}


def served(duration_s: float, max_steps: int, tune: bool = False):
    """Workload config 5 through cb_serve_trace (FP32 form, 150 GB budget): the first
    `duration_s` seconds of the seeded 200 req/s Poisson trace, replayed in real time and
    run until every request has finished; `tune` as in batched().  Each request relaxes
    to |dE/E| < 1e-8 (3,000 to 19,000 accepted steps on these grids), so the offered load
    is far above one GPU's capacity and the queue grows through the trace: latency is
    dominated by queueing, and throughput by the device."""
    from cudabubble_gb300 import capi, shapes, workloads
    reqs = workloads.served(duration_s=duration_s, max_steps=max_steps)
    tuned = {}
    if tune:
        tuned = capi.tune_xy_paths([r.params for r in reqs],
                                   lambda p: shapes.ellipsoid(p.nx, p.nz, shapes.eps_rule(p.epssize, p.nx),
                                                              (1.6, 1.6, 0.8)))
    res, stats, _ = capi.serve_trace(reqs, 150 * 10 ** 9, max_slots_per_class=64, quantum=4)
    lat = np.array([r["latency_s"] for r in res])
    conv = sum(1 for r in res if r["status"] == capi.CB_DONE_CONVERGED)
    per = {}
    for n in sorted({q.params.nx for q in reqs}):
        idx = [i for i, q in enumerate(reqs) if q.params.nx == n]
        ln = np.array([res[i]["latency_s"] for i in idx])
        per[f"{n}^3"] = {"requests": len(idx),
                         "converged": sum(1 for i in idx if res[i]["status"] == capi.CB_DONE_CONVERGED),
                         "p50_latency_s": round(float(np.percentile(ln, 50)), 3),
                         "p99_latency_s": round(float(np.percentile(ln, 99)), 3),
                         "mean_steps": round(float(np.mean([res[i]["steps"] for i in idx])), 1),
                         "mean_service_s": round(float(np.mean([res[i]["finished_s"] - res[i]["admitted_s"]
                                                                for i in idx])), 3)}
    offered = sum(q.params.nx ** 3 for q in reqs) * float(np.mean([r["steps"] for r in res])) / duration_s
    return {"requests": len(reqs), "completed": stats["completed"], "converged": conv,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "per_grid": per,
            "value": stats["point_steps"] / stats["wall_s"], "unit": UNIT, "wall_s": stats["wall_s"],
            "offered_point_steps_per_s": offered, "peak_bytes": stats["peak_bytes"],
            "xy_paths": {f"{k[0]}x{k[0]}x{k[1]}": PATH_NAMES[v] for k, v in tuned.items()} or "size rule",
            "schedule": schedule_defines(),
            "what": f"config 5: the first {duration_s:g} s of a Poisson 200 req/s trace (seed 5), grids "
                    f"{{32..256}}^3 weighted 30/25/20/15/7/3 %, ETD-RK2 to |dE/E|<1e-8 (max {max_steps} steps), "
                    "150 GB budget, continuous batching (per-class streams, arenas carved up front), FP32 form; "
                    "latency = finish - arrival"}


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The largest x over the ranks (the slowest replica's time); x itself on one rank."""
    if world <= 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(points: int, steps: int, seconds: float, world: int) -> float:
    """Whole-job grid-point*steps/s: each of the `world` ranks advances its own replica
    of the workload (no exchange between replicas), timed by the slowest."""
    return world * points * steps / seconds


def xy_path_config(tune) -> dict:
    """The xy path of the headline handle: the autotuner's choice and timings, or the size
    rule (the two-CTA cluster pass at 128^2 planes)."""
    if tune is None:
        return {"xy_path": "size rule (cluster)"}
    return {"xy_path": PATH_NAMES[tune["path"]],
            "xy_path_ms_per_attempt": {PATH_NAMES[k]: round(v, 4) for k, v in tune["timed"].items()}}


def run_ours(args, rank: int, world: int):
    import torch
    from cudabubble_gb300 import capi

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    p0 = phi0()
    N = N_GRID ** 3
    params = capi.default_params(nx=N_GRID, ny=N_GRID, nz=N_GRID, epssize=EPSSIZE, method=capi.CB_ETD2,
                                 precision=capi.CB_FP32, time_step=DT0, fixed_time_step=0.0, M1=1e4, M2=1e4)
    st = capi.Stepper(params)
    # warm-up on the same workload (and, with --tune, the xy path picked by the autotuner),
    # then phi0 again
    st.set_phi(p0)
    st.run(args.warmup)
    tune = st.autotune(10) if args.tune else None
    st.set_phi(p0)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        t0 = time.perf_counter()
        r = st.run_timed(args.steps, FLUSH_BYTES)
        wall = time.perf_counter() - t0
    torch.cuda.synchronize()
    sc = st.scalars()
    ms = r["device_ms"]
    ms = max_over_ranks(ms, world)
    steps = sc["steps"]
    attempts = r["attempts"]
    rejects = sc["rejects"]
    value = job_throughput(N, steps, ms / 1e3, world)
    ref_E = golden_energy(steps)
    rel_E = abs(sc["E"] - ref_E) / abs(ref_E) if ref_E else None

    # per-kernel device time (kernel by kernel, L2 flushed between attempts)
    st.set_phi(p0)
    st.run(min(args.steps, 40))  # profile in the steady state after the dt ramp
    s0 = st.scalars()
    prof_att = 16
    prof = st.profile_kernels(prof_att, FLUSH_BYTES)
    s1 = st.scalars()
    prej = s1["rejects"] - s0["rejects"]
    ab, F = algorithmic_bytes(N_GRID, 4, prof_att, prej)
    kern = {}
    for k, (kms, cnt) in prof.items():
        if k in ab and kms > 0:
            kern[k] = {"ms_total": kms, "launches": cnt, "algorithmic_bytes": ab[k],
                       "achieved_gbs": ab[k] / (kms / 1e3) / 1e9}
    total_ms = sum(v[0] for v in prof.values())
    dom = max(kern, key=lambda k: kern[k]["ms_total"])
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tr_path):
        traffic = json.load(open(tr_path)).get(dom)
    d = kern[dom]
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(d["achieved_gbs"], 1), "peak": hbm_peak,
                "unit": "GB/s", "frac": round(d["achieved_gbs"] / hbm_peak, 4), "traffic": traffic,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6800",
                "bytes_per_launch": d["algorithmic_bytes"] / d["launches"],
                "share_of_step_time": round(d["ms_total"] / total_ms, 3),
                "per_kernel": {k: {"avg_us": round(1e3 * v["ms_total"] / v["launches"], 2),
                                   "achieved_gbs": round(v["achieved_gbs"], 1),
                                   "share": round(v["ms_total"] / total_ms, 3)} for k, v in kern.items()}}

    # end to end through the C ABI with host buffers in pinned memory:
    # set_phi(host) + run(K) + get_phi(host)
    pin_in = torch.from_numpy(p0).pin_memory()
    pin_out = torch.empty(p0.shape, dtype=torch.float64).pin_memory()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    # the median of three passes, each from phi0 (the first pass also pays one-time costs of
    # the pinned pages)
    walls, parts = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        st.set_phi(pin_in.numpy())
        t1 = time.perf_counter()
        rr = st.run(args.steps)
        t2 = time.perf_counter()
        out = st.get_phi(out=pin_out.numpy())
        t3 = time.perf_counter()
        sc2 = st.scalars()
        t4 = time.perf_counter()
        walls.append(t4 - t0)
        parts.append((t4 - t0, {"set_phi": t1 - t0, "run": t2 - t1, "get_phi": t3 - t2, "scalars": t4 - t3}))
    e2e_s = max_over_ranks(sorted(walls)[1], world)
    # each call returns after its own stream sync, so the host clock splits the median pass
    split = sorted(parts, key=lambda x: x[0])[1][1]
    e2e_steps = sc2["steps"]
    e2e = {"value": job_throughput(N, e2e_steps, e2e_s, world), "unit": UNIT,
           "h2d_bytes_per_step": int(p0.nbytes / max(e2e_steps, 1)),
           "d2h_bytes_per_step": int((out.nbytes + 120) / max(e2e_steps, 1)),
           "what": "cb_set_phi(pinned host phi0) + cb_run(K) + cb_get_phi(pinned host) + cb_scalars_get, wall clock, "
                   "median of 3 passes",
           "split_ms": {k: round(v * 1e3, 4) for k, v in split.items()}}
    st.close()

    res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": args.warmup,
           "ms_per_step": ms / max(steps, 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 (FFT + pointwise), f64 reductions / scalars / energy test", "data": "synthetic",
           "config": workload_config(),
           "run": {"attempts": attempts, "rejects": rejects,
                   "parallelism": "replicas" if world > 1 else "single GPU", **xy_path_config(tune)},
           "accuracy": {"E_step_K": sc["E"], "E_reference_fp64_cufft": ref_E, "rel_E_error": rel_E},
           "e2e": e2e, "gpu_launches": attempts * LAUNCHES_PER_ATTEMPT, "roofline": roofline,
           "wall_s_timed_region": wall}
    clk_sum = clk.summary()
    res["clocks"] = clk_sum
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--only", choices=["batched", "batched_persistent", "served"], default=None,
                    help="run one extra workload alone and print its JSON (for profiling it)")
    ap.add_argument("--tune", action="store_true", help="choose xy paths with cb_autotune (default: size rule)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        if rank != 0:
            return
        cores = os.cpu_count() or 1
        steps = max(1, min(args.steps, 20))
        r = cpu_reference_run(steps, max(0, min(args.warmup, 3)))
        v = N_GRID ** 3 * r["steps"] / r["seconds"]
        res = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": r["steps"],
               "warmup": args.warmup, "ms_per_step": 1e3 * r["seconds"] / r["steps"], "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": workload_config(),
               "run": {"attempts": None, "note": "steps capped at 20 per run to bound CPU time",
                       "parallelism": f"OpenMP, {r['threads']} host threads"},
               "cpu_baseline": {"value": v, "unit": UNIT, "cores": r["threads"], "kind": "port",
                                "sample": f"steps 1..{r['steps']} of the workload (oracle/cstep.c, FP64, OpenMP on "
                                          f"{r['threads']} of {cores} host threads)"},
               "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(res))
        return

    if args.only:  # one extra workload alone, e.g. under a profiler
        if rank == 0:
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            if args.only == "served":
                r = served(SERVE_TRACE_S, SERVE_MAX_STEPS, args.tune)
            else:
                r = batched(min(args.steps, 60), args.tune, persistent=args.only == "batched_persistent")
            print(json.dumps({"only": args.only, args.only: r}))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res = run_ours(args, rank, world)
    if rank == 0 and not args.no_extra:
        pf = plain_fp64(args.steps)
        res["plain_fp64"] = pf
        res["speedup_fp32_over_plain_fp64"] = res["value"] / pf["value"]
        res["batched"] = batched(min(args.steps, 60), args.tune)
        try:
            res["batched_persistent"] = batched(min(args.steps, 60), False, persistent=True)
        except Exception as e:  # reported, not fatal: the default mode above is the batched figure
            res["batched_persistent"] = {"error": str(e)}
        res["served"] = served(SERVE_TRACE_S, SERVE_MAX_STEPS, args.tune)
        res["ref_cufft"] = ref_cufft(args.steps)
        if "value" in res["ref_cufft"]:
            res["speedup_fp32_over_ref_cufft"] = res["value"] / res["ref_cufft"]["value"]
    if rank == 0:
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = cpu_baseline()
        print(json.dumps(res))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
