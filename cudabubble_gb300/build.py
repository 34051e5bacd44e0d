"""Builds libcbstep.so (the C-ABI stepper) in-tree for sm_103a with nvcc.

Translation units compile in parallel; objects go to ``_build/`` at the
repository root and the shared library to ``cudabubble_gb300/lib/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libcbstep.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["kernels_f32.cu", "kernels_f32_z.cu", "kernels_f64.cu", "kernels_f64_z.cu", "kernels_mega.cu", "stepper.cu",
           "pool.cu", "noalloc.cu"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


STAMP = os.path.join(LIBDIR, "build_defines.txt")


SCHEDULE = os.path.join(PKG, "schedule.txt")


def defines() -> list[str]:
    """Extra -D flags for the launch schedules (z tile, thread counts, plane FFT split):
    CB_NVCC_DEFINES when set, else the schedule the tuner (tune.py) chose, kept in
    schedule.txt; the library is rebuilt whenever they change."""
    env = os.environ.get("CB_NVCC_DEFINES")
    if env is None and os.path.exists(SCHEDULE):
        env = " ".join(l.split("#")[0] for l in open(SCHEDULE))
    return [d for d in (env or "").split() if d.startswith("-D")]


def _compile(src: str, build_dir: str = BUILD) -> str:
    obj = os.path.join(build_dir, os.path.splitext(os.path.basename(src))[0] + ".o")
    cmd = [nvcc(), "-std=c++17", *ARCH, "-lineinfo", "-O3", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
           *defines(), "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    old = open(STAMP).read() if os.path.exists(STAMP) else ""
    if old != " ".join(defines()):
        return True
    t = os.path.getmtime(LIB)
    for d in (CSRC, INCLUDE, PKG):
        for f in os.listdir(d):
            if not os.path.isfile(os.path.join(d, f)) or not f.endswith((".cu", ".cuh", ".h", "build.py",
                                                                            "schedule.txt")):
                continue
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return False


def build_to(lib: str, build_dir: str) -> str:
    """Compile every translation unit with the current defines into `build_dir` and link
    the shared library at `lib`."""
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, build_dir), SOURCES))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}")
    os.replace(tmp, lib)
    return lib


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    build_to(LIB, BUILD)
    with open(STAMP, "w") as f:
        f.write(" ".join(defines()))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
