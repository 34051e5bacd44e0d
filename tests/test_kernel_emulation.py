"""Index safety of the stepper's kernels on the CPU.

The kernel headers of cudabubble_gb300/csrc are compiled for the host against a
CUDA emulation (tests/emu/fake: one OS thread per CUDA thread, real barriers for
__syncthreads, warp shuffles and cluster barriers) with AddressSanitizer, and one
FP32-form attempt (set-up pass, prologue and coefficient fill, the method's z stages
with their fused xy passes, decide) runs: ETD-RK2 on both xy schedules, ETD-RK4 and
Euler on the one-CTA schedule.  Every device buffer
and every block's shared memory is an exact-size heap allocation, so any access
outside them fails the test.  The two schedules must also leave the same sums.
Needs g++ with AddressSanitizer; no GPU."""
import importlib.util
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.emulation

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cudabubble_gb300", "csrc")
EMU = os.path.join(ROOT, "tests", "emu")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("emu")
    src = d / "src"
    spec = importlib.util.spec_from_file_location("emu_rewrite", os.path.join(EMU, "rewrite.py"))
    rw = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(rw)
    # every kernel's shared-memory declaration becomes the emulated block's buffer
    assert rw.copy_sources(CSRC, str(src)) >= 4
    exe = d / "attempt"
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address", "-fno-omit-frame-pointer", "-ffp-contract=off",
           "-I", os.path.join(EMU, "fake"), "-I", str(src), "-I", os.path.join(ROOT, "include"),
           os.path.join(EMU, "attempt.cpp"), "-o", str(exe), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr and "cannot find" in r.stderr:
        pytest.skip("AddressSanitizer runtime not available")
    assert r.returncode == 0, r.stderr[-4000:]
    return str(exe)


@pytest.fixture(scope="module")
def mega_harness(tmp_path_factory):
    """tests/emu/mega_attempt.cpp: one attempt of a three-instance pool through the
    persistent batched kernel against the one-pass kernels of the same shapes."""
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("emu_mega")
    src = d / "src"
    spec = importlib.util.spec_from_file_location("emu_rewrite", os.path.join(EMU, "rewrite.py"))
    rw = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(rw)
    rw.copy_sources(CSRC, str(src))
    exe = d / "mega_attempt"
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address", "-fno-omit-frame-pointer", "-ffp-contract=off",
           "-I", os.path.join(EMU, "fake"), "-I", str(src), "-I", os.path.join(ROOT, "include"),
           os.path.join(EMU, "mega_attempt.cpp"), "-o", str(exe), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr and "cannot find" in r.stderr:
        pytest.skip("AddressSanitizer runtime not available")
    assert r.returncode == 0, r.stderr[-4000:]
    return str(exe)


def test_persistent_kernel_same_as_one_pass_kernels(mega_harness):
    """Work list, unit hand-over between the CTAs of a cluster, dependency counters and the
    decision by the CTA that ends an instance's last phase: every buffer and control field
    of the three instances bitwise as the one-pass kernels leave them, all phase counters
    complete, no wait run out, every index in bounds."""
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:halt_on_error=1")
    r = subprocess.run([mega_harness], capture_output=True, text=True, env=env, timeout=3000)
    assert "AddressSanitizer" not in r.stderr, r.stderr[-6000:]
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert r.stdout.strip().endswith("SAME"), r.stdout[-3000:]


METHODS = {"euler": 0, "etd2": 1, "etd4": 2}


def run_attempt(exe, n, nz, path, method="etd2"):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:halt_on_error=1")
    r = subprocess.run([exe, str(n), str(nz), str(path), str(METHODS[method])], capture_output=True, text=True,
                       env=env, timeout=900)
    assert "AddressSanitizer" not in r.stderr, r.stderr[-6000:]
    assert r.returncode == 0, r.stderr[-3000:]
    vals = {}
    for line in r.stdout.splitlines():
        head, *rest = line.split()
        for k, v in zip(rest[0::2], rest[1::2]):
            vals[f"{head}.{k}"] = float(v)
    return vals


@pytest.mark.parametrize("n,nz,method", [(16, 16, "etd2"), (32, 32, "etd2"), (48, 16, "etd2"), (32, 32, "etd4"),
                                          (32, 32, "euler")])
def test_single_cta_schedule_in_bounds(harness, n, nz, method):
    v = run_attempt(harness, n, nz, 2, method)
    assert v["ctrl.attempts"] == 1
    # every last-CTA counter was reset by the CTA that finalised
    assert all(v[f"ctrl.{k}"] == 0 for k in ("cnt_xy", "cnt_z"))
    # the synthetic state (a real-space field that does not match its spectrum) keeps the
    # ETD-RK2 candidate finite; the other methods' candidates may overflow in FP32, and
    # decide copies an accepted candidate into the state
    if method == "etd2":
        assert all(abs(v[k]) < float("inf") for k in ("state.V", "state.S", "cand.V", "cand.S"))


@pytest.mark.parametrize("n", [64])
def test_cluster_and_single_schedules_agree(harness, n):
    """64^2 planes (16 of them): the two-CTA cluster pass (distributed shared
    memory exchange) and the one-CTA pass in bounds, with the same sums."""
    a = run_attempt(harness, n, 16, 3)
    b = run_attempt(harness, n, 16, 2)
    # V, S, E: the same up to the order of the FP64 partial sums (per plane vs per half plane)
    for k in ("state.V", "state.S", "state.E", "work.V", "work.S", "cand.V", "cand.S", "cand.E"):
        assert a[k] == pytest.approx(b[k], rel=1e-9), (k, a, b)
    # the G'' and w totals, summed per thread in FP32 before the FP64 partials: equal to
    # the rounding of those per-thread sums
    for k in ("state.sum_g", "work.sum_g", "work.sum_h"):
        assert a[k] == pytest.approx(b[k], rel=1e-8, abs=1e-6 * n * n * 16), (k, a, b)
