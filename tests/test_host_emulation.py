"""The whole library on the CPU: host code and kernels under AddressSanitizer.

stepper.cu and the kernel translation units are compiled for the host against the
emulated runtime in tests/emu/host (host memory; streams that run their work at once;
stream capture and graph launch as recorded closures; kernels with one OS thread per
CUDA thread; a launch above 48 KB of dynamic shared memory fails unless the kernel's
limit was raised).  A C program then drives a session through the C ABI for both
forms at 16^3, and for the FP32 form at 96x96x32 (96^2 planes on the two-CTA cluster
pass over 32 planes): create, set phi, run, autotune, run, get phi, scalars, destroy.
Device buffers and shared memory sit between inaccessible guard regions (EMU_GUARD) and
local variables are pattern-initialised, so a wild or uninitialised index faults too.
Any access outside a host or emulated-device allocation, a refused launch or an error
code fails the test.  Needs g++ with AddressSanitizer; no GPU."""
import importlib.util
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.emulation

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cudabubble_gb300", "csrc")
EMU = os.path.join(ROOT, "tests", "emu")
UNITS = ["stepper.cu", "kernels_f32.cu", "kernels_f32_z.cu", "kernels_f64.cu", "kernels_f64_z.cu"]


def _rewrite():
    spec = importlib.util.spec_from_file_location("emu_rewrite", os.path.join(EMU, "rewrite.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def session_exe(tmp_path_factory):
    if not shutil.which("g++") or not shutil.which("gcc"):
        pytest.skip("g++ / gcc not available")
    d = tmp_path_factory.mktemp("hostemu")
    src = d / "src"
    n_decl = _rewrite().copy_sources(CSRC, str(src), sizes=[16, 32, 96], launches=True)
    assert n_decl >= 4
    fl = ["-O1", "-g", "-fsanitize=address", "-fno-omit-frame-pointer", "-ffp-contract=off"]
    probe = subprocess.run(["g++", "-ftrivial-auto-var-init=pattern", "-x", "c++", "-fsyntax-only", "-"],
                           input="int main() { return 0; }", capture_output=True, text=True)
    if probe.returncode == 0:
        fl.append("-ftrivial-auto-var-init=pattern")
    inc = ["-I", os.path.join(EMU, "host"), "-I", str(src), "-I", os.path.join(ROOT, "include")]
    jobs, objs = [], []
    for u in UNITS:
        o = str(d / (u + ".o"))
        objs.append(o)
        jobs.append(subprocess.Popen(["g++", "-std=c++17", *fl, *inc, "-x", "c++", "-c", str(src / u), "-o", o],
                                     stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    o = str(d / "runtime.o")
    objs.append(o)
    jobs.append(subprocess.Popen(["g++", "-std=c++17", *fl, *inc, "-c", os.path.join(EMU, "host", "runtime.cpp"),
                                  "-o", o], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    o = str(d / "sequence.o")
    objs.append(o)
    jobs.append(subprocess.Popen(["gcc", *fl, "-I", os.path.join(ROOT, "include"), "-c",
                                  os.path.join(EMU, "host", "sequence.c"), "-o", o],
                                 stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    for j in jobs:
        out = j.communicate()[0]
        if j.returncode != 0 and "sanitize" in out and "cannot find" in out:
            pytest.skip("AddressSanitizer runtime not available")
        assert j.returncode == 0, out[-4000:]
    exe = str(d / "session")
    r = subprocess.run(["g++", "-fsanitize=address", *objs, "-o", exe, "-lpthread", "-lm"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:halt_on_error=1", EMU_GUARD="1")


def test_session_through_the_c_abi_in_bounds(session_exe):
    r = subprocess.run([session_exe, "16"], capture_output=True, text=True, env=ENV, timeout=1200)
    assert "AddressSanitizer" not in r.stderr, r.stderr[-6000:]
    assert "EMU:" not in r.stderr, r.stderr[-3000:]  # a refused launch
    assert r.returncode == 0, (r.stdout, r.stderr[-3000:])
    rows = {}
    for line in r.stdout.splitlines():
        f = line.split()
        rows[int(f[1])] = {k: float(v) for k, v in zip(f[2::2], f[3::2])}
    assert set(rows) == {0, 1}
    for form in (0, 1):
        v = rows[form]
        assert v["rc"] == 0 and v["steps"] == 5
        assert 0.9 < v["maxphi"] < 1.1
    # the two forms integrate the same problem: same volume and area to the FP32 form's accuracy
    assert rows[1]["V"] == pytest.approx(rows[0]["V"], rel=1e-5)
    assert rows[1]["S"] == pytest.approx(rows[0]["S"], rel=1e-5)


def test_fp32_session_on_96x96x32_in_bounds(session_exe):
    """The FP32 form on 96^2 planes over 32 of them: cb_set_phi (FP64 plane and z
    transforms, then the FP32 z pass and the cluster fused pass), the stepping loop and
    cb_autotune over the cluster and one-CTA plane passes."""
    r = subprocess.run([session_exe, "96", "32", "1"], capture_output=True, text=True, env=ENV, timeout=5400)
    assert "AddressSanitizer" not in r.stderr, r.stderr[-6000:]
    assert "EMU:" not in r.stderr, r.stderr[-3000:]
    assert r.returncode == 0, (r.stdout, r.stderr[-3000:])
    f = r.stdout.split()
    v = {k: float(x) for k, x in zip(f[2::2], f[3::2])}
    assert v["rc"] == 0 and v["steps"] == 5
    assert 0.9 < v["maxphi"] < 1.1
