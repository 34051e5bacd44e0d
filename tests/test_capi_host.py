"""Host-side checks of the C ABI (no GPU needed): the library loads, exports
every symbol include/cbstep.h declares, parses the reference's ini first line
like fluidbase.cpp:33-143, and fails loudly (never falls back) without a GPU."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "cbstep.h")).read()
    return sorted(set(re.findall(r"\b(cb_[A-Za-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(cblib):
    from cudabubble_gb300 import capi
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(cblib, n), n
    assert set(names) == set(capi.SIGNATURES), set(names) ^ set(capi.SIGNATURES)


def test_ini0_first_line(cblib):
    from cudabubble_gb300 import capi
    line = open(os.path.join(ROOT, "tests", "golden", "ini0_line.txt")).read()
    p = capi.params_from_ini(line)
    assert (p.nx, p.ny, p.nz) == (128, 128, 128)
    assert p.epssize == 200 and p.time_step == 1e-7 and p.fixed_time_step == 1
    assert p.M1 == 1e4 and p.M2 == 1e4 and p.eta == 1 and p.ga == 1
    assert p.alpha == 0 and p.beta == 0  # beta < 0 -> alpha = beta = 0 (fluidbase.cpp:143)
    assert p.method == capi.CB_ETD4 and p.precision == capi.CB_FP64  # main.cpp:18, no selector fields
    eps = cblib.cb_params_eps(p)
    assert eps == pytest.approx(2.0 * 2 * 3.141592653589793 / 128, rel=1e-15)  # epssize 200 -> 2h


def test_ini_selector_fields_and_errors(cblib):
    from cudabubble_gb300 import capi
    base = open(os.path.join(ROOT, "tests", "golden", "ini0_line.txt")).read().split()
    p = capi.params_from_ini(" ".join(base + ["1", "1"]))
    assert p.method == capi.CB_ETD2 and p.precision == capi.CB_FP32
    with pytest.raises(capi.CBError):
        capi.params_from_ini("100 0 0 0")
    with pytest.raises(capi.CBError):
        capi.params_from_ini(" ".join(base + ["7"]))
    # a short line keeps defaults for the fields fscanf never reached
    p = capi.params_from_ini("5 32 32 16 1 1 1")
    assert (p.nx, p.nz) == (32, 16) and p.M1 == 0


def test_eps_rule_matches_reference_table(cblib):
    from cudabubble_gb300 import capi, shapes
    h = 2 * 3.141592653589793 / 64
    want = {1: 2.5 * (2 ** 0.5) * h / 2, 2: 2.5 * h, 3: 1.5 * h, 4: 1.25 * h, 5: h, 6: 0.7 * h, 7: 4 * h,
            8: 2.5 * (2 ** 0.5) * h / 2 * 1.22, 150: 1.5 * h, 200: 2 * h, 0: 2 * h, 9: 2 * h}
    for es, e in want.items():
        p = capi.default_params(nx=64, nz=64, epssize=es)
        assert cblib.cb_params_eps(p) == pytest.approx(e, rel=1e-14), es
        assert shapes.eps_rule(es, 64) == pytest.approx(e, rel=1e-14), es


def test_supported_and_bytes(cblib):
    from cudabubble_gb300 import capi
    for n in (16, 24, 32, 48, 64, 96, 128):
        p = capi.default_params(nx=n, ny=n, nz=n, precision=capi.CB_FP32, method=capi.CB_ETD2)
        assert cblib.cb_supported(p) == 1
        assert cblib.cb_instance_bytes(p) > 12 * n * n * (n // 2 + 1) * 8
    p = capi.default_params(nx=30, nz=30)
    assert cblib.cb_supported(p) == 0
    p = capi.default_params(nx=31, nz=32)
    assert cblib.cb_instance_bytes(p) == -1


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="checks the no-GPU error path")
def test_create_fails_loudly_without_gpu(cblib):
    from cudabubble_gb300 import capi
    p = capi.default_params(nx=16, ny=16, nz=16)
    with pytest.raises(capi.CBError) as ei:
        capi.Stepper(p)
    assert ei.value.code == capi.CB_ECUDA


C_PROGRAM = r"""
#include <stddef.h>
#include <stdio.h>
#include "cbstep.h"
int main(int argc, char** argv) {
    cb_params p;
    cb_params_default(&p);
    if (cb_params_from_ini_line(argv[1], &p) != CB_OK) { printf("ERR %s\n", cb_last_error()); return 1; }
    printf("%d %d %d %.17g %d %d\n", p.nx, p.ny, p.nz, cb_params_eps(&p), p.method, p.precision);
    printf("%zu %zu %zu %zu %zu\n", sizeof(cb_params), offsetof(cb_params, reject_tol), offsetof(cb_params, spont_c),
           sizeof(cb_run_stats), sizeof(cb_adjust_stats));
    return 0;
}
"""


@pytest.mark.parametrize("compiler", ["gcc", "g++"])
def test_header_compiles_and_links_from_c_and_cpp(cblib, tmp_path, compiler):
    """The drop-in boundary from the reference's own side: a C (and C++) caller
    includes include/cbstep.h, links libcbstep.so and parses the ini line; the
    struct layouts agree with the ctypes mirror the tests use."""
    import ctypes
    import shutil
    import subprocess
    from cudabubble_gb300 import capi
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not installed")
    src = tmp_path / ("t.c" if compiler == "gcc" else "t.cpp")
    src.write_text(C_PROGRAM)
    exe = tmp_path / "t"
    libdir = os.path.dirname(capi.LIB_PATH)
    r = subprocess.run([compiler, "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe), "-L", libdir, "-lcbstep", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    line = open(os.path.join(ROOT, "tests", "golden", "ini0_line.txt")).read().strip()
    out = subprocess.run([str(exe), line], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    l1, l2 = out.stdout.split("\n")[:2]
    p = capi.params_from_ini(line)
    f = l1.split()
    assert (int(f[0]), int(f[1]), int(f[2])) == (p.nx, p.ny, p.nz)
    assert float(f[3]) == capi.lib().cb_params_eps(ctypes.byref(p))
    sizes = [int(v) for v in l2.split()]
    assert sizes == [ctypes.sizeof(capi.cb_params), capi.cb_params.reject_tol.offset, capi.cb_params.spont_c.offset,
                     ctypes.sizeof(capi.cb_run_stats), ctypes.sizeof(capi.cb_adjust_stats)]
