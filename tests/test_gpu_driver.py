"""The reference-compatible driver (cudabubble_gb300/driver.py) on the GPU:
a run writes the reference's outputs, and a run resumed from its .out /
.info files (ninit = 7) continues the uninterrupted trajectory."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ini(ifold, ninit):
    # ifold nx ny nz xlen ylen zlen b_shape time_step fluid_dt fixed_dt ninit nflush surctrl epssize ncur angle
    # re eta ga alpha beta M1 M2 M3 M4 tmax output_interval gweight einit k c linet alpha3 | method precision
    return (f"{ifold} 32 32 32 1 1 1 0 1e-6 5e-6 0 {ninit} -1 1 150 0 30 1.0 1 1 -1 -1 1.0e4 1.0e4 1.0e4 1.0e4 "
            f"100.0 30 0.05 0 30.0 70 10 -1 1 0\n")


def test_driver_outputs_and_resume(cblib, tmp_path):
    from cudabubble_gb300 import capi, checkpoint, driver
    res = str(tmp_path)
    (tmp_path / "ini0.dat").write_text(_ini(7, 2))
    driver.Run(res, 0, output_seconds=1e9).run(max_steps=32)
    fold = os.path.join(res, "7")
    for name in ("d32x32x32.out", "32x32x32.info", "energy32x32x32.txt", "vol_sur32x32x32.txt",
                 "lamb32x32x32.txt", "error32x32x32.txt", "time_step32x32x32.txt", "alpha_beta32x32x32.txt",
                 "output32x32x32.txt", "ini0.dat"):
        assert os.path.exists(os.path.join(fold, name)), name
    assert len(open(os.path.join(fold, "vol_sur32x32x32.txt")).readlines()) == 2  # start and end
    assert "Start STATIC Running" in open(os.path.join(fold, "output32x32x32.txt")).read()
    info = checkpoint.read_info(fold, (32, 32, 32))
    d32 = checkpoint.read_out(fold, "d", (32, 32, 32))

    # the same 48 steps uninterrupted
    p = capi.params_from_ini(_ini(7, 2))
    st = capi.Stepper(p)
    st.set_phi(driver.Run(res, 0).initial_phi())
    st.run(32)
    s32 = st.scalars()
    assert s32["t"] == pytest.approx(info["time_current"], rel=1e-15)
    assert s32["dt"] == info["time_step"]
    assert np.abs(st.get_phi() - d32).max() == 0.0
    st.run(16)
    want_E, want_phi = st.scalars()["E"], st.get_phi()
    st.close()

    # resume from the files: ninit = 7 loads d<grid>.out, the .info restores time, dt, alpha, beta
    (tmp_path / "ini0.dat").write_text(_ini(7, 7))
    driver.Run(res, 0, output_seconds=1e9).run(max_steps=16)
    got = checkpoint.read_out(fold, "d", (32, 32, 32))
    info2 = checkpoint.read_info(fold, (32, 32, 32))
    assert np.abs(got - want_phi).max() <= 1e-10
    E2 = float(open(os.path.join(fold, "energy32x32x32.txt")).readlines()[-1].split(",")[4])
    assert E2 == pytest.approx(want_E, abs=2e-5)  # the log keeps 5 decimals
    assert info2["time_current"] > info["time_current"]


def test_driver_shape_adjust_on_new_run(cblib, tmp_path):
    """A new run with a nonzero shape flag (ini field 8) relaxes the start shape
    first (belastic.cpp:558-560); a resumed run does not."""
    from cudabubble_gb300 import capi, checkpoint, driver
    res = str(tmp_path)
    line = _ini(9, 2).split()
    line[7] = "1"
    (tmp_path / "ini0.dat").write_text(" ".join(line) + "\n")
    driver.Run(res, 0, output_seconds=1e9).run(max_steps=16)
    fold = os.path.join(res, "9")
    out = open(os.path.join(fold, "output32x32x32.txt")).read()
    assert "Start Shape Adjusting" in out and "Shape Adjust Ended successfully" in out
    d16 = checkpoint.read_out(fold, "d", (32, 32, 32))

    p = capi.params_from_ini(" ".join(line))
    st = capi.Stepper(p)
    st.set_phi(driver.Run(res, 0).initial_phi())
    a = st.shape_adjust()
    assert a["steps"] > 0 and a["E_end"] < a["E_start"]
    st.run(16)
    assert np.abs(st.get_phi() - d16).max() < 1e-12
    st.close()

    # resuming from the .info file skips the adjustment
    line[11] = "7"
    (tmp_path / "ini0.dat").write_text(" ".join(line) + "\n")
    driver.Run(res, 0, output_seconds=1e9).run(max_steps=4)
    out2 = open(os.path.join(fold, "output32x32x32.txt")).read()
    assert out2.count("Start Shape Adjusting") == 1
