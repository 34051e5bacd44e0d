"""The reference's checkpoint and log formats (cudabubble_gb300/checkpoint.py),
on the host: .out raw FP64 fields and their names, the 7-double .info with
load_info's repairs, and the text log lines."""
import os
import struct

import numpy as np

from cudabubble_gb300 import checkpoint as ck


def test_out_round_trip_and_names(tmp_path):
    rng = np.random.default_rng(0)
    big = rng.standard_normal((32, 32, 32))  # 262 kB: one file per name
    p = ck.write_out(str(tmp_path), "d", big, 0.00123)
    assert os.path.basename(p) == "d32x32x32.out"
    assert os.path.getsize(p) == big.size * 8
    assert np.array_equal(ck.read_out(str(tmp_path), "d", big.shape, 5.0), big)
    small = rng.standard_normal((8, 16, 16))  # 16 kB: the time index joins the name
    p = ck.write_out(str(tmp_path), "d", small, 2.5e-5)
    assert os.path.basename(p) == "d16x16x8_00000025.out"
    assert np.array_equal(ck.read_out(str(tmp_path), "d", small.shape, 2.5e-5), small)
    assert ck.read_out(str(tmp_path), "d", small.shape, 0.0) is None
    # x fastest, as tool.cpp writes d[i][j] rows of nx doubles
    raw = np.fromfile(os.path.join(str(tmp_path), "d32x32x32.out"), dtype=np.float64)
    assert raw[1] == big[0, 0, 1] and raw[32] == big[0, 1, 0]


def test_info_layout_and_repairs(tmp_path):
    shape = (16, 24, 24)
    ck.write_info(str(tmp_path), shape, {"time_current": 0.0, "time_step": 1e-20, "alpha": 9.3, "beta": 21.8})
    raw = open(os.path.join(str(tmp_path), "24x24x16.info"), "rb").read()
    assert len(raw) == 56
    assert struct.unpack("=7d", raw)[:4] == (0.0, 1e-20, 9.3, 21.8)
    info = ck.read_info(str(tmp_path), shape)
    assert info["time_current"] == 1e-13 and info["time_step"] == 1e-7  # fluidbase.cpp:2818-2819
    assert (info["alpha"], info["beta"]) == (9.3, 21.8)
    assert ck.read_info(str(tmp_path), (8, 8, 8)) is None


def test_log_lines():
    assert ck.log_line(3.2e-5, 1.5) == "00000032,  1.500000000000\n"
    assert ck.log_line(1e-6, 9.25, -0.5) == "00000001,  9.250000000000, -0.500000000000\n"
    line = ck.log_line(0.0, 1.0, 2.0, 3.0, 6.0)
    assert line.startswith("00000000,  1.00000,  2.00000,  3.00000,  6.00000,  0.00000")
    assert line.count(",") == 9
