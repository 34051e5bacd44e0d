"""The reference's on-disk formats, so a run can resume from the reference's
files and the reference can resume from ours.

* ``.out``: the raw FP64 phase field ``[nz][ny][nx]``, x fastest, host byte
  order, no header (``tool.cpp:28-59``).  Grids above 100,000 bytes use one
  file per name; smaller ones carry the output time index
  (``fluidbase.cpp:260-276``).
* ``.info``: seven doubles: current time, time step, alpha, beta, alpha3,
  alpha_1, beta_1 (``fluidbase.cpp:2776-2826``).
* ``<name><nx>x<ny>x<nz>.txt`` logs: one line per output,
  ``%08d, %15.12f`` (one or two values) or ``%08d, %8.5f x 9`` (more), the
  leading field being round(time / 1e-6) (``fluidbase.cpp:286-323``).
* ``_xz`` / ``_xy`` text slices of a field at y = ny/2 and z = nz/2
  (``fluidbase.cpp:224-258``).
"""
from __future__ import annotations

import math
import os
import struct

import numpy as np

TIME_STEP_OUTPUT = 1e-6  # stdafx.h:41


def roundx(x: float) -> int:
    """tool.cpp:23-26."""
    return int(math.floor(x + 0.5))


def tag(shape) -> str:
    nz, ny, nx = shape
    return f"{nx}x{ny}x{nz}"


def out_path(folder: str, name: str, shape, time: float) -> str:
    nz, ny, nx = shape
    if nx * ny * nz * 8 > 100000:
        return os.path.join(folder, f"{name}{tag(shape)}.out")
    return os.path.join(folder, f"{name}{tag(shape)}_{roundx(time / TIME_STEP_OUTPUT):08d}.out")


def write_out(folder: str, name: str, u: np.ndarray, time: float) -> str:
    path = out_path(folder, name, u.shape, time)
    np.ascontiguousarray(u, dtype=np.float64).tofile(path)
    return path


def read_out(folder: str, name: str, shape, time: float = 0.0) -> np.ndarray | None:
    """The field, or None when the file is missing (the reference zeroes the
    array then, tool.cpp:49-53; the caller decides)."""
    path = out_path(folder, name, shape, time)
    if not os.path.exists(path):
        return None
    a = np.fromfile(path, dtype=np.float64)
    if a.size != int(np.prod(shape)):
        raise ValueError(f"{path}: {a.size} values, expected {int(np.prod(shape))}")
    return a.reshape(shape)


INFO_FIELDS = ("time_current", "time_step", "alpha", "beta", "alpha3", "alpha_1", "beta_1")


def info_path(folder: str, shape) -> str:
    return os.path.join(folder, f"{tag(shape)}.info")


def write_info(folder: str, shape, info: dict) -> str:
    path = info_path(folder, shape)
    with open(path, "wb") as f:
        f.write(struct.pack("=7d", *[float(info.get(k, 0.0)) for k in INFO_FIELDS]))
    return path


def read_info(folder: str, shape) -> dict | None:
    """The .info values with load_info's repairs (fluidbase.cpp:2818-2819): a
    time step below 1e-13 becomes 1e-7 and a zero time becomes 1e-13.  None
    when there is no file (a new experiment)."""
    path = info_path(folder, shape)
    if not os.path.exists(path):
        return None
    with open(path, "rb") as f:
        vals = struct.unpack("=7d", f.read(56))
    info = dict(zip(INFO_FIELDS, vals))
    if info["time_step"] < 1e-13:
        info["time_step"] = 1e-7
    if info["time_current"] == 0.0:
        info["time_current"] = 1e-13
    return info


def log_line(time: float, *values: float) -> str:
    idx = roundx(time / TIME_STEP_OUTPUT)
    if len(values) == 1:
        return f"{idx:08d}, {values[0]:15.12f}\n"
    if len(values) == 2:
        return f"{idx:08d}, {values[0]:15.12f}, {values[1]:15.12f}\n"
    v = list(values) + [0.0] * (9 - len(values))
    return f"{idx:08d}, " + ", ".join(f"{x:8.5f}" for x in v[:9]) + "\n"


def append_log(folder: str, name: str, shape, time: float, *values: float) -> None:
    with open(os.path.join(folder, f"{name}{tag(shape)}.txt"), "a") as f:
        f.write(log_line(time, *values))


def write_slices(folder: str, name: str, u: np.ndarray, time: float) -> None:
    nz, ny, nx = u.shape
    idx = roundx(time / TIME_STEP_OUTPUT)
    with open(os.path.join(folder, f"{name}{tag(u.shape)}_{idx:08d}_xz.txt"), "w") as f:
        for i in range(nz):
            f.write("".join(f"{x:7.5f} " for x in u[i, ny // 2, :]) + "\n")
    with open(os.path.join(folder, f"{name}{tag(u.shape)}_{idx:08d}_xy.txt"), "w") as f:
        for i in range(ny):
            f.write("".join(f"{x:6.3f} " for x in u[nz // 2, i, :]) + "\n")
