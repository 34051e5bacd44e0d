"""The schedule tuner's coordinate search (cudabubble_gb300/tune.py) on the CPU: the
timing of a candidate build is replaced by a fixed cost table, so only the search and
the schedule file it writes are tested here; its GPU use is a tool run."""
import os

from cudabubble_gb300 import tune


def test_coordinate_search_keeps_the_fastest_option_per_knob(tmp_path, monkeypatch):
    # cost of a schedule: a base, minus what each define saves; one option drifts too far
    saves = {"-DCB_Z_TX=8": 0.02, "-DCB_Z_TX=32": -0.05, "-DCB_PLAN128_8X16": 0.01, "-DCB_PLAN96_12X8": 0.03,
             "-DCB_XY_CLUSTER=0": -0.1}
    drift = {"-DCB_PLAN96_12X8": 1e-3}
    calls = []

    def fake(defs, sizes, steps):
        calls.append(tuple(defs))
        ms = 0.2 - sum(saves.get(d, 0.0) for d in defs)
        e = 10.0 * (1 + sum(drift.get(d, 0.0) for d in defs))
        return {str(n): {"ms_per_attempt": ms, "E": e, "steps": steps, "rejects": 0} for n in sizes}

    monkeypatch.setattr(tune, "_measure", fake)
    monkeypatch.setattr(tune.B, "SCHEDULE", str(tmp_path / "schedule.txt"))
    final, table = tune.tune([64, 128], [1.0, 1.0], 50, write=True, log=lambda *a: None)
    # z tile 8 x 128 and the 8 x 16 split are faster; 12 x 8 is refused for its energy drift
    assert final == ["-DCB_Z_TX=8", "-DCB_Z_NT=128", "-DCB_PLAN128_8X16"]
    assert len(set(calls)) == len(calls)  # every candidate built and timed once
    text = open(tmp_path / "schedule.txt").read()
    lines = [l for l in text.splitlines() if l and not l.startswith("#")]
    assert lines == final
    # build.py reads the chosen defines back from the file
    monkeypatch.delenv("CB_NVCC_DEFINES", raising=False)
    assert tune.B.defines() == final
