"""Host-side arithmetic of bench.py (no GPU): the work model and the
step-level roofline built from the per-phase fractions."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_work_model_per_particle():
    W = bench.WORK
    # neighbour walk: positions in, the count and the list out
    assert bench.work_model("neighbors", 100.0, True) == {
        "flop": 0.0, "byte": W["BYTES_NEIGHBORS"] + 4 * 100.0}
    # the signal speed rides in the mixed acceleration pass
    assert bench.work_model("accel", 10.0, True)["flop"] == (82 + 27) * 10.0
    assert bench.work_model("accel", 10.0, False)["flop"] == 82 * 10.0
    assert bench.work_model("energy", 10.0, True, thermokinetic=False)["flop"] == 84 * 10.0
    assert bench.work_model("gravity", 10.0, True) is None
    assert bench.work_model("integrate", 10.0, True) == {"flop": 0.0, "byte": 288.0}
    assert bench.work_model("sort", 10.0, True) == {"flop": 0.0, "byte": 304.0}


def test_work_model_is_the_header():
    """bench.py's constants are the ones include/fsph_work.h defines, and
    the per-phase bytes add up to the header's per-particle-step total."""
    import re
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "include", "fsph_work.h")).read()
    defs = {m.group(1): float(m.group(2))
            for m in re.finditer(r"#define FSPH_(\w+) ([0-9.]+)", hdr)}
    assert defs == bench.WORK
    phases = ["RANGE_KEYS", "SORT", "TREE", "DENSITY", "ACCEL", "DEDT",
              "RECOMPUTE_P", "INTEGRATE", "DT"]
    assert sum(defs["BYTES_" + k] for k in phases) == defs["BYTES_PARTICLE_STEP_FP64"]
    assert defs["BYTES_PAIR_LISTS"] == 5 * defs["BYTES_PAIR_LIST"]


def test_phase_roofline_picks_the_binding_resource():
    # 1e6 particles: 100 flop/particle at 10 TFLOP/s is 0.01 ms; 1000 B at
    # 1000 GB/s is 1 ms, so the phase is HBM-bound
    r = bench.phase_roofline({"flop": 100.0, "byte": 1000.0}, 1e6, 2e-3, 10.0, "fp32",
                             peak_hbm=1000.0)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(500.0)
    assert r["frac"] == pytest.approx(0.5)
    assert r["t_roof_ms"] == pytest.approx(1.0)
    r = bench.phase_roofline({"flop": 1e5, "byte": 10.0}, 1e6, 0.02, 10.0, "fp32",
                             peak_hbm=1000.0)
    assert r["bound"] == "fp32" and r["frac"] == pytest.approx(0.5)


def test_step_roofline_sums_modelled_phases():
    per_phase = {"sort": {"frac": 0.5}, "accel": {"frac": 0.25}}
    phase_ms = {"sort": 0.4, "accel": 1.2, "gravity": 3.0}
    r = bench.step_roofline(per_phase, phase_ms, 5.0)
    assert r["t_roof_ms"] == pytest.approx(0.5 * 0.4 + 0.25 * 1.2)
    assert r["frac"] == pytest.approx(0.5 / 5.0)
    assert r["unmodelled_ms"] == {"gravity": 3.0}
    assert r["t_step_ms"] == 5.0


def test_step_roofline_empty_step():
    r = bench.step_roofline({}, {}, 0.0)
    assert r["t_roof_ms"] == 0 and r["frac"] is None
