"""Host-side arithmetic of bench.py (no GPU): the work model and the
step-level roofline built from the per-phase fractions."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_work_model_per_particle():
    # neighbour walk: packed record, the list and its count
    assert bench.work_model("neighbors", 100.0, True) == ("byte", 64 + 4 * 100.0 + 4)
    # the signal speed rides in the mixed acceleration pass
    assert bench.work_model("accel", 10.0, True) == ("flop", (82 + 27) * 10.0)
    assert bench.work_model("accel", 10.0, False) == ("flop", 82 * 10.0)
    assert bench.work_model("gravity", 10.0, True) == (None, None)


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
