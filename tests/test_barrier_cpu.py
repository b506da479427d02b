"""Host logic of the barrier / end-state convergence summary (no GPU)."""
import numpy as np

from mepgl_gb300 import barrier, schedule


def test_time_within_needs_the_value_to_stay():
    t = [0.0, 1.0, 2.0, 3.0, 4.0]
    v = [2.0, 1.0000001, 1.5, 1.0000002, 1.0]
    assert barrier.time_within(t, v, 1.0, 1e-6) == 3.0
    assert barrier.time_within(t, v, 1.0, 1e-9) == 4.0
    assert barrier.time_within(t, [5.0] * 5, 1.0, 1e-6) is None


def test_summary_spreads_and_ends():
    rec = [(0.1 * k, 1.0 + 0.01 * np.sin(k), 3, -0.5 + 1e-3 / (k + 1), "fp64") for k in range(50)]
    s = barrier.summarise(rec, target_ends=-0.5, rtol=1e-4)
    assert s["iterations"] == 50 and s["argmax"] == 3
    assert np.isclose(s["barrier"], 1.0 + 0.01 * np.sin(49))
    assert 0 < s["barrier_spread"] <= 0.02
    assert s["time_to_ends_s"] is not None and s["time_to_ends_s"] <= 4.9


def test_schedule_barrier_is_max_minus_first():
    assert schedule.barrier([3.0, 5.0, 4.0]) == 2.0
    assert schedule.barrier([3.0, 1.0]) == 0.0


def test_compare_uses_first_run_as_reference(tmp_path):
    import json
    a = dict(summary=dict(schedule="fp64"), trace=[[1.0, 1.0, 1, -0.5, "fp64"], [2.0, 1.0, 1, -0.8, "fp64"]])
    b = dict(summary=dict(schedule="mixed"), trace=[[0.5, 1.0, 1, -0.8 + 1e-3, "fp32"], [0.9, 1.0, 1, -0.8, "fp64"]])
    pa, pb = tmp_path / "a.json", tmp_path / "b.json"
    pa.write_text(json.dumps(a))
    pb.write_text(json.dumps(b))
    rows = barrier.compare([str(pa), str(pb)], 1e-6)
    assert rows[0]["time_to_ends_s"] == 2.0 and rows[1]["time_to_ends_s"] == 0.9


def test_build_applies_autotuned_definitions(tmp_path, monkeypatch):
    import json
    from mepgl_gb300 import build
    t = tmp_path / "tuning.json"
    t.write_text(json.dumps({"selected": {"MEPGL_ROWS_F32": 16, "MEPGL_MINB_DIR": 4}}))
    monkeypatch.setattr(build, "TUNING", str(t))
    monkeypatch.delenv("MEPGL_NO_TUNING", raising=False)
    assert build.tuned_flags() == ["-DMEPGL_MINB_DIR=4", "-DMEPGL_ROWS_F32=16"]
    monkeypatch.setenv("MEPGL_NO_TUNING", "1")
    assert build.tuned_flags() == []
