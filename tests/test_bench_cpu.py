"""Host logic of bench.py (no GPU): the clock-sample summary and its throttle reasons, the byte model of the
roofline, and the committed DRAM-traffic figures it reads."""
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def test_clock_summary_from_nvml_samples():
    s = bench.ClockSampler(0)
    s.samples = [(2070.0, 2070.0, 0x0), (2055.0, 2070.0, 0x4), (2070.0, 2070.0, 0x0)]
    out = s.summary()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 3
    assert out["reasons"] == ["sw_power_cap"] and out["source"] == "nvml"
    s.samples.append((1500.0, 2070.0, 0x8 | 0x40))
    assert s.summary()["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap"]


def test_clock_summary_from_nvidia_smi_lines():
    s = bench.ClockSampler(0)
    s.lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 2040, 2070, 1200.5, 0x4, Not Active, Not Active, Active, Active",
               "garbage"]
    out = s.summary()
    assert out["samples"] == 2 and out["sm_mhz"] == pytest.approx(2055.0)
    assert out["reasons"] == ["sw_power_cap", "sw_thermal_slowdown"] and out["source"] == "nvidia-smi"


def test_algorithmic_bytes_model():
    # 2-D Euler FP32, MUSCL2 (Br = D) with the degree-1 divergence fit (Bd = D + 1)
    flux, gather = bench.algorithmic_bytes(19.26, 2, 4, 2, 3, 4)
    assert flux == pytest.approx(4 * 19.26 + 16 + 72 + 4 * 4 * 7)
    assert gather == pytest.approx(4 * 19.26 + 16 + 32 + 4 * 4 * 3)


def test_recorded_traffic_is_read():
    t = bench.recorded_traffic()
    for w in ("euler2d_quadrant_1M", "euler3d_blast_8M"):
        assert t[f"flux_f32_{w}_bytes_per_point_stage"] > 0.0
        assert t[f"gather_f32_{w}_bytes_per_point_stage"] > 0.0


def test_radial_blast_reference_conserves_mass_and_converges():
    """The 1-D spherical reference of the equal-L1 study: mass is conserved while the waves stay inside, and halving
    the cell size moves the solution by much less than the 3-D errors it judges (~1e-2)."""
    import numpy as np
    r = np.linspace(0.0, 0.6, 2401)
    w = r ** 2
    coarse = bench.radial_blast_reference(0.02, r, n=600)
    fine = bench.radial_blast_reference(0.02, r, n=1200)
    assert np.sum(np.abs(coarse - fine) * w) / np.sum(fine * w) < 5e-3
    m0 = np.sum(np.where(r < 0.2, 1.0, 0.125) * w)
    assert abs(np.sum(fine * w) - m0) / m0 < 2e-3           # trapezoid-free sum on a fine radius grid
    assert fine[0] == 1.0 and fine[-1] == 0.125


def test_predictor_threshold_rule(tmp_path, monkeypatch):
    import json
    table = {"0.9": {"precision": 0.85, "recall": 0.7}, "0.95": {"precision": 0.92, "recall": 0.5},
             "0.99": {"precision": 0.97, "recall": 0.2}}
    monkeypatch.setattr(bench, "PKG", tmp_path)
    (tmp_path / "predictor_euler2d_holdout.json").write_text(
        json.dumps({"min_precision": 0.9, "table": table, "threshold": 0.95}))
    thr, rule, ok = bench._predictor_threshold()
    assert thr == 0.95 and ok and "held-out" in rule
    (tmp_path / "predictor_euler2d_holdout.json").write_text(
        json.dumps({"min_precision": 0.99, "table": table, "threshold": None}))
    thr, rule, ok = bench._predictor_threshold()
    assert thr == 0.9 and not ok and "0.97 at 0.99" in rule
    (tmp_path / "predictor_euler2d_holdout.json").unlink()
    assert bench._predictor_threshold()[2] is False


def test_recorded_learned_ratio(tmp_path, monkeypatch):
    import json
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    (tmp_path / "profiles").mkdir()
    assert bench.learned_l1_ratio("euler3d_blast_8M", 0.9)[0] is None
    (tmp_path / "profiles" / "accuracy_equal_l1.json").write_text(
        json.dumps({"threshold": 0.9, "euler3d_blast_8M": {"learned_over_fp64": 1.5}}))
    assert bench.learned_l1_ratio("euler3d_blast_8M", 0.9)[0] == 1.5
    assert bench.learned_l1_ratio("euler3d_blast_8M", 0.99)[0] is None
    (tmp_path / "profiles" / "accuracy_learned.json").write_text(
        json.dumps({"euler3d_blast_8M": {"learned": {"0.99": {"over_fp64": 1.05}}}}))
    assert bench.learned_l1_ratio("euler3d_blast_8M", 0.99) == (1.05, "profiles/accuracy_learned.json")
    assert bench.learned_l1_ratio("euler3d_blast_8M", 0.9)[0] == 1.5


def test_committed_holdout_table_is_consistent():
    import json
    d = json.loads((ROOT / "hypercloudcore.jl_gb300" / "predictor_euler2d_holdout.json").read_text())
    q = [float(k) for k, v in d["table"].items() if v["precision"] >= d["min_precision"]]
    assert d["threshold"] == (min(q) if q else None)
    for v in d["table"].values():
        assert v["precision"] == pytest.approx(v["tp"] / (v["tp"] + v["fp"]))
        assert v["recall"] == pytest.approx(v["tp"] / (v["tp"] + v["fn"]))
