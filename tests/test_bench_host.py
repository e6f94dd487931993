"""Host-side pieces of bench.py that need no GPU: the metric and unit the
line is quoted in, the algorithmic bytes per cell-step the rooflines use,
the workload record both arms print, and the committed roofline traffic
entries the default line reads."""
import json

import bench
from opensayal_gb300 import scenarios
from tests.conftest import ROOT


def test_bytes_per_cell_step():
    # forces 8, diffusion 8 a sweep, projection 17 a sweep, advection 17 + 17
    assert bench.bytes_per_cell_step(50, True) == 1292
    assert bench.bytes_per_cell_step(50, False) == 892
    assert bench.bytes_per_cell_step(200, True) == 25 * 200 + 42


def test_workload_record_is_the_same_for_both_arms():
    cfg = scenarios.default_tunnel_config()
    a = bench.config_record(cfg, "default", 1)
    b = bench.config_record(cfg, "default", 1)
    assert a == b
    assert (a["width"], a["height"], a["projection_n"]) == (1920, 1080, 50)
    assert a["storage"] == "f32" and a["parallelism"] == "single"
    assert "model" not in a
    assert bench.config_record(cfg, "default", 4)["parallelism"] == "replicas"


def test_metric_and_unit():
    assert bench.UNIT == "cell-steps/s"
    assert bench.METRIC.startswith("cell-steps/s")


def test_roofline_traffic_entries():
    entries = json.loads((ROOT / "profiles" / "roofline_traffic.json").read_text())
    resident = entries["default:block8:resident"]
    # about the compulsory u, v and flag bytes once per phase (9 B a cell)
    assert 0.95 < resident["bytes_per_launch"] / (1920 * 1080 * 9) < 1.05
    assert 0.0 < resident["smsp__issue_active"] <= 1.0
    assert 0.0 < resident["l1tex__throughput"] <= 1.0
    for entry in entries.values():
        assert entry["bytes_per_launch"] > 0
        assert entry["source"].startswith(("measured", "scaled"))
