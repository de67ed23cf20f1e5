"""Host logic of the launch-shape autotuner (no GPU): candidate choice per objective."""
import pytest

from yatfhe_gb300 import autotune

RESULTS = [
    {"layout": 0, "per_cta": 4, "ctas_per_sm": 0, "bootstraps_per_s": 22000.0, "single_ms": 17.8},
    {"layout": 0, "per_cta": 2, "ctas_per_sm": 0, "bootstraps_per_s": 22700.0, "single_ms": 17.1},
    {"layout": 1, "per_cta": 1, "ctas_per_sm": 0, "bootstraps_per_s": 22400.0, "single_ms": 10.1},
    {"layout": 1, "per_cta": 2, "ctas_per_sm": 0, "bootstraps_per_s": 18000.0, "single_ms": 9.0},
]


def test_throughput_objective_takes_the_fastest_shape():
    assert autotune.pick(RESULTS, "throughput") is RESULTS[1]


def test_latency_objective_takes_the_quickest_shape_near_peak_throughput():
    # 9.0 ms is quicker but 21 % below peak throughput; 10.1 ms is within 15 %
    assert autotune.pick(RESULTS, "latency") is RESULTS[2]


def test_unknown_objective_is_rejected():
    with pytest.raises(ValueError):
        autotune.tune(None, None, None, objective="energy")
