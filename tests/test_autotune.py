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


def test_cluster_layouts_are_candidates_but_never_persistent(monkeypatch):
    """Both cluster layouts (two and six CTAs per ciphertext) are timed as one-ciphertext
    shapes; neither gets a persistent grid; shapes that fit no SM are left out."""
    from yatfhe_gb300 import _lib

    def fake_fit(ctx, per_cta, layout):
        if layout in (_lib.LAYOUT_ROW_CLUSTER, _lib.LAYOUT_CHANNEL_CLUSTER):
            return 1 if per_cta == 1 else 0
        return 2 if per_cta < 4 else 1

    monkeypatch.setattr(autotune.api, "ctas_per_sm", fake_fit)
    shapes = autotune.candidates(None)
    for layout in (_lib.LAYOUT_ROW_CLUSTER, _lib.LAYOUT_CHANNEL_CLUSTER):
        assert (layout, 1, 0) in shapes
        assert not [s for s in shapes if s[0] == layout and (s[1] != 1 or s[2] != 0)]
    assert (_lib.LAYOUT_CHANNEL_ROW, 2, 2) in shapes  # persistent shapes for the batched layouts
