"""CPU test of bench.py's reference arm: one JSON line with the keys the benchmark contract
names (metric, unit, config, e2e with zero copy bytes, cpu_baseline describing the run), on
a small sample so that it finishes in seconds.  Also the workload helpers the GPU legs share:
the synthetic inputs are seeded, and the test polynomial is a valid torus polynomial."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup",
                        "0", "--cpu-sample", "4"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] and d["unit"] == "bootstraps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1
    assert d["config"]["workload"] == "t32_n1024_batch65536" and d["config"]["cpu_sample_per_step"] == 4
    assert d["e2e"] == {"value": d["value"], "unit": "bootstraps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]


def test_workload_helpers_are_seeded_and_in_range():
    sys.path.insert(0, str(ROOT))
    import bench
    from yatfhe_gb300.params import T32_N1024, WWL24_T56_N2048

    for p in (T32_N1024, WWL24_T56_N2048):
        a, b = bench.synthetic_lwe(p, 5, 7), bench.synthetic_lwe(p, 5, 7)
        assert a.shape == (5, p.n + 1) and a.dtype == np.int32
        np.testing.assert_array_equal(a, b)
        lut = bench.workload_lut(p)
        assert lut.shape == (p.N,) and lut.dtype == np.int64
        half = 1 << (p.torus_bits - 1)
        assert np.all(lut >= -half) and np.all(lut < half)
