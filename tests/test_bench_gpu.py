"""The GPU arm of bench.py prints the benchmark contract's line (a small
headline case, 2^18 rows): metric, value and timing keys, the workload, the
roofline object (bound, achieved, peak, fraction, the timed kernel), the CPU
baseline, the end-to-end object with its host-link floor, the launch count
and the clock record."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_gpu_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--headline-only", "--log2n", "18", "--steps", "3", "--warmup", "3"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks"):
        assert key in d, key
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["dtype"] == "f64"
    assert "n=2^18" in d["config"]["workload"]
    rf = d["roofline"]
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s" and rf["peak"] > 0
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-3
    assert rf["kernel"] in ("csr_sell_kernel", "csr_pair_kernel")
    assert rf["traffic"] is None  # measured for the 2^24 workload only
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] == "port"
    e = d["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] == e["d2h_bytes_per_step"] == (1 << 18) * 8
    assert e["transfer_floor_ms"] > 0 and 0 < e["of_transfer_floor"] <= 1.5
    assert d["gpu_launches"] >= d["steps"]
    assert d["clocks"]["sm_max_mhz"] > 0
