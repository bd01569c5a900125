"""The benchmark's reference arm on the CPU: one JSON line with the keys of
the contract (impl, metric, value, unit, timing, config, cpu_baseline, e2e)
and the same metric, unit and workload as the GPU arm, on a small cqmat
matrix (2^16 rows) so that it runs in seconds."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--log2n", "16", "--steps", "2",
                        "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    sys.path.insert(0, ROOT)
    import bench
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "GB/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["config"]["workload"] == bench.WORKLOAD.format(log2n=16)
    assert d["config"]["n"] == 1 << 16 and d["config"]["nnz"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_loads_no_product_library():
    """The reference arm generates and multiplies with the oracle alone: the
    product library is never loaded into its process."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--log2n', '14', '--steps', '1', "
            "'--warmup', '1']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('PRODUCT_LOADED', 'libtbsla_gb300' in maps, 'ORACLE_LOADED', 'liboracle' in maps)")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "PRODUCT_LOADED False ORACLE_LOADED True" in r.stdout, r.stdout[-1000:]
