"""The driver programs (tbsla_gb300/apps, built into tbsla_gb300/bin) on the
GPU: tbsla_page_rank with the reference driver's flags
(src/cpp/apps/tbsla_page_rank.cpp:17-82) on a Matrix Market file, its
iteration count and vector against the oracle's Matrix::page_rank of the same
COO matrix; tbsla_perf with the reference's flags
(src/cpp/apps/tbsla_perf.cpp:27-194), its report carrying the reference's keys
plus the GPU figures."""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(capi, name, args):
    from tbsla_gb300 import build
    exe = build.app_path(name)
    assert os.path.exists(exe), exe
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = r.stdout.splitlines()
    return lines, json.loads([ln for ln in lines if ln.startswith("{")][-1])


def _write_mm(path, n, rows, cols, vals):
    with open(path, "w") as fh:
        fh.write("%%MatrixMarket matrix coordinate real general\n")
        fh.write(f"{n} {n} {len(vals)}\n")
        for r, c, v in zip(rows, cols, vals):
            fh.write(f"{int(r) + 1} {int(c) + 1} {float(v)!r}\n")


@pytest.mark.parametrize("fmt", ["COO", "CSR", "ELL"])
def test_page_rank_driver_against_oracle(gpu, orc, tmp_path, fmt):
    n = 3000
    g = gpu.generate("COO", "cqmat_stochastic", n, n, 9, 0.2, 4)
    path = str(tmp_path / "m.mtx")
    _write_mm(path, n, g.idx0, g.idx1, g.values)
    lines, rep = _run(gpu, "tbsla_page_rank", ["--matrix_input", path, "--beta", "0.85", "--epsilon", "1e-9",
                                              "--max-iterations", "500", "--format", fmt])
    # the oracle of the same format: MatrixCOO as read, or its conversion
    o = orc.from_arrays("COO", n, n, g.values, g.idx0, g.idx1)
    o.update_nnz()
    if fmt != "COO":
        o = o.convert(fmt)
    b, it = o.page_rank(1e-9, 0.85, 500)
    assert int(rep["nb_iterations"]) == it, (rep["nb_iterations"], it)
    assert rep["test"] == "page_rank" and rep["matrix_format"] == fmt and int(rep["n"]) == n
    assert int(rep["nnz"]) == g.values.size
    for key in ("time_read_m", "time_page_rank", "time_app", "lang", "matrix_input", "device"):
        assert key in rep
    sol = [ln for ln in lines if ln.startswith("SOLUTION")][0]
    printed = [float(t) for t in sol[sol.index("[") + 1:sol.index("]")].split(",") if t.strip()]
    assert np.allclose(printed, b[:4], rtol=1e-5)
    # personalised
    _, rep = _run(gpu, "tbsla_page_rank", ["--matrix_input", path, "--beta", "0.85", "--epsilon", "1e-9",
                                           "--max-iterations", "500", "--format", fmt, "--personalized", "1,5,5,77"])
    _, it = o.personalized_page_rank(1e-9, 0.85, 500, [1, 5, 5, 77])
    assert rep["test"] == "personalized_page_rank" and int(rep["nb_iterations"]) == it


@pytest.mark.parametrize("fmt,op", [("CSR", "spmv"), ("ELL", "a_axpx"), ("COO", "Ax"), ("DENSE", "spmv")])
def test_perf_driver_report(gpu, fmt, op):
    n = 2000 if fmt == "DENSE" else 100000
    _, rep = _run(gpu, "tbsla_perf", ["--format", fmt, "--matrix", "cqmat", "--NR", str(n), "--NC", str(n),
                                      "--C", "10", "--Q", "0.1", "--S", "0", "--op", op, "--reps", "5"])
    reference_keys = {"test", "matrix_format", "n_row", "n_col", "nnz", "time_app_in", "time_op", "gflops", "lang",
                      "matrix_type", "compiler", "compile_options", "cqmat_c", "cqmat_q", "cqmat_s"}
    assert reference_keys <= set(rep), reference_keys - set(rep)
    assert rep["test"] == op and int(rep["n_row"]) == n and rep["matrix_type"] == "cqmat"
    for key in ("time_op", "time_op_device", "gbps", "gbps_device", "peak_gbs", "roofline_frac"):
        assert float(rep[key]) > 0, (key, rep[key])
    assert float(rep["roofline_frac"]) < 1.5
