"""Files straight into device handles (tbsla_matrix_read_file,
tbsla_matrix_read_mm).

Binary files are written in the reference's layout (Matrix*::write,
MatrixCSR.cpp:179-204 and siblings) by the oracle's writer; two matrices
share one file and the second is read at its byte offset, as
C_CPP_Matrix*_read's `seek` does.  The loaded handle must give the same
product, bit for bit, as a handle created from the same arrays.  Matrix
Market files (general and symmetric, as MatrixCOO::readMM reads them) are
checked against a dense numpy product; other kinds are refused.
"""
import numpy as np
import pytest

from oracle.oracle import Arrays, write_binary

pytestmark = pytest.mark.gpu
FORMATS = ["COO", "SCOO", "CSR", "ELL", "DENSE"]


def _arrays(g):
    n_row, n_col, ln_row, ln_col, f_row, f_col, pr, pc, NR, NC, max_col = g.geom
    return Arrays(g.fmt, n_row, n_col, ln_row, ln_col, f_row, f_col, g.nnz, pr, pc, NR, NC, max_col,
                  g.values, g.idx0, g.idx1)


@pytest.mark.parametrize("fmt", FORMATS)
def test_binary_file_into_device(gpu, tmp_path, fmt):
    n = 900 if fmt == "DENSE" else 20000
    g1 = gpu.generate(fmt, "cqmat", n, n, 9, 0.1, 2)
    g2 = gpu.generate(fmt, "cdiag", n, n, 3, 0.0, 1)
    first = write_binary(_arrays(g1))
    path = tmp_path / f"m_{fmt}.bin"
    path.write_bytes(first + write_binary(_arrays(g2)))
    x = np.random.default_rng(1).uniform(-1, 1, n)
    for g, seek in ((g1, 0), (g2, len(first))):
        A = gpu.DeviceMatrix.read_file(str(path), fmt, seek)
        B = gpu.DeviceMatrix.from_generated(g)
        assert np.array_equal(A.spmv_host(x), B.spmv_host(x))


def test_matrix_market_into_device(gpu, tmp_path):
    rng = np.random.default_rng(4)
    nr, nc, nv = 300, 200, 2500
    r, c = rng.integers(1, nr + 1, nv), rng.integers(1, nc + 1, nv)
    v = rng.uniform(-1, 1, nv)
    gen = tmp_path / "g.mtx"
    gen.write_text("%%MatrixMarket matrix coordinate real general\n% a comment\n"
                   + f"{nr} {nc} {nv}\n" + "".join(f"{a} {b} {float(w)!r}\n" for a, b, w in zip(r, c, v)))
    dense = np.zeros((nr, nc))
    np.add.at(dense, (r - 1, c - 1), v)
    x = rng.uniform(-1, 1, nc)
    for fmt in FORMATS:
        A = gpu.DeviceMatrix.read_mm(str(gen), fmt)
        assert np.allclose(A.spmv_host(x), dense @ x, rtol=1e-12, atol=1e-12), fmt
    # symmetric: the mirror of each off-diagonal entry is added
    n = 150
    rs, cs = rng.integers(1, n + 1, 800), rng.integers(1, n + 1, 800)
    lo = rs >= cs
    rs, cs = rs[lo], cs[lo]
    vs = rng.uniform(-1, 1, rs.size)
    sym = tmp_path / "s.mtx"
    sym.write_text("%%MatrixMarket matrix coordinate real symmetric\n"
                   + f"{n} {n} {rs.size}\n" + "".join(f"{a} {b} {float(w)!r}\n" for a, b, w in zip(rs, cs, vs)))
    ds = np.zeros((n, n))
    np.add.at(ds, (rs - 1, cs - 1), vs)
    off = rs != cs
    np.add.at(ds, (cs[off] - 1, rs[off] - 1), vs[off])
    xs = rng.uniform(-1, 1, n)
    A = gpu.DeviceMatrix.read_mm(str(sym), "CSR")
    assert np.allclose(A.spmv_host(xs), ds @ xs, rtol=1e-12, atol=1e-12)
    arr = tmp_path / "a.mtx"
    arr.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(gpu.TbslaError) as e:
        gpu.DeviceMatrix.read_mm(str(arr), "CSR")
    assert e.value.status == 6  # TBSLA_ERR_UNSUPPORTED
