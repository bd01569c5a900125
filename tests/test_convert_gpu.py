"""Device-side COO -> CSR conversion (tbsla_coo_to_csr) against the oracle's
restatement of MatrixCSR(const MatrixCOO&) (MatrixCSR.cpp:29-74, entries by
(row, column), equal pairs in input order): rowptr, colidx and values bit for
bit, on unsorted triplets with repeated (row, column) pairs, empty rows, and
the cqmat matrix at 2^22."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(gpu, orc, n_row, n_col, row, col, val):
    C = gpu.DeviceMatrix.coo(n_row, n_col, row, col, val)
    A = C.to_csr()
    rp, ci, va = A.csr_download()
    o = orc.from_arrays("COO", n_row, n_col, val, row, col).convert("CSR").arrays
    assert np.array_equal(rp, o.idx0)
    assert np.array_equal(ci, o.idx1)
    assert np.array_equal(va, o.values)
    x = np.random.default_rng(0).uniform(-1, 1, n_col)
    B = gpu.DeviceMatrix.csr(n_row, n_col, o.idx0, o.idx1, o.values)
    assert np.array_equal(A.spmv_host(x), B.spmv_host(x))


def test_coo_to_csr_small_cases(gpu, orc):
    rng = np.random.default_rng(12)
    for (nr, nc, nnz) in [(1, 1, 1), (10, 7, 0), (50, 40, 300), (3000, 5000, 60000), (200, 100000, 40000)]:
        row = rng.integers(0, nr, nnz).astype(np.int32)
        col = rng.integers(0, nc, nnz).astype(np.int32)
        if nnz > 10:
            row[-5:], col[-5:] = row[0], col[0]  # the same (row, col) several times
        val = rng.standard_normal(nnz)
        _check(gpu, orc, nr, nc, row, col, val)


def test_coo_to_csr_cqmat_2p22(gpu, orc):
    n = 1 << 22
    g = gpu.generate("COO", "cqmat", n, n, 16, 0.1, 0)
    _check(gpu, orc, n, n, g.idx0, g.idx1, g.values)
