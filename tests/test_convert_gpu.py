"""Device-side conversions of COO handles against the oracle's restatements:
CSR (tbsla_coo_to_csr, MatrixCSR(const MatrixCOO&), MatrixCSR.cpp:29-74,
entries by (row, column), equal pairs in input order), ELL and DENSE
(tbsla_coo_to_ell / tbsla_coo_to_dense): arrays bit for bit, on unsorted
triplets with repeated (row, column) pairs, empty rows, and the cqmat matrix
at 2^22."""
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


def _check_ell_dense(gpu, orc, n_row, n_col, row, col, val):
    """Device ELL / DENSE conversions against the oracle's restatement of
    MatrixELL(COO) (MatrixELL.cpp:12-53) and MatrixDENSE(COO)
    (MatrixDENSE.cpp:11-28): arrays bit for bit, and products equal to
    handles built on the host from the oracle's arrays."""
    C = gpu.DeviceMatrix.coo(n_row, n_col, row, col, val)
    o = orc.from_arrays("COO", n_row, n_col, val, row, col)
    x = np.random.default_rng(1).uniform(-1, 1, n_col)
    E = C.to_ell(stores=gpu.STORE_F64 | gpu.STORE_F32)
    oe = o.convert("ELL").arrays
    assert E.info().max_col == oe.max_col
    cols, vals = E.ell_download()
    assert np.array_equal(cols, oe.idx0[: cols.size]) and cols.size == oe.idx0.size
    assert np.array_equal(vals, oe.values[: vals.size]) and vals.size == oe.values.size
    H = gpu.DeviceMatrix.ell(n_row, n_col, oe.max_col, oe.idx0, oe.values)
    assert np.array_equal(E.spmv_host(x), H.spmv_host(x)), "ELL product"
    D = C.to_dense()
    od = o.convert("DENSE").arrays
    dv = D.dense_download()
    assert dv.size == od.values.size and np.array_equal(dv.view(np.int64), od.values.view(np.int64))
    assert np.array_equal(D.spmv_host(x), gpu.DeviceMatrix.dense(n_row, n_col, n_row, n_col, od.values).spmv_host(x))


def test_coo_to_ell_and_dense(gpu, orc):
    rng = np.random.default_rng(21)
    for (nr, nc, nnz) in [(1, 1, 1), (10, 7, 0), (50, 40, 300), (3000, 500, 60000), (997, 2000, 5000)]:
        row = rng.integers(0, nr, nnz).astype(np.int32)
        col = rng.integers(0, nc, nnz).astype(np.int32)
        if nnz > 10:
            row[-5:], col[-5:] = row[0], col[0]  # repeated (row, col): DENSE adds them in input order
        val = rng.standard_normal(nnz)
        if nnz > 10:
            val[-1] = -0.0
        _check_ell_dense(gpu, orc, nr, nc, row, col, val)
