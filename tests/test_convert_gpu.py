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


def test_coo_to_scoo_copy(gpu, orc):
    """MatrixSCOO(COO) copies the arrays: the device copy gives the same
    products (every kernel variant, row shifts) as the COO handle."""
    rng = np.random.default_rng(5)
    n_row, n_col, nnz = 3000, 2000, 40000
    row = rng.integers(0, n_row, nnz).astype(np.int32)
    col = rng.integers(0, n_col, nnz).astype(np.int32)
    val = rng.standard_normal(nnz)
    C = gpu.DeviceMatrix.coo(n_row, n_col, row, col, val)
    S = C.to_scoo(stores=gpu.STORE_F64 | gpu.STORE_F32)
    i, j = C.info(), S.info()
    assert (i.n_row, i.n_col, i.stored) == (j.n_row, j.n_col, j.stored)
    x = rng.uniform(-1, 1, n_col)
    for v in (0, 1):
        C.set_variant(v)
        S.set_variant(v)
        for incr in (0, 2):
            assert np.array_equal(C.spmv_host(x, incr), S.spmv_host(x, incr)), f"variant {v} shift {incr}"


def test_csr_normalize_columns(gpu, orc):
    """MatrixCSR::normalize_columns on the device: values bit-identical to the
    oracle's restatement (column sums in the reference's loop order), the
    derived FP32 store and the transposed copy refreshed."""
    rng = np.random.default_rng(6)
    for (nr, nc, nnz) in [(1, 1, 1), (500, 300, 4000), (20000, 15000, 300000)]:
        row = np.sort(rng.integers(0, nr, nnz)).astype(np.int64)
        rp = np.zeros(nr + 1, np.int64)
        np.add.at(rp, row + 1, 1)
        rp = np.cumsum(rp).astype(np.int32)
        ci = rng.integers(0, nc, nnz).astype(np.int32)
        va = rng.uniform(0.1, 2.0, nnz)
        m = gpu.DeviceMatrix.csr(nr, nc, rp, ci, va, stores=gpu.STORE_F64 | gpu.STORE_F32)
        m.spmv_host(rng.uniform(-1, 1, nc))
        m.normalize_columns()
        o = orc.from_arrays("CSR", nr, nc, va, rp, ci)
        o.normalize_columns()
        ov = o.arrays.values
        _, _, got = m.csr_download()
        assert np.array_equal(got.view(np.int64), ov.view(np.int64))
        B = gpu.DeviceMatrix.csr(nr, nc, rp, ci, ov)
        xc = rng.uniform(-1, 1, nc)
        assert np.array_equal(m.spmv_host(xc), B.spmv_host(xc))


def _device_vs_oracle(gpu, orc, fmt, gen, nr, nc, c, q, s, blk):
    """A handle from tbsla_generate_device against the oracle's fill of the
    same block: the arrays bit for bit, and the same info as the handle the
    host arrays give."""
    A = gpu.DeviceMatrix.generate_device(fmt, gen, nr, nc, c, q, s, *blk)
    fill = {"cdiag": lambda: orc.fill_cdiag(fmt, nr, nc, c, *blk),
            "cqmat_stochastic": lambda: orc.fill_cqmat_stochastic(fmt, nr, nc, c, q, s, *blk)}[gen]
    a = fill().arrays
    H = gpu.DeviceMatrix.from_generated(gpu.generate(fmt, gen, nr, nc, c, q, s, *blk))
    i, h = A.info(), H.info()
    tag = (fmt, gen, nr, nc, c, q, s, blk)
    assert (i.n_row, i.n_col, i.f_col, i.rows, i.max_col, i.stored) == \
        (h.n_row, h.n_col, h.f_col, h.rows, h.max_col, h.stored), tag
    if fmt == "CSR":
        rp, ci, va = A.csr_download()
        if a.values.size:
            assert np.array_equal(rp, a.idx0) and np.array_equal(ci, a.idx1), tag
        assert np.array_equal(va, a.values), tag
    elif fmt == "ELL":
        cols, vals = A.ell_download()
        assert np.array_equal(cols, a.idx0[: cols.size]) and np.array_equal(vals, a.values[: vals.size]), tag
    else:
        assert np.array_equal(A.dense_download(), a.values), tag
    x = np.random.default_rng(1).uniform(-1, 1, nc)
    assert np.array_equal(A.spmv_host(x), H.spmv_host(x)), tag


@pytest.mark.parametrize("fmt", ["CSR", "ELL", "DENSE"])
def test_device_generators_match_oracle(gpu, orc, fmt):
    """fill_cdiag generated on the device and fill_cqmat_stochastic divided on
    the device (tbsla_generate_device) give the reference's arrays for whole
    matrices and blocks, square and not."""
    blocks = [(0, 0, 1, 1), (1, 0, 2, 1), (0, 1, 1, 2), (1, 2, 3, 4)]
    for (nr, nc) in [(30, 30), (50, 20), (20, 50), (1, 1)]:
        for blk in blocks:
            for c in (0, 1, 3, 25):
                _device_vs_oracle(gpu, orc, fmt, "cdiag", nr, nc, c, 0.0, 0, blk)
            for (c, q, s) in [(5, 0.1, 1), (8, 0.5, 3)]:
                _device_vs_oracle(gpu, orc, fmt, "cqmat_stochastic", nr, nc, c, q, s, blk)
    if fmt == "CSR":
        # the format sweep's cdiag case at 2^26 rows and a 2^20 stochastic matrix
        n = 1 << 26
        A = gpu.DeviceMatrix.generate_device("CSR", "cdiag", n, n, 1)
        rp, ci, va = A.csr_download()
        assert rp[-1] == 2 * n - 2 and np.all(va == 1.0)
        assert np.array_equal(rp[:4], [0, 1, 3, 5]) and np.array_equal(ci[:5], [1, 0, 2, 1, 3])
        assert ci[-1] == n - 2
        _device_vs_oracle(gpu, orc, "CSR", "cqmat_stochastic", 1 << 20, 1 << 20, 16, 0.1, 0, (0, 0, 1, 1))
