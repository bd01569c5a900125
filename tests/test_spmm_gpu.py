"""tbsla_spmm: Y = A X for k row-major vectors of CSR and COO handles.

Each column of Y against the one-vector product of that vector (bit for bit
for rows of at most 32 entries with TBSLA_TUNE_SHORT_ROWS = 0, the same
stored-order FMA sum) and against the FP64 oracle (|y - y_o| <= 1e-12 *
sum|a x| per row); FP32 / BF16 stores against the FP64 oracle at 2e-6 / 8e-3."""
import numpy as np
import pytest

from conftest import assert_close
from test_spmv_gpu import random_csr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _run(gpu, m, store, X, k, ldx, n_row, dt):
    dev = torch.device("cuda")
    Xd = torch.zeros((X.shape[0], ldx), dtype=dt, device=dev)
    Xd[:, :k] = torch.from_numpy(X).to(dt)
    ldy = ldx + 3
    Yd = torch.full((n_row, ldy), float("nan"), dtype=dt, device=dev)
    m.spmm(store, k, Xd.data_ptr(), ldx, Yd.data_ptr(), ldy)
    torch.cuda.synchronize()
    Y = Yd.cpu().double().numpy()
    assert np.all(np.isnan(Y[:, k:]))  # columns past k untouched
    return Y[:, :k]


def test_spmm_csr_against_single_products_and_oracle(gpu, orc):
    rng = np.random.default_rng(51)
    skew = rng.zipf(1.5, 8000).clip(0, 12000)
    cases = [(6000, 5000, np.full(6000, 16), True), (7001, 3000, rng.integers(0, 33, 7001), True),
             (8000, 8000, skew, False)]
    for (nr, nc, lens, all_short) in cases:
        rp, ci, va = random_csr(rng, nr, nc, lens)
        m = gpu.DeviceMatrix.csr(nr, nc, rp, ci, va, stores=gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16)
        m.tune(gpu.TUNE_SHORT_ROWS, 0)
        o = orc.from_arrays("CSR", nr, nc, va, rp, ci)
        so = orc.from_arrays("CSR", nr, nc, np.abs(va), rp, ci)
        for k in (1, 3, 16, 40):
            X = rng.uniform(-1, 1, (nc, k))
            Y = _run(gpu, m, gpu.F64, X, k, k + (k % 5), nr, torch.float64)
            for c in range(k):
                y1 = m.spmv_host(np.ascontiguousarray(X[:, c]))
                if all_short:
                    assert np.array_equal(Y[:, c], y1), (nr, k, c)
                assert_close(Y[:, c], o.spmv(X[:, c]), so.spmv(np.abs(X[:, c])), 1e-12, f"spmm {nr} k={k} c={c}")
        X = rng.uniform(-1, 1, (nc, 8))
        for store, rtol in ((gpu.F32, 2e-6), (gpu.BF16, 8e-3)):
            Y = _run(gpu, m, store, X, 8, 8, nr, torch.float32)
            for c in range(8):
                assert_close(Y[:, c], o.spmv(X[:, c]), so.spmv(np.abs(X[:, c])), rtol, f"spmm store {store}")


def test_spmm_coo_and_partial_rows(gpu, orc):
    rng = np.random.default_rng(52)
    n_row, n_col, nnz = 3000, 2500, 40000
    row = rng.integers(0, n_row, nnz).astype(np.int32)
    col = rng.integers(0, n_col, nnz).astype(np.int32)
    val = rng.standard_normal(nnz)
    C = gpu.DeviceMatrix.coo(n_row, n_col, row, col, val)
    o = orc.from_arrays("COO", n_row, n_col, val, row, col)
    so = orc.from_arrays("COO", n_row, n_col, np.abs(val), row, col)
    X = rng.uniform(-1, 1, (n_col, 5))
    Y = _run(gpu, C, gpu.F64, X, 5, 5, n_row, torch.float64)
    for c in range(5):
        assert_close(Y[:, c], o.spmv(X[:, c]), so.spmv(np.abs(X[:, c])), 1e-12, "coo spmm")
    # a CSR handle whose kernels visit 100 of 250 rows: the rest are zero
    rp, ci, va = random_csr(rng, 100, 90, rng.integers(0, 20, 100))
    m = gpu.DeviceMatrix.csr(250, 90, rp, ci, va, rows=100)
    m.tune(gpu.TUNE_SHORT_ROWS, 0)
    X = rng.uniform(-1, 1, (90, 4))
    Y = _run(gpu, m, gpu.F64, X, 4, 4, 250, torch.float64)
    assert np.all(Y[100:] == 0)
    for c in range(4):
        assert np.array_equal(Y[:, c], m.spmv_host(np.ascontiguousarray(X[:, c])))


def test_spmm_f32_over_ell_layout_copy(gpu, orc):
    """FP32 panels of a handle with the ELL-layout copy (every row short and
    even, at least 2^16 rows) take sell_spmm_kernel when the panel and the
    leading dimensions are whole float4 runs: each vector summed in stored
    order, so Y equals the CSR-array kernel (TBSLA_TUNE_SHORT_ROWS = 0) bit for
    bit, and the oracle within the FP32 bound; panels of 4, 8 or 12 vectors
    take it, other widths the CSR arrays."""
    rng = np.random.default_rng(53)
    nr = nc = 70000
    lens = np.full(nr, 12)
    lens[rng.choice(nr, 500, replace=False)] = 10
    rp, ci, va = random_csr(rng, nr, nc, lens)
    m = gpu.DeviceMatrix.csr(nr, nc, rp, ci, va, stores=gpu.STORE_F64 | gpu.STORE_F32)
    assert m.info().slices > 0
    o = orc.from_arrays("CSR", nr, nc, va, rp, ci)
    so = orc.from_arrays("CSR", nr, nc, np.abs(va), rp, ci)
    for k, ldx in ((4, 4), (8, 8), (32, 32), (40, 44), (12, 16), (6, 8), (8, 9)):
        X = rng.uniform(-1, 1, (nc, k)).astype(np.float32)
        m.tune(gpu.TUNE_SHORT_ROWS, -1)
        Y = _run(gpu, m, gpu.F32, X, k, ldx, nr, torch.float32)
        m.tune(gpu.TUNE_SHORT_ROWS, 0)
        Y0 = _run(gpu, m, gpu.F32, X, k, ldx, nr, torch.float32)
        assert np.array_equal(Y, Y0), (k, ldx)
        for c in (0, k - 1):
            xc = X[:, c].astype(np.float64)
            assert_close(Y[:, c], o.spmv(xc), so.spmv(np.abs(xc)), 2e-6, f"sliced spmm k={k} c={c}")
    m.tune(gpu.TUNE_SHORT_ROWS, -1)
