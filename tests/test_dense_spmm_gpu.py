"""Multi-vector DENSE product (tbsla_dense_spmm, cuBLAS GEMM) against numpy:
FP64 within the FP64 bound of the product tests, FP32 within 1e-5 and the
BF16 store (tensor cores, inputs rounded to BF16) within 1e-2 of
sum |a_ij x_jc|; leading dimensions larger than the shapes; rows past ln_row
give 0."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_dense_multi_vector(gpu):
    rng = np.random.default_rng(6)
    n_row, ln_row, ln_col, k, ldx, ldy = 800, 700, 500, 16, 512, 808
    a = rng.uniform(-1, 1, (ln_row, ln_col))
    A = gpu.DeviceMatrix.dense(n_row, ln_col, ln_row, ln_col, a.ravel(),
                               stores=gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16)
    x = rng.uniform(-1, 1, (ln_col, k))
    ref = np.zeros((n_row, k))
    ref[:ln_row] = a @ x
    bound = np.zeros((n_row, k))
    bound[:ln_row] = np.abs(a) @ np.abs(x)
    dev = torch.device("cuda")
    for store, tdt, tol in ((gpu.F64, torch.float64, 1e-12), (gpu.F32, torch.float32, 1e-5),
                            (gpu.BF16, torch.float32, 1e-2)):
        X = torch.zeros((k, ldx), dtype=tdt, device=dev)  # column c at X[c, :]
        X[:, :ln_col] = torch.from_numpy(x.T.copy()).to(dev, tdt)
        Y = torch.full((k, ldy), float("nan"), dtype=tdt, device=dev)
        A.dense_spmm(store, k, X.data_ptr(), ldx, Y.data_ptr(), ldy)
        torch.cuda.synchronize()
        y = Y[:, :n_row].double().cpu().numpy().T
        assert np.all(np.abs(y - ref) <= tol * bound + 1e-300), store
        assert np.all(y[ln_row:] == 0)
