"""Multi-vector DENSE product (tbsla_dense_spmm) against the oracle's k
DENSE products (MatrixDENSE::Ax, src/cpp/matrix/MatrixDENSE.cpp:64-73).

The F32 and BF16 stores run on the tensor cores (the library's tcgen05
kernel): TF32 within 4e-3 and BF16 within 1.2e-2 of sum_j |a_ij x_jc| (the
operands' rounding: 2^-10 / 2^-8 relative each, plus FP32 accumulation); the
BF16 result also against the FP64 product of the rounded operands within
K * 2^-23 of the same sum (accumulation error only).  F64 (FP64 pipe) within
the FP64 bound of the product tests.  Shapes cover row tiles cut by the
matrix edge, K not a multiple of the 128-byte stage, unaligned leading
dimensions (padded copies), one to several vector panels, rows past ln_row
(zero), every K split, and the same bits on a repeated call.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SHAPES = [
    # n_row, ln_row, ln_col, k, ldx, ldy
    (800, 700, 500, 16, 512, 808),
    (1000, 1000, 1024, 64, 1024, 1000),
    (300, 257, 333, 5, 340, 300),
    (256, 256, 2048, 100, 2050, 260),
    (130, 130, 4096, 300, 4096, 130),
    (128, 128, 64, 1, 64, 128),
]


def bf16_round(a):
    """Round-to-nearest-even of each value to BF16 (8 significant bits) in one
    step, as the device's BF16 store (from FP64) and X copy (from FP32) do:
    the significand scaled to 8 bits, rounded half to even, scaled back (all
    exact in FP64)."""
    m, e = np.frexp(np.asarray(a, np.float64))
    return np.ldexp(np.rint(m * 256.0) / 256.0, e)


def oracle_products(orc, a, x, n_row):
    """Column c = the oracle's MatrixDENSE product of vector c (rows past
    ln_row are 0)."""
    ln_row, ln_col = a.shape
    geom = [n_row, ln_col, ln_row, ln_col, 0, 0, 0, 0, 1, 1, 0]
    m = orc.from_layout("DENSE", geom, a.size, a.ravel(), np.zeros(0, np.int32), np.zeros(0, np.int32))
    return np.stack([m.spmv(x[:, c]) for c in range(x.shape[1])], axis=1)


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_dense_multi_vector_against_oracle(gpu, orc, shape):
    n_row, ln_row, ln_col, k, ldx, ldy = shape
    rng = np.random.default_rng(hash(shape) % 2**32)
    a = rng.uniform(-1, 1, (ln_row, ln_col))
    A = gpu.DeviceMatrix.dense(n_row, ln_col, ln_row, ln_col, a.ravel(),
                               stores=gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16)
    x = rng.uniform(-1, 1, (ln_col, k))
    ref = oracle_products(orc, a, x, n_row)
    bound = oracle_products(orc, np.abs(a), np.abs(x), n_row)
    ar, xr = bf16_round(a), bf16_round(x.astype(np.float32))
    ref_r = oracle_products(orc, ar, xr, n_row)
    dev = torch.device("cuda")
    for store, tdt, tol in ((gpu.F64, torch.float64, 1e-12), (gpu.F32, torch.float32, 4e-3),
                            (gpu.BF16, torch.float32, 1.2e-2)):
        X = torch.zeros((k, ldx), dtype=tdt, device=dev)  # vector c at X[c, :ln_col]
        X[:, :ln_col] = torch.from_numpy(x.T.copy()).to(dev, tdt)
        splits = (0,) if store == gpu.F64 else (0, 1, 2, 4)
        for split in splits:
            A.tune(gpu.TUNE_TC_SPLIT, split)
            outs = []
            for _ in range(2):
                Y = torch.full((k, ldy), float("nan"), dtype=tdt, device=dev)
                A.dense_spmm(store, k, X.data_ptr(), ldx, Y.data_ptr(), ldy)
                torch.cuda.synchronize()
                outs.append(Y[:, :n_row].double().cpu().numpy().T)
            y = outs[0]
            assert np.array_equal(outs[0], outs[1]), (store, split, "results differ between two calls")
            err = np.abs(y - ref)
            assert np.all(err <= tol * bound + 1e-300), (store, split, float((err / (bound + 1e-300)).max()))
            assert np.all(y[ln_row:] == 0)
            if store == gpu.BF16:
                err_r = np.abs(y - ref_r)
                assert np.all(err_r <= ln_col * 2.0 ** -23 * bound + 1e-300), (split, float(err_r.max()))
            # the columns past n_row of Y are not written
            Yfull = Y.cpu()
            if ldy > n_row:
                assert torch.isnan(Yfull[:, n_row:]).all()
    assert A.device_status() == 0


def test_dense_multi_vector_splits_agree(gpu):
    """Every K split (1 to 16 parts of an 8192-long sum) is within the FP32
    accumulation bound K * 2^-23 * sum |a x| of the FP64 product of the
    BF16-rounded operands."""
    rng = np.random.default_rng(3)
    n, K, k = 512, 8192, 64
    a = rng.uniform(0, 1, (n, K))
    A = gpu.DeviceMatrix.dense(n, K, n, K, a.ravel(), stores=gpu.STORE_BF16 | gpu.STORE_F64)
    x = rng.uniform(0, 1, (k, K)).astype(np.float32)
    X = torch.from_numpy(x).cuda()
    ref = bf16_round(a) @ bf16_round(x).T  # n x k, all terms positive: sum |a x| = ref
    for split in (1, 2, 4, 8, 16):
        A.tune(gpu.TUNE_TC_SPLIT, split)
        Y = torch.empty((k, n), dtype=torch.float32, device="cuda")
        A.dense_spmm(gpu.BF16, k, X.data_ptr(), K, Y.data_ptr(), n)
        torch.cuda.synchronize()
        y = Y.double().cpu().numpy().T
        err = float((np.abs(y - ref) / ref).max())
        assert err <= K * 2.0 ** -23, (split, err)
    assert A.device_status() == 0
