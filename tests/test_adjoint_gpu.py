"""Differentiation on the GPU: the transposed product, the values gradient,
value replacement, the teleport-form PageRank and its adjoint, the
torch.autograd shim.

Oracles: scipy/numpy for the products (A^T x, a[row]*b[col]); the FP64 CPU
restatement oracle/tbsla_oracle.c (orc_pagerank_teleport,
orc_pagerank_adjoint) for the fixed point and its gradients; central finite
differences of the oracle's forward solve on 1000 random edges and 50
teleport entries, to 1e-6 relative; torch.autograd.gradcheck through the GPU
forward for the shim.
"""
import math

import numpy as np
import pytest

from test_pagerank_gpu import rmat_csr_oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _random_csr(rng, n_row, n_col):
    """Row lengths from 0 to 12000: every bin (thread per row, the four lane
    groups, chunked huge rows) is used; repeated columns allowed."""
    lens = rng.integers(0, 33, n_row)
    lens[::97] = rng.integers(33, 97, lens[::97].size)
    lens[5::101] = rng.integers(97, 257, lens[5::101].size)
    lens[7::211] = rng.integers(257, 1025, lens[7::211].size)
    lens[11] = 5000
    lens[13] = 12000
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    ci = rng.integers(0, n_col, rp[-1]).astype(np.int32)
    return rp, ci


def test_transpose_product_and_values_gradient(gpu):
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(5)
    n_row, n_col = 3000, 20000
    rp, ci = _random_csr(rng, n_row, n_col)
    vals = rng.uniform(-1, 1, rp[-1])
    A = gpu.DeviceMatrix.csr(n_row, n_col, rp, ci, vals, stores=gpu.STORE_F64 | gpu.STORE_F32)
    S = sp.csr_matrix((vals, ci, rp), shape=(n_row, n_col))
    Sabs = sp.csr_matrix((np.abs(vals), ci, rp), shape=(n_row, n_col))
    gy = rng.uniform(-1, 1, n_row)
    x = rng.uniform(-1, 1, n_col)
    dev = torch.device("cuda")
    tgy, tx = torch.from_numpy(gy).to(dev), torch.from_numpy(x).to(dev)
    out = torch.empty(n_col, dtype=torch.float64, device=dev)
    A.spmv_transpose_ex(gpu.F64, gpu.F64, tgy.data_ptr(), gpu.F64, out.data_ptr())
    torch.cuda.synchronize()
    ref = S.T @ gy
    bound = Sabs.T @ np.abs(gy)
    assert np.all(np.abs(out.cpu().numpy() - ref) <= 1e-12 * bound)
    gv = torch.empty(vals.size, dtype=torch.float64, device=dev)
    A.grad_values(gpu.F64, tgy.data_ptr(), tx.data_ptr(), 1.0, gv.data_ptr())
    torch.cuda.synchronize()
    rows = np.repeat(np.arange(n_row), np.diff(rp))
    assert np.array_equal(gv.cpu().numpy(), gy[rows] * x[ci])  # bit-exact
    # FP32 (the inputs stay referenced until the kernel has run)
    gy32, x32 = tgy.float(), tx.float()
    gv32 = torch.empty(vals.size, dtype=torch.float32, device=dev)
    A.grad_values(gpu.F32, gy32.data_ptr(), x32.data_ptr(), 2.0, gv32.data_ptr())
    torch.cuda.synchronize()
    exp32 = (np.float32(2.0) * gy.astype(np.float32)[rows]) * x.astype(np.float32)[ci]
    assert np.array_equal(gv32.cpu().numpy(), exp32)
    # new values reach the product and the transposed copy
    new = rng.uniform(0, 2, vals.size)
    tnew = torch.from_numpy(new).to(dev)
    A.set_values(gpu.F64, tnew.data_ptr())
    S2 = sp.csr_matrix((new, ci, rp), shape=(n_row, n_col))
    y = A.spmv_host(x)
    assert np.allclose(y, S2 @ x, rtol=1e-12, atol=1e-12)
    A.spmv_transpose_ex(gpu.F64, gpu.F64, tgy.data_ptr(), gpu.F64, out.data_ptr())
    torch.cuda.synchronize()
    assert np.allclose(out.cpu().numpy(), S2.T @ gy, rtol=1e-12, atol=1e-12)


def test_values_gradient_all_short_rows(gpu):
    """Every row short (the warp-segment kernel): bit-exact in FP64 and FP32,
    including empty rows and a row count that is not a multiple of 32."""
    rng = np.random.default_rng(9)
    n_row, n_col = 100003, 7000
    lens = rng.integers(0, 20, n_row)
    lens[::7] = 0
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    ci = rng.integers(0, n_col, rp[-1]).astype(np.int32)
    vals = rng.uniform(-1, 1, rp[-1])
    A = gpu.DeviceMatrix.csr(n_row, n_col, rp, ci, vals, stores=gpu.STORE_F64 | gpu.STORE_F32)
    rows = np.repeat(np.arange(n_row), lens)
    dev = torch.device("cuda")
    gy, x = rng.uniform(-1, 1, n_row), rng.uniform(-1, 1, n_col)
    tgy, tx = torch.from_numpy(gy).to(dev), torch.from_numpy(x).to(dev)
    gv = torch.full((vals.size,), float("nan"), dtype=torch.float64, device=dev)
    A.grad_values(gpu.F64, tgy.data_ptr(), tx.data_ptr(), 1.0, gv.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(gv.cpu().numpy(), gy[rows] * x[ci])
    gy32, x32 = tgy.float(), tx.float()
    gv32 = torch.full((vals.size,), float("nan"), dtype=torch.float32, device=dev)
    A.grad_values(gpu.F32, gy32.data_ptr(), x32.data_ptr(), 0.5, gv32.data_ptr())
    torch.cuda.synchronize()
    exp32 = (np.float32(0.5) * gy.astype(np.float32)[rows]) * x.astype(np.float32)[ci]
    assert np.array_equal(gv32.cpu().numpy(), exp32)


def _rmat(gpu, orc, scale, seed):
    m = 16 << scale
    A = gpu.DeviceMatrix.rmat_pagerank(scale, m, seed=seed)
    rp, ci, va, dang = rmat_csr_oracle(orc, scale, m, seed)
    return A, rp, ci, va, dang


@pytest.mark.parametrize("uniform,accel", [(True, 0), (False, 0), (False, 1)])
def test_teleport_pagerank_and_adjoint_match_oracle(gpu, orc, uniform, accel):
    A, rp, ci, va, dang = _rmat(gpu, orc, 12, 4)
    n = rp.size - 1
    rng = np.random.default_rng(2)
    v = np.full(n, 1.0 / n) if uniform else rng.uniform(0.5, 1.5, n) / n
    w = rng.standard_normal(n)
    dev = torch.device("cuda")
    tv, tw = torch.from_numpy(v).to(dev), torch.from_numpy(w).to(dev)
    x = torch.empty(n, dtype=torch.float64, device=dev)
    r = A.pagerank_teleport(tv.data_ptr(), x.data_ptr(), 0.85, 1e-15, 2000, accel=accel)
    assert r.converged
    xo, _, _ = orc.pagerank_teleport(rp, ci, va, dang, v, 0.85, 0.0, 400)
    assert np.abs(x.cpu().numpy() - xo).sum() < 1e-13
    if uniform:
        # for a column-stochastic matrix the teleport form is the dangling mode
        xd, _ = A.pagerank_host(tol=1e-15, max_iter=2000, mode=gpu.PR_DANGLING)
        assert np.abs(xd - x.cpu().numpy()).sum() < 1e-13
    gvals = torch.empty(va.size, dtype=torch.float64, device=dev)
    gv = torch.empty(n, dtype=torch.float64, device=dev)
    # lambda is O(1) per entry: an L1 tolerance of n * 1e-15
    ra = A.pagerank_adjoint(tv.data_ptr(), x.data_ptr(), tw.data_ptr(), gvals.data_ptr(), gv.data_ptr(), 0.85,
                            n * 1e-15, 3000, accel=accel)
    assert ra.converged
    go_vals, go_v, _ = orc.pagerank_adjoint(rp, ci, va, dang, v, xo, w, 0.85, 0.0, 400)
    assert np.max(np.abs(gvals.cpu().numpy() - go_vals)) <= 1e-10 * np.max(np.abs(go_vals))
    assert np.max(np.abs(gv.cpu().numpy() - go_v)) <= 1e-10 * np.max(np.abs(go_v))


def test_adjoint_against_finite_differences(gpu, orc):
    """1000 random edges and 50 teleport entries, finite differences of the
    oracle's forward solve, relative error <= 1e-6.  The differences are
    fourth order (Richardson: (8(f(h)-f(-h)) - (f(2h)-f(-2h))) / 12h) with
    h = 3e-3 of the entry: the loss carries ~1e-16 of rounding, so a small
    step would drown small gradients in noise."""
    A, rp, ci, va, dang = _rmat(gpu, orc, 10, 6)
    n = rp.size - 1
    v = np.full(n, 1.0 / n)
    w = np.random.default_rng(2).standard_normal(n)
    dev = torch.device("cuda")
    tv, tw = torch.from_numpy(v).to(dev), torch.from_numpy(w).to(dev)
    x = torch.empty(n, dtype=torch.float64, device=dev)
    A.pagerank_teleport(tv.data_ptr(), x.data_ptr(), 0.85, 0.0, 400)
    gvals = torch.empty(va.size, dtype=torch.float64, device=dev)
    gv = torch.empty(n, dtype=torch.float64, device=dev)
    A.pagerank_adjoint(tv.data_ptr(), x.data_ptr(), tw.data_ptr(), gvals.data_ptr(), gv.data_ptr(), 0.85, 0.0, 400)
    gvals, gv = gvals.cpu().numpy(), gv.cpu().numpy()

    def loss(vals, vv):
        xx, _, _ = orc.pagerank_teleport(rp, ci, vals, dang, vv, 0.85, 0.0, 260)
        return math.fsum(w * xx)

    def fd4(f, base, idx):
        h = 3e-3 * base[idx]
        out = []
        for s in (1, -1, 2, -2):
            b = base.copy()
            b[idx] += s * h
            out.append(f(b))
        return (8 * (out[0] - out[1]) - (out[2] - out[3])) / (12 * h)

    rng = np.random.default_rng(7)
    worst = 0.0
    for k in rng.choice(va.size, 1000, replace=False):
        fd = fd4(lambda b: loss(b, v), va, k)
        worst = max(worst, abs(gvals[k] - fd) / max(abs(fd), 1e-300))
    assert worst <= 1e-6, worst
    worst = 0.0
    for i in rng.choice(n, 50, replace=False):
        fd = fd4(lambda b: loss(va, b), v, i)
        worst = max(worst, abs(gv[i] - fd) / max(abs(fd), 1e-300))
    assert worst <= 1e-6, worst


def test_autograd_shim_gradcheck(gpu, orc):
    from tbsla_gb300 import autograd as ag
    dev = torch.device("cuda")
    # SpMV, FP64
    g = gpu.generate("CSR", "cqmat", 40, 30, 6, 0.3, 2)
    A = gpu.DeviceMatrix.csr(40, 30, g.idx0, g.idx1, g.values, stores=gpu.STORE_F64 | gpu.STORE_F32)
    vals = torch.rand(g.values.size, dtype=torch.float64, device=dev, requires_grad=True)
    x = torch.rand(30, dtype=torch.float64, device=dev, requires_grad=True)
    assert torch.autograd.gradcheck(lambda a, b: ag.csr_spmv(A, a, b), (vals, x), eps=1e-6, atol=1e-9, rtol=1e-7)
    # SpMV, FP32 backward against the FP64 one
    vals32 = vals.detach().float().requires_grad_()
    x32 = x.detach().float().requires_grad_()
    ag.csr_spmv(A, vals32, x32).sum().backward()
    ag.csr_spmv(A, vals, x).sum().backward()
    assert torch.allclose(vals32.grad.double(), vals.grad, rtol=1e-6, atol=1e-6)
    assert torch.allclose(x32.grad.double(), x.grad, rtol=1e-5, atol=1e-5)
    # PageRank fixed point
    P, rp, ci, va, dang = _rmat(gpu, orc, 5, 8)
    n = rp.size - 1
    pv = torch.from_numpy(va).to(dev).requires_grad_()
    tv = torch.full((n,), 1.0 / n, dtype=torch.float64, device=dev, requires_grad=True)
    wt = torch.from_numpy(np.random.default_rng(1).standard_normal(n)).to(dev)
    f = lambda a, b: (ag.pagerank(P, a, b, tol=1e-15) * wt).sum()
    assert torch.autograd.gradcheck(f, (pv, tv), eps=1e-7, atol=1e-7, rtol=1e-5)
    f0 = lambda a, b: (ag.pagerank(P, a, b, tol=1e-15, accel=0) * wt).sum()
    assert torch.autograd.gradcheck(f0, (pv, tv), eps=1e-7, atol=1e-7, rtol=1e-5)


def test_adjoint_against_finite_differences_rmat_2p22(gpu):
    """The differentiation configuration's graph (R-MAT 2^22, 2^26 draws,
    seed 1; w ~ N(0,1) seed 2): the adjoint values gradient against central
    fourth-order differences of the GPU forward solve on 60 random edges
    (bench.py checks 1000), relative error <= 1e-6; the step grows for small
    gradients so that the loss difference stands above its FP64 rounding
    (bench.fd_check_edges)."""
    import bench
    scale = 22
    G = gpu.DeviceMatrix.rmat_pagerank(scale, 16 << scale, seed=1)
    n, nnz = G.info().n_row, int(G.info().stored)
    dev = torch.device("cuda")
    w = torch.from_numpy(np.random.default_rng(2).standard_normal(n)).to(dev)
    v = torch.full((n,), 1.0 / n, dtype=torch.float64, device=dev)
    x = torch.empty(n, dtype=torch.float64, device=dev)
    gvals = torch.empty(nnz, dtype=torch.float64, device=dev)
    G.pagerank_teleport(v.data_ptr(), x.data_ptr(), 0.85, 1e-15, 2000, accel=1)
    r = G.pagerank_adjoint(v.data_ptr(), x.data_ptr(), w.data_ptr(), gvals.data_ptr(), 0, 0.85, n * 1e-15, 2000,
                           accel=1)
    assert r.converged
    fd = bench.fd_check_edges(gpu, G, v, w, gvals.cpu().numpy(), 60, seed=11)
    assert fd["rel_err_max"] <= 1e-6, fd
