"""PageRank on the GPU against the oracle, through the C ABI.

Reference mode (Matrix::page_rank / personalized_page_rank, Matrix.cpp:13-114):
same iteration count as the oracle and vectors equal to 1e-12 (the GPU sums
in another order).  Dangling mode: FP64 and mixed precision against the
oracle's FP64 iteration run to a tighter tolerance, L1 distance <= 1e-10.
"""
import math

import numpy as np
import pytest

from test_oracle import FORMATS

pytestmark = pytest.mark.gpu


def rmat_csr_oracle(orc, scale, m, seed):
    """The R-MAT PageRank matrix built in numpy from the oracle's edges."""
    src, dst = orc.rmat_edges(scale, m, seed=seed)
    n = 1 << scale
    key = np.unique((dst.astype(np.int64) << scale) | src.astype(np.int64))
    d = (key >> scale).astype(np.int32)
    s = (key & (n - 1)).astype(np.int32)
    rowptr = np.zeros(n + 1, np.int32)
    np.add.at(rowptr, d + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    outdeg = np.bincount(s, minlength=n)
    values = 1.0 / outdeg[s]
    dangling = (outdeg == 0).astype(np.uint8)
    return rowptr, s, values, dangling


def test_rmat_matrix_matches_oracle(gpu, orc):
    for (scale, m, seed) in [(6, 300, 1), (10, 16 << 10, 1), (12, 16 << 12, 7)]:
        A = gpu.DeviceMatrix.rmat_pagerank(scale, m, seed=seed)
        rp, ci, va = A.csr_download()
        orp, oci, ova, _ = rmat_csr_oracle(orc, scale, m, seed)
        assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
        assert np.array_equal(va, ova)


@pytest.mark.parametrize("fmt", FORMATS)
def test_reference_mode_matches_golden_and_oracle(gpu, orc, golden, fmt):
    for rec in golden["page_rank"]:
        if rec["format"] != fmt:
            continue
        nr, nc, c = rec["shape"]
        g = gpu.generate(fmt, "cqmat_stochastic", nr, nc, c, rec["q"], rec["seed"])
        m = gpu.DeviceMatrix.from_generated(g)
        for key, (eps, beta, mx) in (("swapped", (0.85, 0.01, 10)), ("tight", (1e-10, 0.85, 500))):
            b, r = m.pagerank_host(beta=beta, tol=eps, max_iter=mx, mode=gpu.PR_REFERENCE)
            ref = np.array([float(v) for v in rec[key]["b"]])
            assert r.iterations == rec[key]["it"], (fmt, rec["shape"], key, r.iterations, rec[key]["it"])
            np.testing.assert_allclose(b, ref, rtol=1e-12, atol=1e-15)
        p, r = m.personalized_pagerank_host([1, 3], beta=0.01, tol=0.85, max_iter=10)
        ref = np.array([float(v) for v in rec["ppr"]["b"]])
        assert r.iterations == rec["ppr"]["it"]
        np.testing.assert_allclose(p, ref, rtol=1e-12, atol=1e-15)


def test_reference_mode_larger_against_oracle(gpu, orc):
    for fmt in ("CSR", "ELL", "COO"):
        g = gpu.generate(fmt, "cqmat_stochastic", 20000, 20000, 12, 0.3, 1)
        m = gpu.DeviceMatrix.from_generated(g)
        o = orc.from_layout(fmt, g.geom, g.nnz, g.values, g.idx0, g.idx1)
        b, r = m.pagerank_host(beta=0.85, tol=1e-6, max_iter=200, mode=gpu.PR_REFERENCE)
        bo, it = o.page_rank(1e-6, 0.85, 200)
        assert r.iterations == it
        assert np.abs(b - bo).sum() < 1e-12
        p, r = m.personalized_pagerank_host([5, 77, 9000, 5], beta=0.85, tol=1e-6, max_iter=200)
        po, it = o.personalized_page_rank(1e-6, 0.85, 200, [5, 77, 9000, 5])
        assert r.iterations == it
        assert np.abs(p - po).sum() < 1e-12


# scale 18 has a row of 15910 entries: the product cuts it into chunks, and
# the chunk fixup's sums must enter the sweep's mass and residual
@pytest.mark.parametrize("scale", [10, 14, 18])
def test_dangling_mode_fp64_and_mixed(gpu, orc, scale):
    m = 16 << scale
    A = gpu.DeviceMatrix.rmat_pagerank(scale, m, seed=1,
                                       stores=gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16)
    rp, ci, va, dang = rmat_csr_oracle(orc, scale, m, 1)
    if scale == 18:
        assert np.diff(rp).max() > 8192
    # The oracle sums the mass sequentially and does not normalise; its total
    # drifts from 1 (by 1.2e-12 after 8 sweeps at scale 18).  The sweep is
    # linear and homogeneous in x, and the GPU returns x / sum(x), so the
    # oracle's vectors are compared after an exact normalisation (fsum).
    xo, it_o, res_o = orc.page_rank_dangling(rp, ci, va, dang, 0.85, 1e-14, 5000)
    assert res_o < 1e-14
    xo = xo / math.fsum(xo)
    # same number of sweeps from the same start: the FP64 iterates agree
    x8, r8 = A.pagerank_host(beta=0.85, tol=0.0, max_iter=8, mode=gpu.PR_DANGLING)
    x8o, _, _ = orc.page_rank_dangling(rp, ci, va, dang, 0.85, 0.0, 8)
    x8o = x8o / math.fsum(x8o)
    assert r8.iterations == 8 and np.abs(x8 - x8o).sum() < 1e-13
    sweeps = {}
    for prec in (gpu.F64, gpu.F32, gpu.BF16):
        x, r = A.pagerank_host(beta=0.85, tol=1e-11, max_iter=5000, mode=gpu.PR_DANGLING, precision=prec)
        assert r.converged, prec
        assert abs(x.sum() - 1.0) < 1e-12
        err = np.abs(x - xo).sum()
        assert err < 1e-10, (prec, err, r.iterations, r.iterations_f64)
        sweeps[prec] = r.iterations
    # Anderson-accelerated FP64: same fixed point, same stopping rule, fewer sweeps
    x, r = A.pagerank_host(beta=0.85, tol=1e-11, max_iter=5000, mode=gpu.PR_DANGLING, accel=1)
    assert r.converged and r.residual < 1e-11
    assert abs(x.sum() - 1.0) < 1e-12
    assert np.abs(x - xo).sum() < 1e-10, (r.iterations, np.abs(x - xo).sum())
    # mixed precision with Anderson-accelerated inner (correction) solves
    for prec in (gpu.F32, gpu.BF16):
        xm, rm = A.pagerank_host(beta=0.85, tol=1e-11, max_iter=5000, mode=gpu.PR_DANGLING, precision=prec,
                                 accel=1)
        assert rm.converged and abs(xm.sum() - 1.0) < 1e-12, prec
        assert np.abs(xm - xo).sum() < 1e-10, (prec, np.abs(xm - xo).sum(), rm.iterations, rm.iterations_f64)
    # (at scale 10 the plain iteration converges as fast: 17 sweeps both)
    assert r.iterations <= sweeps[gpu.F64] - (2 if scale >= 14 else 0), (r.iterations, sweeps[gpu.F64])


@pytest.mark.parametrize("scale,mode", [(14, 1), (20, -1)])
def test_relabelled_pagerank(gpu, orc, scale, mode):
    """PageRank on the degree-relabelled copy (forced at scale 14, chosen by
    the automatic rule at 2^20) returns the vector of the original labels."""
    m = 16 << scale
    A = gpu.DeviceMatrix.rmat_pagerank(scale, m, seed=3, stores=gpu.STORE_F64 | gpu.STORE_BF16)
    P = gpu.DeviceMatrix.rmat_pagerank(scale, m, seed=3, stores=gpu.STORE_F64 | gpu.STORE_BF16)
    P.tune(gpu.TUNE_PR_RELABEL, 0)
    A.tune(gpu.TUNE_PR_RELABEL, mode)
    rp, ci, va, dang = rmat_csr_oracle(orc, scale, m, 3)
    xo, _, res_o = orc.page_rank_dangling(rp, ci, va, dang, 0.85, 1e-14, 5000, threads=8)
    xo = xo / math.fsum(xo)
    for prec, acc in ((gpu.F64, 0), (gpu.BF16, 0), (gpu.F64, 1)):
        x, r = A.pagerank_host(tol=1e-11, max_iter=5000, mode=gpu.PR_DANGLING, precision=prec, accel=acc)
        xp, rp_ = P.pagerank_host(tol=1e-11, max_iter=5000, mode=gpu.PR_DANGLING, precision=prec, accel=acc)
        assert r.converged and rp_.converged
        assert np.abs(x - xo).sum() < 1e-10, (prec, acc)
        assert np.abs(x - xp).sum() < 1e-10, (prec, acc)


@pytest.mark.parametrize("relabel", [-1, 1])
def test_reference_mode_large_skewed_against_oracle(gpu, orc, relabel):
    """Matrix::page_rank / personalized_page_rank (Matrix.cpp:13-114) on a
    non-banded R-MAT graph of 2^20 vertices, where the dangling mode takes the
    degree-relabelled copy: the reference mode sweeps the handle itself (with
    the automatic rule and with relabelling forced), so it stops after the
    oracle's iteration count.  Its vector is within 1e-12 of the reference's
    iteration with correctly rounded sums (page_rank_exact_sums); the
    reference's own left-to-right sums of 2^20 positive values move its
    vector by up to (n-1) u, 1.5e-11 here, and the GPU stays within that
    bound of the reference-faithful oracle."""
    from oracle.oracle import page_rank_exact_sums
    scale = 20
    m = 16 << scale
    A = gpu.DeviceMatrix.rmat_pagerank(scale, m, seed=3)
    A.tune(gpu.TUNE_PR_RELABEL, relabel)
    rp, ci, va, _ = rmat_csr_oracle(orc, scale, m, 3)
    n = 1 << scale
    sum_bound = 4 * n * 2.0 ** -53
    o = orc.from_arrays("CSR", n, n, va, rp, ci)
    for eps in (1e-9, 1e-6):
        b, r = A.pagerank_host(beta=0.85, tol=eps, max_iter=500, mode=gpu.PR_REFERENCE)
        bo, it = o.page_rank(eps, 0.85, 500, threads=1)
        be, ite = page_rank_exact_sums(rp, ci, va, eps, 0.85, 500)
        assert r.iterations == it == ite, (eps, r.iterations, it, ite)
        assert np.abs(b - be).sum() <= 1e-12, (eps, np.abs(b - be).sum())
        assert np.abs(b - bo).sum() <= sum_bound, (eps, np.abs(b - bo).sum())
    nodes = [0, 7, 7, n - 1, 12345]
    p, r = A.personalized_pagerank_host(nodes, beta=0.85, tol=1e-9, max_iter=500)
    po, it = o.personalized_page_rank(1e-9, 0.85, 500, nodes, threads=1)
    pe, ite = page_rank_exact_sums(rp, ci, va, 1e-9, 0.85, 500, nodes)
    assert r.iterations == it == ite, (r.iterations, it, ite)
    assert np.abs(p - pe).sum() <= 1e-12, np.abs(p - pe).sum()
    assert np.abs(p - po).sum() <= sum_bound, np.abs(p - po).sum()


def test_pagerank_argument_checks(gpu):
    g = gpu.generate("CSR", "cqmat_stochastic", 50, 40, 5, 0.1, 0)
    m = gpu.DeviceMatrix.from_generated(g)
    with pytest.raises(gpu.TbslaError):
        m.pagerank_host()  # not square
    g = gpu.generate("CSR", "cqmat_stochastic", 50, 50, 5, 0.1, 0)
    m = gpu.DeviceMatrix.from_generated(g)
    with pytest.raises(gpu.TbslaError):
        m.pagerank_host(precision=gpu.BF16)  # no BF16 store
    with pytest.raises(gpu.TbslaError):
        m.pagerank_host(mode=gpu.PR_REFERENCE, precision=gpu.F32)
    with pytest.raises(gpu.TbslaError):
        m.pagerank_host(mode=gpu.PR_REFERENCE, accel=1)  # acceleration: dangling mode only
    with pytest.raises(gpu.TbslaError):
        m.pagerank_host(accel=2)
