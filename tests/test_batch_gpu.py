"""Batching on the GPU: many matrices in one launch, and many personalized
PageRank vectors of one graph solved together.

Multi-matrix batch: every member's product equals the one-matrix product of
the same handle bit for bit (both sum each row in its stored order), masked
members are left untouched, the graph-replayed launch gives the same
vectors.  Batched PageRank: each vector against the FP64 CPU restatement of
the teleport-form PageRank (oracle/tbsla_oracle.c, orc_pagerank_teleport)
with the vector's seed distribution, L1 <= 1e-12 and the same number of
sweeps (within one) for FP64; FP32 iterates within 1e-5 of it.
"""
import numpy as np
import pytest

from test_pagerank_gpu import rmat_csr_oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_multi_matrix_batch_matches_single_products(gpu):
    rng = np.random.default_rng(3)
    dev = torch.device("cuda")
    members, xs, ys = [], [], []
    for m in range(12):
        # two members large enough for the ELL-layout copy (read from it, two
        # rows per thread, for the F64 and F32 stores; BF16 from the CSR arrays)
        n = 70000 + 61000 * (m - 10) if m >= 10 else int(np.exp(rng.uniform(np.log(1000), np.log(60000))))
        c = int(rng.integers(8, 33))
        members.append(gpu.DeviceMatrix.generate("CSR", "cqmat", n, n, c, 0.1, m + 1,
                                                 stores=gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16))
    assert members[10].info().slices > 0 and members[11].info().slices > 0
    B = gpu.Batch(members)
    for A in members:  # the batch sums each row in one thread, in stored order
        A.tune(gpu.TUNE_SHORT_ROWS, 0)
    for store, tdt in ((gpu.F64, torch.float64), (gpu.F32, torch.float32), (gpu.BF16, torch.float32)):
        xs = [torch.rand(A.info().n_col, dtype=tdt, device=dev) for A in members]
        ys = [torch.full((A.info().n_row,), float("nan"), dtype=tdt, device=dev) for A in members]
        B.bind(store, [x.data_ptr() for x in xs], [y.data_ptr() for y in ys])
        B.spmv()
        torch.cuda.synchronize()
        vt = gpu.F64 if store == gpu.F64 else gpu.F32
        for A, x, y in zip(members, xs, ys):
            ref = torch.empty_like(y)
            A.spmv_ex(store, vt, x.data_ptr(), vt, ref.data_ptr(), 0, None)
            torch.cuda.synchronize()
            assert torch.equal(y, ref)
        # the graph replay
        for y in ys:
            y.fill_(float("nan"))
        B.spmv(graph=True)
        B.spmv(graph=True)
        torch.cuda.synchronize()
        for A, x, y in zip(members, xs, ys):
            ref = torch.empty_like(y)
            A.spmv_ex(store, vt, x.data_ptr(), vt, ref.data_ptr(), 0, None)
            torch.cuda.synchronize()
            assert torch.equal(y, ref)
    # per-member mask: masked members keep their y
    mask = torch.tensor([m % 3 != 0 for m in range(12)], dtype=torch.int32, device=dev)
    B.set_mask(mask.data_ptr())
    for y in ys:
        y.fill_(-7.0)
    B.spmv()
    torch.cuda.synchronize()
    for m, y in enumerate(ys):
        assert bool((y == -7.0).all()) == (m % 3 == 0)
    B.close()


def _seed_sets(rng, n, k):
    sets = []
    for _ in range(k):
        size = int(np.exp(rng.uniform(0, np.log(100))))
        sets.append(rng.integers(0, n, size))
    sets[0] = np.array([0, 0, 3])  # repeated seed counts once
    return sets


@pytest.mark.parametrize("tile,relabel,accel", [(2, 1, 0), (4, 0, 0), (8, 0, 0), (16, 0, 0), (32, 1, 0),
                                                (2, 0, 1), (8, 1, 1), (32, 1, 1)])
def test_batched_ppr_matches_oracle(gpu, orc, tile, relabel, accel):
    """Every vector against the oracle's teleport-form solve (L1 < 1e-12 at
    tol 1e-13; the plain solve also within one sweep of the oracle's count);
    the FP32 solve within 1e-5 and the refined FP32 solve to the FP64
    tolerance.  accel = 1: the Anderson-accelerated solves (fewer sweeps, same
    fixed point and stopping rule)."""
    scale = 12
    m = 16 << scale
    A = gpu.DeviceMatrix.rmat_pagerank(scale, m, seed=5, stores=gpu.STORE_F64 | gpu.STORE_F32)
    A.tune(gpu.TUNE_PR_RELABEL, relabel)
    rp, ci, va, dang = rmat_csr_oracle(orc, scale, m, 5)
    n = rp.size - 1
    rng = np.random.default_rng(tile)
    k = 40
    sets = _seed_sets(rng, n, k)
    dev = torch.device("cuda")
    out = torch.empty(k * n, dtype=torch.float64, device=dev)
    its, res = gpu.ppr_batched(A, sets, out.data_ptr(), tol=1e-13, max_iter=1000, tile=tile, accel=accel)
    got = out.cpu().numpy().reshape(k, n)
    sweeps, sweeps_oracle = 0, 0
    for c in (0, 1, 7, 20, 39):
        v = np.zeros(n)
        seeds = np.unique(sets[c])
        v[seeds] = 1.0 / seeds.size
        xo, ito, _ = orc.pagerank_teleport(rp, ci, va, dang, v, 0.85, 1e-13, 1000)
        assert np.abs(got[c] - xo).sum() < 1e-12, c
        assert res[c] < 1e-13
        if accel:
            assert int(its[c]) <= ito, (c, int(its[c]), ito)
        else:
            assert abs(int(its[c]) - ito) <= 1
        sweeps += int(its[c])
        sweeps_oracle += ito
    if accel:
        assert sweeps < sweeps_oracle
    # FP32 iterates and store
    out32 = torch.empty(k * n, dtype=torch.float64, device=dev)
    its32, res32 = gpu.ppr_batched(A, sets, out32.data_ptr(), tol=1e-6, max_iter=1000, tile=tile,
                                   precision=gpu.F32, accel=accel)
    got32 = out32.cpu().numpy().reshape(k, n)
    assert np.max(np.abs(got32 - got).sum(axis=1)) < 1e-5
    # FP32 sweeps with FP64 defect correction: every vector to the FP64 tolerance
    outr = torch.empty(k * n, dtype=torch.float64, device=dev)
    itsr, resr = gpu.ppr_batched(A, sets, outr.data_ptr(), tol=1e-12, max_iter=1000, tile=tile,
                                 precision=gpu.F32, refined=True, accel=accel)
    assert (resr < 1e-12).all(), resr.max()
    gotr = outr.cpu().numpy().reshape(k, n)
    for c in (0, 1, 7, 20, 39):
        v = np.zeros(n)
        seeds = np.unique(sets[c])
        v[seeds] = 1.0 / seeds.size
        xo, _, _ = orc.pagerank_teleport(rp, ci, va, dang, v, 0.85, 1e-14, 2000)
        assert np.abs(gotr[c] - xo).sum() < 1e-11, (c, np.abs(gotr[c] - xo).sum())


@pytest.mark.parametrize("tile,check_every,prec,accel", [(8, 1, "F64", 0), (4, 3, "F64", 0), (32, 2, "F32", 0),
                                                         (8, 1, "F64", 1), (32, 3, "F64", 1), (16, 2, "F32", 1)])
def test_batched_ppr_repacking_is_exact(gpu, tile, check_every, prec, accel):
    """Vectors stop at different sweeps and the running ones are repacked
    into fewer tiles between rounds (accelerated solves: with their output
    and residual histories); a column's arithmetic does not depend on its
    tile or lane, so each vector equals the same vector solved alone bit for
    bit, with the same sweep count and residual."""
    scale = 11
    A = gpu.DeviceMatrix.rmat_pagerank(scale, 16 << scale, seed=9, stores=gpu.STORE_F64 | gpu.STORE_F32)
    n = A.info().n_row
    rng = np.random.default_rng(3)
    k = 37
    sets = _seed_sets(rng, n, k)
    dev = torch.device("cuda")
    precision = getattr(gpu, prec)
    tol = 1e-12 if prec == "F64" else 1e-6
    out = torch.empty(k * n, dtype=torch.float64, device=dev)
    its, res = gpu.ppr_batched(A, sets, out.data_ptr(), tol=tol, max_iter=1000, tile=tile, precision=precision,
                               check_every=check_every, accel=accel)
    assert its.min() < its.max()  # the vectors stop at different sweeps
    got = out.view(k, n)
    one = torch.empty(n, dtype=torch.float64, device=dev)
    for c in (0, 5, int(np.argmin(its)), int(np.argmax(its)), k - 1):
        i1, r1 = gpu.ppr_batched(A, [sets[c]], one.data_ptr(), tol=tol, max_iter=1000, tile=tile,
                                 precision=precision, check_every=check_every, accel=accel)
        assert torch.equal(one, got[c]), c
        assert int(i1[0]) == int(its[c]) and float(r1[0]) == float(res[c])
    # a sweep cap stops every vector at max_iter; max_iter 0 returns the start vectors
    its5, _ = gpu.ppr_batched(A, sets, out.data_ptr(), tol=0.0, max_iter=5, tile=tile, precision=precision,
                              check_every=check_every, accel=accel)
    assert (its5 == 5).all()
    its0, _ = gpu.ppr_batched(A, sets[:3], out.data_ptr(), tol=tol, max_iter=0, tile=tile, accel=accel)
    assert (its0 == 0).all()
    v = np.zeros(n)
    seeds = np.unique(sets[1])
    v[seeds] = 1.0 / seeds.size
    assert np.array_equal(out.view(k, n)[1].cpu().numpy(), v)


def test_autotuners_keep_results(gpu, orc):
    """The tuners time candidates and keep the fastest; products and
    PageRank vectors are the same before and after."""
    dev = torch.device("cuda")
    A = gpu.DeviceMatrix.rmat_pagerank(12, 16 << 12, seed=2, stores=gpu.STORE_F64 | gpu.STORE_F32)
    x = np.random.default_rng(0).uniform(-1, 1, 1 << 12)
    before = A.spmv_host(x)
    r = A.autotune_spmv(gpu.F64)
    assert r.candidates >= 2 and r.best_ms > 0 and r.choice in (0, 1, 2, 3) and 0.0 <= r.value <= 1.0
    after = A.spmv_host(x)
    assert np.allclose(after, before, rtol=1e-13, atol=1e-15)
    sets = [[i * 37 % 4096] for i in range(48)]
    out0 = torch.empty(48 << 12, dtype=torch.float64, device=dev)
    gpu.ppr_batched(A, sets, out0.data_ptr(), tol=1e-13, max_iter=500, tile=8)
    t = A.autotune_ppr(48, gpu.F64)
    assert t.choice in (2, 4, 8, 16, 32) and t.candidates >= 2
    out1 = torch.empty(48 << 12, dtype=torch.float64, device=dev)
    gpu.ppr_batched(A, sets, out1.data_ptr(), tol=1e-13, max_iter=500)  # tile 0: the tuned one
    assert float((out1 - out0).abs().sum()) < 1e-11
    members = [gpu.DeviceMatrix.generate("CSR", "cqmat", 3000 + 500 * m, 3000 + 500 * m, 10, 0.1, m + 1)
               for m in range(6)]
    B = gpu.Batch(members)
    xs = [torch.rand(M.info().n_col, dtype=torch.float64, device=dev) for M in members]
    ys = [torch.empty(M.info().n_row, dtype=torch.float64, device=dev) for M in members]
    B.bind(gpu.F64, [v.data_ptr() for v in xs], [v.data_ptr() for v in ys])
    B.spmv()
    torch.cuda.synchronize()
    ref = [y.clone() for y in ys]
    b = B.autotune()
    assert b.choice >= 1 and b.candidates >= 4
    B.spmv()
    torch.cuda.synchronize()
    assert all(torch.equal(y, r0) for y, r0 in zip(ys, ref))
    B.close()
