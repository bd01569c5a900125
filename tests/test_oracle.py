"""Pins the CPU oracle (oracle/tbsla_oracle.c) to the TBSLA reference.

Two anchors: the reference itself compiled from its sources (oracle/_ref,
present where the TBSLA sources are) and the golden vectors in
tests/golden/golden.json written from it by tests/golden/make_golden.py.
"""
import numpy as np
import pytest

from conftest import fnv
from oracle.oracle import parse_binary, write_binary

FORMATS = ["COO", "SCOO", "CSR", "ELL", "DENSE"]
SHAPES = [(10, 5, 8), (5, 10, 7), (10, 10, 12), (10, 10, 3), (10, 5, 3), (10, 5, 6), (30, 30, 6), (20, 30, 5),
          (30, 20, 7), (10, 10, 0), (1, 1, 1), (7, 3, 2)]
BLOCKS = [(0, 0, 1, 1), (0, 0, 2, 2), (1, 1, 2, 2), (1, 0, 2, 3), (2, 1, 3, 2)]


def nnz_defined(fmt, gen, n_values):
    """The reference leaves nnz unset for CSR/SCOO fill_cdiag and for fills
    that return before storing anything."""
    if gen == "cdiag" and fmt in ("CSR", "SCOO"):
        return False
    return n_values > 0


def same_arrays(a, b, fmt, gen, tag, check_nnz=None):
    for f in ("n_row", "n_col", "ln_row", "ln_col", "f_row", "f_col", "pr", "pc", "NR", "NC", "max_col"):
        assert getattr(a, f) == getattr(b, f), f"{tag}: {f} {getattr(a, f)} != {getattr(b, f)}"
    if nnz_defined(fmt, gen, b.values.size) if check_nnz is None else check_nnz:
        assert a.nnz == b.nnz, f"{tag}: nnz {a.nnz} != {b.nnz}"
    for f in ("values", "idx0", "idx1"):
        x, y = getattr(a, f), getattr(b, f)
        assert x.shape == y.shape and np.array_equal(x, y), f"{tag}: {f} differs"


@pytest.mark.parametrize("fmt", FORMATS)
def test_generators_match_reference(orc, ref, fmt):
    for (nr, nc, c) in SHAPES:
        for s in (0, 1, 3):
            for q in (0.0, 0.1, 1.0):
                for blk in BLOCKS:
                    same_arrays(orc.fill_cqmat(fmt, nr, nc, c, q, s, *blk).arrays,
                                ref.fill_cqmat(fmt, nr, nc, c, q, s, *blk).arrays, fmt, "cqmat",
                                ("cqmat", nr, nc, c, q, s, blk))
                    same_arrays(orc.fill_cqmat_stochastic(fmt, nr, nc, c, q, s, *blk).arrays,
                                ref.fill_cqmat_stochastic(fmt, nr, nc, c, q, s, *blk).arrays, fmt, "stoch",
                                ("stoch", nr, nc, c, q, s, blk))
        for cd in (0, 1, 2, 5, 9):
            for blk in BLOCKS:
                same_arrays(orc.fill_cdiag(fmt, nr, nc, cd, *blk).arrays, ref.fill_cdiag(fmt, nr, nc, cd, *blk).arrays,
                            fmt, "cdiag", ("cdiag", nr, nc, cd, blk))


def test_conversions_and_products_match_reference(orc, ref):
    rng = np.random.default_rng(5)
    for (nr, nc, c) in SHAPES:
        for s in (0, 1):
            for q in (0.0, 0.3, 1.0):
                a, b = orc.fill_cqmat("COO", nr, nc, c, q, s), ref.fill_cqmat("COO", nr, nc, c, q, s)
                for f in ("SCOO", "CSR", "ELL", "DENSE"):
                    # a conversion copies the COO's nnz, unset when the COO is empty
                    same_arrays(a.convert(f).arrays, b.convert(f).arrays, f, "convert", ("convert", f, nr, nc, c),
                                check_nnz=a.arrays.values.size > 0)
                x = rng.uniform(-1, 1, nc)
                for f in FORMATS:
                    ao, ar = orc.fill_cqmat(f, nr, nc, c, q, s), ref.fill_cqmat(f, nr, nc, c, q, s)
                    assert np.array_equal(ao.spmv(x), ar.spmv(x)), (f, nr, nc, c, q, s)
                    if nr == nc:
                        assert np.array_equal(ao.a_axpx(x), ar.a_axpx(x)), (f, nr, nc, c, q, s)
                        so = orc.fill_cqmat_stochastic(f, nr, nc, c, q, s)
                        sr = ref.fill_cqmat_stochastic(f, nr, nc, c, q, s)
                        for args in ((0.85, 0.01, 10), (1e-10, 0.85, 300)):
                            bo, io = so.page_rank(*args)
                            br, ir = sr.page_rank(*args)
                            assert io == ir and np.array_equal(bo, br), (f, nr, nc, c, q, s, args)
                        bo, io = so.personalized_page_rank(0.85, 0.01, 10, [1, 3])
                        br, ir = sr.personalized_page_rank(0.85, 0.01, 10, [1, 3])
                        assert io == ir and np.array_equal(bo, br)


def test_arrays_constructors_match_reference(orc, ref):
    rng = np.random.default_rng(7)
    for trial in range(20):
        nr, nc = rng.integers(1, 40, 2)
        nnz = int(rng.integers(0, 120))
        row = rng.integers(0, nr, nnz).astype(np.int32)
        col = rng.integers(0, nc, nnz).astype(np.int32)
        val = rng.standard_normal(nnz)
        x = rng.standard_normal(nc)
        a, b = orc.from_arrays("COO", nr, nc, val, row, col), ref.from_arrays("COO", nr, nc, val, row, col)
        a.update_nnz(); b.update_nnz()
        assert np.array_equal(a.spmv(x), b.spmv(x))
        for f in ("CSR", "ELL", "DENSE", "SCOO"):
            ca, cb = a.convert(f), b.convert(f)
            # the reference's std::sort is unstable: tied (row, col) entries may
            # swap, which changes values only when the tied values differ
            ka, kb = ca.arrays, cb.arrays
            if f == "CSR":
                assert np.array_equal(ka.rowptr, kb.rowptr)
                assert np.array_equal(ka.colidx, kb.colidx)
            np.testing.assert_allclose(ca.spmv(x), cb.spmv(x), rtol=1e-12, atol=1e-12)


def test_known_answer(orc, golden):
    ka = golden["known_answer"]
    coo = orc.from_arrays("COO", 5, 5, ka["values"], ka["row"], ka["col"])
    csr = orc.from_arrays("CSR", 5, 5, ka["values"], ka["rowptr"], ka["col"])
    assert coo.spmv(ka["x"]).tolist() == ka["coo"] == [20, 12, 10, 40, 85]
    assert csr.spmv(ka["x"]).tolist() == ka["csr"] == [20, 12, 10, 40, 85]


def test_generators_match_golden(orc, golden):
    for rec in golden["generators"]:
        f, gen = rec["format"], rec["gen"]
        if gen == "cdiag":
            m = orc.fill_cdiag(f, *rec["shape"], *rec["block"])
        else:
            fill = orc.fill_cqmat if gen == "cqmat" else orc.fill_cqmat_stochastic
            m = fill(f, *rec["shape"], rec["q"], rec["seed"], *rec["block"])
        a = m.arrays
        tag = (f, gen, rec["shape"], rec.get("q"), rec.get("seed"), rec["block"])
        assert [a.n_row, a.n_col, a.ln_row, a.ln_col, a.f_row, a.f_col, a.pr, a.pc, a.NR, a.NC,
                a.max_col] == rec["geom"], tag
        if nnz_defined(f, gen, rec["n_values"]):
            assert a.nnz == rec["nnz"], tag
        assert (fnv(a.values), fnv(a.idx0), fnv(a.idx1)) == (rec["values"], rec["idx0"], rec["idx1"]), tag


def test_spmv_iota_and_page_rank_match_golden(orc, golden):
    for rec in golden["spmv_iota"]:
        nr, nc, c = rec["shape"]
        m = orc.fill_cqmat(rec["format"], nr, nc, c, rec["q"], rec["seed"])
        assert m.spmv(np.arange(nc, dtype=np.float64)).tolist() == rec["y"], rec
    for rec in golden["page_rank"]:
        nr, nc, c = rec["shape"]
        m = orc.fill_cqmat_stochastic(rec["format"], nr, nc, c, rec["q"], rec["seed"])
        b, it = m.page_rank(0.85, 0.01, 10)
        assert it == rec["swapped"]["it"] and [repr(float(v)) for v in b] == rec["swapped"]["b"]
        b, it = m.page_rank(1e-10, 0.85, 500)
        assert it == rec["tight"]["it"] and [repr(float(v)) for v in b] == rec["tight"]["b"]
        b, it = m.personalized_page_rank(0.85, 0.01, 10, [1, 3])
        assert it == rec["ppr"]["it"] and [repr(float(v)) for v in b] == rec["ppr"]["b"]


def test_exact_sum_page_rank_against_golden_and_oracle(orc, golden):
    """The exact-sum restatement of Matrix::page_rank / personalized_page_rank
    (oracle.page_rank_exact_sums) against the reference's golden vectors
    (small: the sums' order is immaterial there) and, on an R-MAT graph of
    2^16 vertices, against the reference-faithful oracle: same iteration
    counts, vectors within the reference's own summation error (n-1) u."""
    from oracle.oracle import page_rank_exact_sums
    for rec in golden["page_rank"]:
        nr, nc, c = rec["shape"]
        if nr != nc or rec["format"] != "CSR":
            continue
        a = orc.fill_cqmat_stochastic("CSR", nr, nc, c, rec["q"], rec["seed"]).arrays
        b, it = page_rank_exact_sums(a.rowptr, a.colidx, a.values, 1e-10, 0.85, 500)
        ref = np.array([float(v) for v in rec["tight"]["b"]])
        assert it == rec["tight"]["it"] and np.abs(b - ref).sum() < 1e-14
        p, it = page_rank_exact_sums(a.rowptr, a.colidx, a.values, 0.85, 0.01, 10, [1, 3])
        ref = np.array([float(v) for v in rec["ppr"]["b"]])
        assert it == rec["ppr"]["it"] and np.abs(p - ref).sum() < 1e-14
    scale = 16
    n = 1 << scale
    src, dst = orc.rmat_edges(scale, 16 << scale, seed=3)
    key = np.unique((dst.astype(np.int64) << scale) | src.astype(np.int64))
    d, sc = (key >> scale).astype(np.int32), (key & (n - 1)).astype(np.int32)
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, d + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    va = 1.0 / np.bincount(sc, minlength=n)[sc]
    o = orc.from_arrays("CSR", n, n, va, rp, sc)
    bo, it = o.page_rank(1e-9, 0.85, 500)
    be, ite = page_rank_exact_sums(rp, sc, va, 1e-9, 0.85, 500)
    assert it == ite and np.abs(be - bo).sum() <= n * 2.0 ** -53


def test_cfg1_matches_golden(orc, golden):
    g = golden["cfg1"]
    m = orc.fill_cqmat("CSR", 100000, 100000, 10, 0.1, 0)
    a = m.arrays
    r = g["arrays"]
    assert (a.nnz, a.values.size, a.idx0.size) == (r["nnz"], r["n_values"], r["n_idx0"])
    assert (fnv(a.values), fnv(a.idx0), fnv(a.idx1)) == (r["values"], r["idx0"], r["idx1"])
    x = np.random.default_rng(g["x_seed"]).random(100000)
    y = m.spmv(x, threads=4)
    assert fnv(y) == g["y_fnv"] and repr(float(y.sum())) == g["y_sum"]


def test_rmat_oracle_is_deterministic(orc):
    s1, d1 = orc.rmat_edges(10, 5000, seed=1)
    s2, d2 = orc.rmat_edges(10, 5000, seed=1)
    s3, _ = orc.rmat_edges(10, 5000, seed=2)
    assert np.array_equal(s1, s2) and np.array_equal(d1, d2) and not np.array_equal(s1, s3)
    assert s1.min() >= 0 and s1.max() < 1024 and d1.max() < 1024
    # quadrant frequencies of the top bit follow (a+b, c+d) = (0.76, 0.24)
    top = (s1 >> 9) & 1
    assert abs(top.mean() - 0.24) < 0.03


def _same_bytes(mine, raw, fmt, gen, tag):
    """Equal bytes; the nnz field (bytes 24-31) only where the reference sets it."""
    if not nnz_defined(fmt, gen, parse_binary(fmt, raw).values.size):
        raw, mine = raw[:24] + raw[32:], mine[:24] + mine[32:]
    assert mine == raw, tag


@pytest.mark.parametrize("fmt", FORMATS)
def test_binary_writer_matches_reference_bytes(orc, ref, fmt):
    """write_binary (the layout the drop-in classes' write and the file
    loaders follow) reproduces the reference's own Matrix*::write output byte
    for byte, from the reference's arrays and from the oracle's fill (the nnz
    field where the reference leaves it unset aside, as everywhere)."""
    for (nr, nc, c) in SHAPES[:6]:
        for blk in BLOCKS[:3]:
            raw = ref.fill_cqmat(fmt, nr, nc, c, 0.1, 1, *blk).serialized()
            assert write_binary(parse_binary(fmt, raw)) == raw, (fmt, nr, nc, c, blk)
            _same_bytes(write_binary(orc.fill_cqmat(fmt, nr, nc, c, 0.1, 1, *blk).arrays), raw, fmt, "cqmat",
                        (fmt, "cqmat", nr, nc, c, blk))
            raw = ref.fill_cdiag(fmt, nr, nc, 2, *blk).serialized()
            _same_bytes(write_binary(orc.fill_cdiag(fmt, nr, nc, 2, *blk).arrays), raw, fmt, "cdiag",
                        (fmt, "cdiag", nr, nc, blk))
