"""The product's host generators (tbsla_generate, host_gen.cpp) against the
oracle and the golden fingerprints written from the reference.  CPU only:
generation runs on the host."""
import numpy as np
import pytest

from conftest import fnv
from test_oracle import BLOCKS, FORMATS, SHAPES, nnz_defined


def same(g, a, gen, tag):
    geo = [a.n_row, a.n_col, a.ln_row, a.ln_col, a.f_row, a.f_col, a.pr, a.pc, a.NR, a.NC, a.max_col]
    assert list(g.geom) == geo, f"{tag}: geometry {g.geom} vs {geo}"
    if nnz_defined(g.fmt, gen, a.values.size):
        assert g.nnz == a.nnz, f"{tag}: nnz {g.nnz} vs {a.nnz}"
    for f in ("values", "idx0", "idx1"):
        x, y = getattr(g, f), getattr(a, f)
        assert x.shape == y.shape and np.array_equal(x, y), f"{tag}: {f} differs"


@pytest.mark.parametrize("fmt", FORMATS)
def test_generate_matches_oracle(capi, orc, fmt):
    for (nr, nc, c) in SHAPES + [(100, 100, 10), (64, 40, 9)]:
        for s in (0, 1, 3):
            for q in (0.0, 0.1, 1.0):
                for blk in BLOCKS:
                    for gen in ("cqmat", "cqmat_stochastic"):
                        g = capi.generate(fmt, gen, nr, nc, c, q, s, *blk)
                        fill = orc.fill_cqmat if gen == "cqmat" else orc.fill_cqmat_stochastic
                        same(g, fill(fmt, nr, nc, c, q, s, *blk).arrays, gen, (gen, fmt, nr, nc, c, q, s, blk))
        for cd in (0, 1, 2, 5, 9):
            for blk in BLOCKS:
                g = capi.generate(fmt, "cdiag", nr, nc, cd, 0.0, 0, *blk)
                same(g, orc.fill_cdiag(fmt, nr, nc, cd, *blk).arrays, "cdiag", ("cdiag", fmt, nr, nc, cd, blk))


def test_generate_matches_golden(capi, golden):
    for rec in golden["generators"]:
        f, gen = rec["format"], rec["gen"]
        if gen == "cdiag":
            g = capi.generate(f, "cdiag", *rec["shape"], 0.0, 0, *rec["block"])
        else:
            g = capi.generate(f, gen, *rec["shape"], rec["q"], rec["seed"], *rec["block"])
        tag = (f, gen, rec["shape"], rec.get("q"), rec.get("seed"), rec["block"])
        assert list(g.geom) == rec["geom"], tag
        if nnz_defined(f, gen, rec["n_values"]):
            assert g.nnz == rec["nnz"], tag
        assert (fnv(g.values), fnv(g.idx0), fnv(g.idx1)) == (rec["values"], rec["idx0"], rec["idx1"]), tag


def test_cfg1_arrays_match_golden(capi, golden):
    g = capi.generate("CSR", "cqmat", 100000, 100000, 10, 0.1, 0)
    r = golden["cfg1"]["arrays"]
    assert (g.nnz, g.values.size, g.idx0.size, g.idx1.size) == (r["nnz"], r["n_values"], r["n_idx0"], r["n_idx1"])
    assert (fnv(g.values), fnv(g.idx0), fnv(g.idx1)) == (r["values"], r["idx0"], r["idx1"])


def test_cfg2_arrays_match_golden(capi, golden):
    """The full n=2^24, c=16, q=0.1 matrix the bench times (2.7e8 entries)."""
    g = capi.generate("CSR", "cqmat", 1 << 24, 1 << 24, 16, 0.1, 0)
    r = golden["cfg2"]["arrays"]
    assert (g.nnz, g.values.size, g.idx0.size, g.idx1.size) == (r["nnz"], r["n_values"], r["n_idx0"], r["n_idx1"])
    assert (fnv(g.values), fnv(g.idx0), fnv(g.idx1)) == (r["values"], r["idx0"], r["idx1"])


def test_generate_rejects_bad_arguments(capi):
    with pytest.raises(capi.TbslaError):
        capi.generate("CSR", "cqmat", 10, 10, -1, 0.1, 0)
    with pytest.raises(capi.TbslaError):
        capi.generate("CSR", "cqmat", 10, 10, 3, 0.1, 0, pr=2, NR=2)


def test_splitmix64_known_answers():
    """The value stream of cqmat_baseline: SplitMix64 from state 0 gives the
    generator's published first outputs (Steele, Lea, Flood 2014)."""
    from oracle.oracle import splitmix64_u01
    first = [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    assert list(splitmix64_u01(0, 0, 3)) == [(v >> 11) * 2.0 ** -53 for v in first]


@pytest.mark.parametrize("fmt", FORMATS)
def test_cqmat_baseline_matches_oracle(capi, orc, fmt):
    """Generator 3 (the benchmark's cqmat n = 1e5, c = 10, q = 0.1 with merged
    duplicates and U(0,1] values) against the oracle's restatement: the
    reference's pattern, unique (row, column) pairs, SplitMix64 values."""
    shapes = [(100000, 100000, 10, 0.1, 0), (300, 200, 12, 0.5, 3), (200, 300, 7, 1.0, 1)]
    if fmt == "DENSE":
        shapes = shapes[1:]
    for (nr, nc, c, q, s) in shapes:
        rp, ci, va = orc.baseline_cqmat(nr, nc, c, q, s)
        assert np.all(va > 0) and np.all(va <= 1)
        g = capi.generate(fmt, "cqmat_baseline", nr, nc, c, q, s)
        assert g.nnz == va.size
        rows = np.repeat(np.arange(nr, dtype=np.int32), np.diff(rp))
        if fmt == "CSR":
            assert np.array_equal(g.idx0, rp) and np.array_equal(g.idx1, ci) and np.array_equal(g.values, va)
        elif fmt in ("COO", "SCOO"):
            assert np.array_equal(g.idx0, rows) and np.array_equal(g.idx1, ci) and np.array_equal(g.values, va)
        elif fmt == "ELL":
            # MatrixELL(const MatrixCOO&) of the merged triplets (the oracle's conversion)
            e = orc.from_arrays("COO", nr, nc, va, rows, ci).convert("ELL").arrays
            assert g.max_col == e.max_col and np.array_equal(g.idx0, e.idx0) and np.array_equal(g.values, e.values)
        else:
            e = orc.from_arrays("COO", nr, nc, va, rows, ci).convert("DENSE").arrays
            assert np.array_equal(g.values, e.values)
    # the raw pattern of the benchmark matrix repeats 11 pairs
    raw = capi.generate("CSR", "cqmat", 100000, 100000, 10, 0.1, 0)
    assert raw.values.size - capi.generate("CSR", "cqmat_baseline", 100000, 100000, 10, 0.1, 0).values.size == 11
    with pytest.raises(capi.TbslaError):
        capi.generate("CSR", "cqmat_baseline", 10, 10, 3, 0.1, 0, pr=1, NR=2)
