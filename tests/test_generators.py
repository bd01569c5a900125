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
