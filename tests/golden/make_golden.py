"""Writes tests/golden/golden.json from the TBSLA reference itself.

Run where the reference sources are present (they are compiled into
oracle/_ref by ``make -C oracle ref``):

    python tests/golden/make_golden.py

Every record is produced by calling the reference's own classes through
oracle/ref_harness.cpp; nothing is computed by this repository's code.
Arrays are fingerprinted with FNV-1a (64-bit) over their little-endian
bytes; small result vectors are stored in full (repr of the doubles).

Contents
  known_answer   the 5x5 COO/CSR products of src/cpp/tests/coo.cpp:8-31
                 and src/cpp/tests/csr.cpp:8-31
  generators     array fingerprints of fill_cqmat / fill_cqmat_stochastic /
                 fill_cdiag for every format over the shapes of
                 src/cpp/tests/test_spmv_cqmat.cpp:193-225 (subset of q)
  spmv_iota      spmv(x = 0..n-1) of the same matrices (test_spmv_cqmat.cpp:53-58)
  page_rank      page_rank / personalized_page_rank vectors of the
                 stochastic cqmat matrices of src/cpp/tests/test_page_rank.cpp:118-131
  cfg1           n=100000, c=10, q=0.1, seed 0 CSR arrays + spmv of a
                 seeded x
  cfg2           n=2^24, c=16, q=0.1, seed 0 CSR array fingerprints
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference, build, reference_available  # noqa: E402

FORMATS = ["COO", "SCOO", "CSR", "ELL", "DENSE"]
SHAPES = [(10, 5, 8), (5, 10, 7), (10, 10, 12), (10, 10, 3), (10, 5, 3), (10, 5, 6), (30, 30, 6),
          (20, 30, 10), (30, 20, 14), (10, 10, 0), (30, 30, 24)]
QS = [0.0, 0.1, 1.0]
SEEDS = [0, 2]
BLOCKS = [(0, 0, 1, 1), (1, 0, 2, 2), (0, 1, 2, 3)]


def fnv(a: np.ndarray) -> str:
    h = 1469598103934665603
    for b in np.ascontiguousarray(a).tobytes():
        h ^= b
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return f"{h:016x}"


def fnv_fast(a: np.ndarray) -> str:
    """FNV-1a through liboracle's C loop (same function, large arrays)."""
    from oracle.oracle import Oracle
    return f"{Oracle().fnv1a(a):016x}"


def arrays_record(a, big=False) -> dict:
    f = fnv_fast if big else fnv
    return {"geom": [a.n_row, a.n_col, a.ln_row, a.ln_col, a.f_row, a.f_col, a.pr, a.pc, a.NR, a.NC,
                     a.max_col], "nnz": int(a.nnz), "n_values": int(a.values.size),
            "n_idx0": int(a.idx0.size), "n_idx1": int(a.idx1.size),
            "values": f(a.values), "idx0": f(a.idx0), "idx1": f(a.idx1)}


def main() -> None:
    build(ref=True)
    if not reference_available():
        sys.exit("the reference build (oracle/_ref) is not available")
    R = Reference()
    R.set_threads(1)
    out: dict = {"note": "generated from the TBSLA reference by tests/golden/make_golden.py"}

    # known answers (coo.cpp / csr.cpp)
    vals = np.arange(1, 11, dtype=np.float64)
    x = np.arange(1, 6, dtype=np.float64)
    coo = R.from_arrays("COO", 5, 5, vals, [0, 0, 0, 1, 2, 3, 3, 4, 4, 4], [0, 1, 4, 2, 1, 1, 3, 0, 2, 4])
    csr = R.from_arrays("CSR", 5, 5, vals, [0, 3, 4, 5, 7, 10], [0, 1, 4, 2, 1, 1, 3, 0, 2, 4])
    out["known_answer"] = {
        "values": vals.tolist(), "row": [0, 0, 0, 1, 2, 3, 3, 4, 4, 4], "rowptr": [0, 3, 4, 5, 7, 10],
        "col": [0, 1, 4, 2, 1, 1, 3, 0, 2, 4], "x": x.tolist(),
        "coo": coo.spmv(x).tolist(), "csr": csr.spmv(x).tolist()}

    gens, spmv_iota = [], []
    for (nr, nc, c) in SHAPES:
        for s in SEEDS:
            for q in QS:
                for f in FORMATS:
                    for gen in ("cqmat", "cqmat_stochastic"):
                        for blk in BLOCKS:
                            m = (R.fill_cqmat if gen == "cqmat" else R.fill_cqmat_stochastic)(f, nr, nc, c, q, s,
                                                                                              *blk)
                            rec = arrays_record(m.arrays)
                            rec.update({"format": f, "gen": gen, "shape": [nr, nc, c], "q": q, "seed": s,
                                        "block": list(blk)})
                            gens.append(rec)
                    if f != "COO" or True:
                        m = R.fill_cqmat(f, nr, nc, c, q, s)
                        y = m.spmv(np.arange(nc, dtype=np.float64))
                        spmv_iota.append({"format": f, "shape": [nr, nc, c], "q": q, "seed": s,
                                          "y": y.tolist()})
        for f in FORMATS:
            for cd in (0, 1, 2, 5, 9):
                for blk in BLOCKS:
                    m = R.fill_cdiag(f, nr, nc, cd, *blk)
                    rec = arrays_record(m.arrays)
                    rec.update({"format": f, "gen": "cdiag", "shape": [nr, nc, cd], "block": list(blk)})
                    gens.append(rec)
    out["generators"] = gens
    out["spmv_iota"] = spmv_iota

    prs = []
    for (nr, nc, c) in [(10, 10, 12), (10, 10, 3), (30, 30, 6), (30, 30, 24)]:
        for s in (0, 1):
            for q in (0.0, 0.5):
                for f in FORMATS:
                    m = R.fill_cqmat_stochastic(f, nr, nc, c, q, s)
                    b, it = m.page_rank(0.85, 0.01, 10)   # argument order of test_page_rank.cpp:28
                    b2, it2 = m.page_rank(1e-10, 0.85, 500)
                    p, itp = m.personalized_page_rank(0.85, 0.01, 10, [1, 3])
                    prs.append({"format": f, "shape": [nr, nc, c], "q": q, "seed": s,
                                "swapped": {"it": it, "b": [repr(float(v)) for v in b]},
                                "tight": {"it": it2, "b": [repr(float(v)) for v in b2]},
                                "ppr": {"it": itp, "b": [repr(float(v)) for v in p]}})
    out["page_rank"] = prs

    # cfg1: cqmat n=1e5 c=10 q=0.1 seed 0, CSR
    t = time.time()
    m = R.fill_cqmat("CSR", 100000, 100000, 10, 0.1, 0)
    a = m.arrays
    x = np.random.default_rng(0).random(100000)
    R.set_threads(8)
    y = m.spmv(x)
    out["cfg1"] = {"arrays": arrays_record(a, big=True), "x_seed": 0, "y_fnv": fnv_fast(y),
                   "y_sum": repr(float(y.sum())), "y_head": [repr(float(v)) for v in y[:8]]}
    # cfg2: cqmat n=2^24 c=16 q=0.1 seed 0, CSR (fingerprints only)
    m = R.fill_cqmat("CSR", 1 << 24, 1 << 24, 16, 0.1, 0)
    out["cfg2"] = {"arrays": arrays_record(m.arrays, big=True)}
    print(f"cfg1+cfg2 in {time.time() - t:.1f}s")

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(path, "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print(f"wrote {path}: {os.path.getsize(path)} bytes, {len(gens)} generator records")


if __name__ == "__main__":
    main()
