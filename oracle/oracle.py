"""ctypes access to the checker libraries (test infrastructure only).

``Oracle`` wraps ``liboracle.so`` (the C restatement in ``tbsla_oracle.c``);
``Reference`` wraps ``_ref/libtbsla_ref.so`` (the TBSLA reference compiled from
its own sources, present only where those sources are).  Only the tests,
``__graft_entry__.smoke()`` and bench.py's CPU legs import this module; the
product package never does.

Both return matrices as :class:`Arrays`, the reference's storage layout
(values plus two index arrays, see Matrix{COO,CSR,ELL,...}.hpp).
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FORMATS = {"COO": 0, "SCOO": 1, "CSR": 2, "ELL": 3, "DENSE": 4}
FORMAT_NAMES = {v: k for k, v in FORMATS.items()}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


def reference_sources() -> str | None:
    """The reference's src/cpp directory when it is present on this host:
    $TBSLA_REF_SRC, else the default of the build recipe (oracle/Makefile)."""
    path = os.environ.get("TBSLA_REF_SRC")
    if not path:
        r = subprocess.run(["make", "-s", "-C", HERE, "print-ref-src"], capture_output=True, text=True)
        path = r.stdout.strip() if r.returncode == 0 else ""
    return path if path and os.path.isdir(os.path.join(path, "matrix")) else None


def build(ref: bool = True) -> None:
    """Compile liboracle.so (and _ref when the TBSLA sources are present)."""
    targets = ["oracle"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


@dataclass
class Arrays:
    fmt: str
    n_row: int = 0
    n_col: int = 0
    ln_row: int = 0
    ln_col: int = 0
    f_row: int = 0
    f_col: int = 0
    nnz: int = 0
    pr: int = 0
    pc: int = 0
    NR: int = 1
    NC: int = 1
    max_col: int = 0
    values: np.ndarray = field(default_factory=lambda: np.zeros(0))
    idx0: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    idx1: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))

    # reference field names
    @property
    def row(self):
        return self.idx0

    @property
    def col(self):
        return self.idx1

    @property
    def rowptr(self):
        return self.idx0

    @property
    def colidx(self):
        return self.idx1

    @property
    def columns(self):
        return self.idx0


class _OrcMatrix(C.Structure):
    _fields_ = [
        ("fmt", C.c_int),
        ("n_row", C.c_int), ("n_col", C.c_int), ("ln_row", C.c_int), ("ln_col", C.c_int),
        ("f_row", C.c_int), ("f_col", C.c_int), ("pr", C.c_int), ("pc", C.c_int),
        ("NR", C.c_int), ("NC", C.c_int),
        ("nnz", C.c_int64),
        ("max_col", C.c_int),
        ("n_values", C.c_int64), ("values", C.POINTER(C.c_double)),
        ("n_idx0", C.c_int64), ("idx0", C.POINTER(C.c_int)),
        ("n_idx1", C.c_int64), ("idx1", C.POINTER(C.c_int)),
    ]


def _copy(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class _Handle:
    """An orc_matrix owned by Python."""

    def __init__(self, lib, fmt: int):
        self.lib = lib
        self.s = _OrcMatrix()
        lib.orc_matrix_init(C.byref(self.s), fmt)

    def __del__(self):
        try:
            self.lib.orc_matrix_free(C.byref(self.s))
        except Exception:
            pass

    def arrays(self) -> Arrays:
        s = self.s
        return Arrays(FORMAT_NAMES[s.fmt], s.n_row, s.n_col, s.ln_row, s.ln_col, s.f_row, s.f_col,
                      s.nnz, s.pr, s.pc, s.NR, s.NC, s.max_col,
                      _copy(s.values, s.n_values, np.float64), _copy(s.idx0, s.n_idx0, np.int32),
                      _copy(s.idx1, s.n_idx1, np.int32))


def page_rank_exact_sums(rowptr, colidx, values, epsilon, beta, max_iteration, nodes=None):
    """Matrix::page_rank (src/cpp/matrix/Matrix.cpp:13-61), or with `nodes`
    Matrix::personalized_page_rank (Matrix.cpp:63-114), restated in numpy with
    the three reductions of each iteration (the sum of the previous iterate,
    the L1 change, the final sum) correctly rounded (math.fsum) instead of
    summed left to right.  The reference's left-to-right sums of n positive
    values carry a relative error up to (n-1) u (u = 2^-53), which at
    n = 2^20 moves its normalised vector by about 1e-11 in L1; this
    restatement is the iteration those sums approximate.  CSR arrays of a
    square matrix; returns (vector, iterations)."""
    import math
    n = rowptr.size - 1
    rp = np.asarray(rowptr, np.int64)
    rows = np.repeat(np.arange(n), np.diff(rp))
    vals = np.asarray(values, np.float64)
    cols = np.asarray(colidx, np.int64)

    def product(v):
        # each row summed in stored order (np.add.reduceat keeps the order
        # within a segment)
        t = vals * v[cols]
        out = np.zeros(n)
        nz = np.diff(rp) > 0
        out[nz] = np.add.reduceat(t, rp[:-1][nz]) if t.size else 0.0
        return out

    mark = None
    if nodes is not None:
        mark = np.zeros(n, bool)
        nd = np.asarray(nodes, np.int64)
        mark[nd[(nd >= 0) & (nd < n)]] = True
    b = np.full(n, 0.25 if nodes is not None else 1.0)
    it = 0
    while it < max_iteration:
        bt = b
        y = product(bt)
        if nodes is None:
            tele = math.fsum(bt) * ((1 - beta) / n)
            b = beta * y + tele
        else:
            tele = math.fsum(bt) * ((1 - beta) / len(nodes))
            b = beta * y
            b[mark] += tele
        b = b / b.max()
        err = math.fsum(np.abs(b - bt))
        it += 1
        if err < epsilon:
            break
    return b / math.fsum(b), it


def splitmix64_u01(seed: int, stream: int, count: int) -> np.ndarray:
    """u_k in [0, 1), k < count: SplitMix64 (Steele, Lea, Flood, OOPSLA 2014)
    output k from state (stream << 32) | seed, top 53 bits times 2^-53."""
    k = np.arange(1, count + 1, dtype=np.uint64)
    state = np.uint64(((stream & 0xFFFFFFFF) << 32) | (seed & 0xFFFFFFFF))
    with np.errstate(over="ignore"):
        z = state + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


class Oracle:
    """The C restatement (liboracle.so)."""

    def __init__(self, path: str | None = None):
        path = path or os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build(ref=False)
        L = C.CDLL(path)
        P = C.POINTER(_OrcMatrix)
        L.orc_matrix_init.argtypes = [P, C.c_int]
        L.orc_matrix_free.argtypes = [P]
        L.orc_fill_cdiag.argtypes = [P] + [C.c_int] * 7
        L.orc_fill_cqmat.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint] + [C.c_int] * 4
        L.orc_fill_cqmat_stochastic.argtypes = L.orc_fill_cqmat.argtypes
        L.orc_normalize_columns.argtypes = [P]
        L.orc_from_arrays.argtypes = [P, C.c_int, C.c_int, C.c_int, _dp, C.c_int64, _ip, C.c_int64,
                                      _ip, C.c_int64]
        L.orc_update_nnz.argtypes = [P]
        L.orc_convert.argtypes = [P, C.c_int, P]
        L.orc_spmv.argtypes = [P, _dp, _dp, C.c_int, C.c_int]
        L.orc_a_axpx.argtypes = [P, _dp, _dp, C.c_int, C.c_int]
        L.orc_page_rank.argtypes = [P, C.c_double, C.c_double, C.c_int, _dp, C.c_int]
        L.orc_page_rank.restype = C.c_int
        L.orc_personalized_page_rank.argtypes = [P, C.c_double, C.c_double, C.c_int, _ip, C.c_int,
                                                 _dp, C.c_int]
        L.orc_personalized_page_rank.restype = C.c_int
        L.orc_page_rank_dangling.argtypes = [C.c_int, _ip, _ip, _dp, _up, C.c_double, C.c_double,
                                             C.c_int, _dp, C.POINTER(C.c_double), C.c_int]
        L.orc_page_rank_dangling.restype = C.c_int
        vp = C.c_void_p
        L.orc_pagerank_teleport.argtypes = [C.c_int, _ip, _ip, _dp, _up, vp, C.c_double, C.c_double, C.c_int,
                                            _dp, C.POINTER(C.c_double)]
        L.orc_pagerank_teleport.restype = C.c_int
        L.orc_pagerank_adjoint.argtypes = [C.c_int, _ip, _ip, _dp, _up, vp, _dp, _dp, C.c_double, C.c_double,
                                           C.c_int, vp, vp]
        L.orc_pagerank_adjoint.restype = C.c_int
        L.orc_rmat_edges.argtypes = [C.c_int, C.c_int64, C.c_double, C.c_double, C.c_double,
                                     C.c_uint64, _ip, _ip]
        L.orc_cqmat_sum_columns.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_double, C.c_uint,
                                            _dp]
        L.orc_fnv1a.argtypes = [C.c_void_p, C.c_size_t]
        L.orc_fnv1a.restype = C.c_uint64
        self.L = L

    # -- matrices ------------------------------------------------------
    def _new(self, fmt: str) -> _Handle:
        return _Handle(self.L, FORMATS[fmt])

    def _wrap(self, h: _Handle) -> "OracleMatrix":
        return OracleMatrix(self, h)

    def fill_cqmat(self, fmt, n_row, n_col, c, q, seed_mult=1, pr=0, pc=0, NR=1, NC=1):
        h = self._new(fmt)
        self.L.orc_fill_cqmat(C.byref(h.s), n_row, n_col, c, q, seed_mult, pr, pc, NR, NC)
        return self._wrap(h)

    def fill_cqmat_stochastic(self, fmt, n_row, n_col, c, q, seed_mult=1, pr=0, pc=0, NR=1, NC=1):
        h = self._new(fmt)
        self.L.orc_fill_cqmat_stochastic(C.byref(h.s), n_row, n_col, c, q, seed_mult, pr, pc, NR, NC)
        return self._wrap(h)

    def fill_cdiag(self, fmt, n_row, n_col, cdiag, pr=0, pc=0, NR=1, NC=1):
        h = self._new(fmt)
        self.L.orc_fill_cdiag(C.byref(h.s), n_row, n_col, cdiag, pr, pc, NR, NC)
        return self._wrap(h)

    def from_arrays(self, fmt, n_row, n_col, values, idx0, idx1=None):
        h = self._new(fmt)
        v = np.ascontiguousarray(values, np.float64)
        a = np.ascontiguousarray(idx0, np.int32)
        b = np.ascontiguousarray(idx1 if idx1 is not None else np.zeros(0), np.int32)
        self.L.orc_from_arrays(C.byref(h.s), FORMATS[fmt], n_row, n_col, v, v.size, a, a.size, b, b.size)
        return self._wrap(h)

    def from_layout(self, fmt, geom, nnz, values, idx0, idx1):
        """A matrix with explicit geometry (n_row n_col ln_row ln_col f_row
        f_col pr pc NR NC max_col) and arrays in the reference layout."""
        m = self.from_arrays(fmt, geom[0], geom[1], values, idx0, idx1)
        s = m.h.s
        (s.ln_row, s.ln_col, s.f_row, s.f_col, s.pr, s.pc, s.NR, s.NC, s.max_col) = geom[2:11]
        s.nnz = nnz if nnz else s.n_values
        return m

    def rmat_edges(self, scale, m, a=0.57, b=0.19, c=0.19, seed=1):
        src = np.empty(m, np.int32)
        dst = np.empty(m, np.int32)
        self.L.orc_rmat_edges(scale, m, a, b, c, seed, src, dst)
        return src, dst

    def page_rank_dangling(self, rowptr, colidx, values, dangling, beta, tol, max_it, threads=1):
        n = rowptr.size - 1
        x = np.empty(n, np.float64)
        res = C.c_double(0)
        it = self.L.orc_page_rank_dangling(n, np.ascontiguousarray(rowptr, np.int32),
                                           np.ascontiguousarray(colidx, np.int32),
                                           np.ascontiguousarray(values, np.float64),
                                           np.ascontiguousarray(dangling, np.uint8), beta, tol, max_it,
                                           x, C.byref(res), threads)
        return x, it, res.value

    def pagerank_teleport(self, rowptr, colidx, values, dangling, v, beta, tol, max_it):
        """Affine (teleport) PageRank x = beta A x + (beta d.x + 1 - beta) v; v None = uniform."""
        n = rowptr.size - 1
        x = np.empty(n, np.float64)
        res = C.c_double(0)
        vv = None if v is None else np.ascontiguousarray(v, np.float64)
        it = self.L.orc_pagerank_teleport(n, np.ascontiguousarray(rowptr, np.int32),
                                          np.ascontiguousarray(colidx, np.int32),
                                          np.ascontiguousarray(values, np.float64),
                                          np.ascontiguousarray(dangling, np.uint8),
                                          None if vv is None else vv.ctypes.data, beta, tol, max_it, x, C.byref(res))
        return x, it, res.value

    def pagerank_adjoint(self, rowptr, colidx, values, dangling, v, x, w, beta, tol, max_it):
        """Gradients of L(x*) (w = dL/dx*) w.r.t. the values and the teleport vector."""
        n = rowptr.size - 1
        gvals = np.empty(values.size, np.float64)
        gv = np.empty(n, np.float64)
        vv = None if v is None else np.ascontiguousarray(v, np.float64)
        it = self.L.orc_pagerank_adjoint(n, np.ascontiguousarray(rowptr, np.int32),
                                         np.ascontiguousarray(colidx, np.int32),
                                         np.ascontiguousarray(values, np.float64),
                                         np.ascontiguousarray(dangling, np.uint8),
                                         None if vv is None else vv.ctypes.data,
                                         np.ascontiguousarray(x, np.float64), np.ascontiguousarray(w, np.float64),
                                         beta, tol, max_it, gvals.ctypes.data, gv.ctypes.data)
        return gvals, gv, it

    def baseline_cqmat(self, n_row, n_col, c, q, seed=0):
        """The benchmark's cqmat with merged duplicates and random values
        (the library's generator 3): the reference's fill_cqmat pattern
        (MatrixCSR.cpp:299-409, restated here), each (row, column) pair kept
        once in (row, column) order, value k = 1 - u(seed, stream 1, k).
        Returns CSR arrays (rowptr, colidx, values)."""
        a = self.fill_cqmat("CSR", n_row, n_col, c, q, seed).arrays
        rp, ci = a.rowptr.astype(np.int64), a.colidx.astype(np.int64)
        rows = np.repeat(np.arange(rp.size - 1, dtype=np.int64), np.diff(rp))
        key = np.unique(rows * max(n_col, 1) + ci)
        r = key // max(n_col, 1)
        col = (key % max(n_col, 1)).astype(np.int32)
        rowptr = np.zeros(n_row + 1, np.int64)
        np.add.at(rowptr, r + 1, 1)
        rowptr = np.cumsum(rowptr).astype(np.int32)
        values = 1.0 - splitmix64_u01(seed, 1, key.size)
        return rowptr, col, values

    def cqmat_sum_columns(self, nr, nc, c, q, seed_mult):
        s = np.zeros(nc, np.float64)
        self.L.orc_cqmat_sum_columns(nr, nc, c, q, seed_mult, s)
        return s

    def fnv1a(self, arr: np.ndarray) -> int:
        a = np.ascontiguousarray(arr)
        return int(self.L.orc_fnv1a(a.ctypes.data, a.nbytes))


class OracleMatrix:
    def __init__(self, orc: Oracle, h: _Handle):
        self.orc, self.h = orc, h

    @property
    def arrays(self) -> Arrays:
        return self.h.arrays()

    @property
    def n_row(self):
        return self.h.s.n_row

    @property
    def n_col(self):
        return self.h.s.n_col

    def update_nnz(self):
        self.orc.L.orc_update_nnz(C.byref(self.h.s))

    def normalize_columns(self):
        self.orc.L.orc_normalize_columns(C.byref(self.h.s))

    def convert(self, fmt: str) -> "OracleMatrix":
        h = self.orc._new(fmt)
        self.orc.L.orc_convert(C.byref(h.s), FORMATS[fmt], C.byref(self.h.s))
        return OracleMatrix(self.orc, h)

    def spmv(self, v, vect_incr=0, threads=1):
        r = np.zeros(self.n_row, np.float64)
        self.orc.L.orc_spmv(C.byref(self.h.s), np.ascontiguousarray(v, np.float64), r, vect_incr, threads)
        return r

    def a_axpx(self, v, vect_incr=0, threads=1):
        r = np.zeros(self.n_row, np.float64)
        self.orc.L.orc_a_axpx(C.byref(self.h.s), np.ascontiguousarray(v, np.float64), r, vect_incr, threads)
        return r

    def page_rank(self, epsilon, beta, max_iteration, threads=1):
        b = np.zeros(max(self.n_col, self.n_row) + 1, np.float64)
        it = self.orc.L.orc_page_rank(C.byref(self.h.s), epsilon, beta, max_iteration, b, threads)
        return b[: self.n_col].copy(), it

    def personalized_page_rank(self, epsilon, beta, max_iteration, nodes, threads=1):
        b = np.zeros(max(self.n_col, self.n_row) + 1, np.float64)
        nd = np.ascontiguousarray(nodes, np.int32)
        it = self.orc.L.orc_personalized_page_rank(C.byref(self.h.s), epsilon, beta, max_iteration, nd,
                                                   nd.size, b, threads)
        return b[: self.n_col].copy(), it


# --------------------------------------------------------------------------
# the reference itself (oracle/_ref)
# --------------------------------------------------------------------------
def parse_binary(fmt: str, buf: bytes) -> Arrays:
    """Parses the reference binary matrix layout (MatrixCSR.cpp:179-204 and
    the matching write() of each format)."""
    o = 0

    def take(f):
        nonlocal o
        vals = struct.unpack_from(f, buf, o)
        o += struct.calcsize(f)
        return vals

    n_row, n_col, ln_row, ln_col, f_row, f_col = take("<6i")
    (nnz,) = take("<q")
    pr, pc, NR, NC = take("<4i")
    a = Arrays(fmt, n_row, n_col, ln_row, ln_col, f_row, f_col, nnz, pr, pc, NR, NC)
    if fmt == "ELL":
        (a.max_col,) = take("<i")

    def arr(dtype):
        nonlocal o
        (n,) = take("<Q")
        x = np.frombuffer(buf, dtype=dtype, count=n, offset=o).copy()
        o += n * np.dtype(dtype).itemsize
        return x

    a.values = arr(np.float64)
    if fmt in ("COO", "SCOO", "CSR"):
        a.idx0 = arr(np.int32)
        a.idx1 = arr(np.int32)
    elif fmt == "ELL":
        a.idx0 = arr(np.int32)
    return a


def write_binary(a: Arrays) -> bytes:
    """The inverse of :func:`parse_binary`."""
    out = [struct.pack("<6i", a.n_row, a.n_col, a.ln_row, a.ln_col, a.f_row, a.f_col),
           struct.pack("<q", a.nnz), struct.pack("<4i", a.pr, a.pc, a.NR, a.NC)]
    if a.fmt == "ELL":
        out.append(struct.pack("<i", a.max_col))
    arrays = [a.values.astype(np.float64)]
    if a.fmt in ("COO", "SCOO", "CSR"):
        arrays += [a.idx0.astype(np.int32), a.idx1.astype(np.int32)]
    elif a.fmt == "ELL":
        arrays += [a.idx0.astype(np.int32)]
    for x in arrays:
        out.append(struct.pack("<Q", x.size))
        out.append(np.ascontiguousarray(x).tobytes())
    return b"".join(out)


def reference_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libtbsla_ref.so"))


class Reference:
    """The TBSLA reference classes through ref_harness.cpp."""

    def __init__(self, path: str | None = None):
        path = path or os.path.join(HERE, "_ref", "libtbsla_ref.so")
        L = C.CDLL(path)
        vp = C.c_void_p
        L.ref_set_threads.argtypes = [C.c_int]
        L.ref_new.argtypes = [C.c_int]
        L.ref_new.restype = vp
        L.ref_delete.argtypes = [vp, C.c_int]
        L.ref_fill_cqmat.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint] + [C.c_int] * 4
        L.ref_fill_cqmat_stochastic.argtypes = L.ref_fill_cqmat.argtypes
        L.ref_fill_cdiag.argtypes = [vp] + [C.c_int] * 7
        L.ref_normalize_columns.argtypes = [vp]
        L.ref_from_arrays.argtypes = [C.c_int, C.c_int, C.c_int, _dp, C.c_long, _ip, C.c_long, _ip, C.c_long]
        L.ref_from_arrays.restype = vp
        L.ref_update_nnz.argtypes = [vp]
        L.ref_convert.argtypes = [vp, C.c_int]
        L.ref_convert.restype = vp
        L.ref_serialize.argtypes = [vp, C.c_char_p, C.c_long]
        L.ref_serialize.restype = C.c_long
        L.ref_deserialize.argtypes = [C.c_int, C.c_char_p, C.c_long]
        L.ref_deserialize.restype = vp
        L.ref_read_mm.argtypes = [C.c_char_p]
        L.ref_read_mm.restype = vp
        L.ref_get_nnz.argtypes = [vp]
        L.ref_get_nnz.restype = C.c_long
        L.ref_get_n_row.argtypes = [vp]
        L.ref_get_n_col.argtypes = [vp]
        L.ref_spmv.argtypes = [vp, _dp, C.c_long, _dp, C.c_int]
        L.ref_a_axpx.argtypes = [vp, _dp, C.c_long, _dp]
        L.ref_page_rank.argtypes = [vp, C.c_double, C.c_double, C.c_int, _dp]
        L.ref_page_rank.restype = C.c_int
        L.ref_personalized_page_rank.argtypes = [vp, C.c_double, C.c_double, C.c_int, _ip, C.c_int, _dp]
        L.ref_personalized_page_rank.restype = C.c_int
        self.L = L

    def set_threads(self, n: int):
        self.L.ref_set_threads(n)

    def _wrap(self, p, fmt):
        return ReferenceMatrix(self, p, fmt)

    def new(self, fmt):
        return self._wrap(self.L.ref_new(FORMATS[fmt]), fmt)

    def fill_cqmat(self, fmt, n_row, n_col, c, q, seed_mult=1, pr=0, pc=0, NR=1, NC=1):
        m = self.new(fmt)
        self.L.ref_fill_cqmat(m.p, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC)
        return m

    def fill_cqmat_stochastic(self, fmt, n_row, n_col, c, q, seed_mult=1, pr=0, pc=0, NR=1, NC=1):
        m = self.new(fmt)
        self.L.ref_fill_cqmat_stochastic(m.p, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC)
        return m

    def fill_cdiag(self, fmt, n_row, n_col, cdiag, pr=0, pc=0, NR=1, NC=1):
        m = self.new(fmt)
        self.L.ref_fill_cdiag(m.p, n_row, n_col, cdiag, pr, pc, NR, NC)
        return m

    def from_arrays(self, fmt, n_row, n_col, values, idx0, idx1):
        v = np.ascontiguousarray(values, np.float64)
        a = np.ascontiguousarray(idx0, np.int32)
        b = np.ascontiguousarray(idx1, np.int32)
        return self._wrap(self.L.ref_from_arrays(FORMATS[fmt], n_row, n_col, v, v.size, a, a.size, b, b.size),
                          fmt)

    def read_mm(self, path: str):
        """MatrixCOO::readMM of the reference, or None where it throws."""
        p = self.L.ref_read_mm(path.encode())
        return self._wrap(p, "COO") if p else None

    def deserialize(self, fmt, buf: bytes):
        return self._wrap(self.L.ref_deserialize(FORMATS[fmt], buf, len(buf)), fmt)


class ReferenceMatrix:
    def __init__(self, ref: Reference, p, fmt: str):
        self.ref, self.p, self.fmt = ref, p, fmt

    def __del__(self):
        try:
            self.ref.L.ref_delete(self.p, FORMATS[self.fmt])
        except Exception:
            pass

    @property
    def n_row(self):
        return self.ref.L.ref_get_n_row(self.p)

    @property
    def n_col(self):
        return self.ref.L.ref_get_n_col(self.p)

    @property
    def nnz(self):
        return self.ref.L.ref_get_nnz(self.p)

    def serialized(self) -> bytes:
        """The bytes the reference's Matrix*::write produces."""
        n = self.ref.L.ref_serialize(self.p, None, 0)
        buf = C.create_string_buffer(n)
        self.ref.L.ref_serialize(self.p, buf, n)
        return buf.raw

    @property
    def arrays(self) -> Arrays:
        return parse_binary(self.fmt, self.serialized())

    def update_nnz(self):
        self.ref.L.ref_update_nnz(self.p)

    def normalize_columns(self):
        self.ref.L.ref_normalize_columns(self.p)

    def convert(self, fmt):
        return self.ref._wrap(self.ref.L.ref_convert(self.p, FORMATS[fmt]), fmt)

    def spmv(self, v, vect_incr=0):
        r = np.zeros(self.n_row, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        self.ref.L.ref_spmv(self.p, v, v.size, r, vect_incr)
        return r

    def a_axpx(self, v):
        r = np.zeros(self.n_row, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        self.ref.L.ref_a_axpx(self.p, v, v.size, r)
        return r

    def page_rank(self, epsilon, beta, max_iteration):
        b = np.zeros(max(self.n_col, self.n_row) + 1, np.float64)
        it = self.ref.L.ref_page_rank(self.p, epsilon, beta, max_iteration, b)
        return b[: self.n_col].copy(), it

    def personalized_page_rank(self, epsilon, beta, max_iteration, nodes):
        b = np.zeros(max(self.n_col, self.n_row) + 1, np.float64)
        nd = np.ascontiguousarray(nodes, np.int32)
        it = self.ref.L.ref_personalized_page_rank(self.p, epsilon, beta, max_iteration, nd, nd.size, b)
        return b[: self.n_col].copy(), it
