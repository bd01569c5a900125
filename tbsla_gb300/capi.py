"""ctypes binding of the C ABI in include/tbsla_gb300.h.

This is how Python callers (the tests, bench.py) reach the library: every
call goes through the same extern "C" entry points a C or C++ caller uses.
The library must have been built (``tbsla_gb300.build.build()``); loading
fails loudly otherwise -- there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtbsla_gb300.so")

FMT = {"COO": 0, "SCOO": 1, "CSR": 2, "ELL": 3, "DENSE": 4}
FMT_NAME = {v: k for k, v in FMT.items()}
F64, F32, BF16 = 0, 1, 2
STORE_F64, STORE_F32, STORE_BF16 = 1, 2, 4
PR_REFERENCE, PR_DANGLING, PR_TELEPORT = 0, 1, 2
TUNE_X_L2_KEEP, TUNE_PR_RELABEL, TUNE_X_L2_RANGE, TUNE_SHORT_ROWS, TUNE_TC_SPLIT, TUNE_SELL_ROWS = 0, 1, 2, 3, 4, 5
TUNE_DROP_SLICED_COPY = 6
GEN = {"cqmat": 0, "cdiag": 1, "cqmat_stochastic": 2, "cqmat_baseline": 3}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_vp = C.c_void_p


class TbslaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"tbsla status {status}: {msg}")
        self.status = status


class MatrixInfo(C.Structure):
    _fields_ = [("format", C.c_int), ("n_row", C.c_int), ("n_col", C.c_int), ("f_row", C.c_int),
                ("f_col", C.c_int), ("rows", C.c_int), ("max_col", C.c_int), ("stored", C.c_int64),
                ("stores", C.c_int), ("device_bytes", C.c_int64), ("kernels", C.c_int), ("slices", C.c_int)]


class PageRankParams(C.Structure):
    _fields_ = [("beta", C.c_double), ("tol", C.c_double), ("max_iter", C.c_int), ("mode", C.c_int),
                ("precision", C.c_int), ("check_every", C.c_int), ("accel", C.c_int)]


class AutotuneResult(C.Structure):
    _fields_ = [("candidates", C.c_int), ("best_ms", C.c_float), ("choice", C.c_int), ("value", C.c_double)]


class PageRankResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("iterations_f64", C.c_int), ("residual", C.c_double),
                ("converged", C.c_int)]


_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with tbsla_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    st = C.c_int
    P = _vp
    sig = {
        "tbsla_last_error": ([], C.c_char_p),
        "tbsla_status_string": ([C.c_int], C.c_char_p),
        "tbsla_version": ([], C.c_int),
        "tbsla_set_device": ([C.c_int], st),
        "tbsla_csr_create": ([C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, C.POINTER(P)], st),
        "tbsla_ell_create": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, C.c_int, C.POINTER(P)],
                             st),
        "tbsla_coo_create": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, _vp, _vp, _vp, C.c_int,
                              C.POINTER(P)], st),
        "tbsla_dense_create": ([C.c_int, C.c_int, C.c_int, C.c_int, _vp, C.c_int, C.POINTER(P)], st),
        "tbsla_matrix_destroy": ([P], st),
        "tbsla_matrix_set_variant": ([P, C.c_int], st),
        "tbsla_matrix_tune": ([P, C.c_int, C.c_double], st),
        "tbsla_matrix_info": ([P, C.POINTER(MatrixInfo)], st),
        "tbsla_matrix_device_status": ([P, C.POINTER(C.c_int)], st),
        "tbsla_generate_device": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint, C.c_int,
                                   C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(P)], st),
        "tbsla_spmv": ([P, _vp, _vp, C.c_int, _vp], st),
        "tbsla_spmv_ex": ([P, C.c_int, C.c_int, _vp, C.c_int, _vp, C.c_int, _vp], st),
        "tbsla_spmv_host": ([P, _vp, C.c_int64, _vp, C.c_int64, C.c_int], st),
        "tbsla_a_axpx": ([P, _vp, _vp, _vp, C.c_int, _vp], st),
        "tbsla_a_axpx_host": ([P, _vp, C.c_int64, _vp, C.c_int64, C.c_int], st),
        "tbsla_generate": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint, C.c_int,
                            C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int),
                            C.POINTER(C.c_int64), _vp, _vp, _vp], st),
        "tbsla_generate_matrix": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint, C.c_int,
                                   C.POINTER(P)], st),
        "tbsla_device_alloc": ([C.POINTER(_vp), C.c_size_t], st),
        "tbsla_device_free": ([_vp], st),
        "tbsla_memcpy_h2d": ([_vp, _vp, C.c_size_t, _vp], st),
        "tbsla_memcpy_d2h": ([_vp, _vp, C.c_size_t, _vp], st),
        "tbsla_stream_sync": ([_vp], st),
        "tbsla_host_alloc": ([C.POINTER(_vp), C.c_size_t], st),
        "tbsla_host_free": ([_vp], st),
        "tbsla_kernel_timing_enable": ([P, C.c_int], st),
        "tbsla_kernel_timing_read": ([P, C.POINTER(C.c_double), C.POINTER(C.c_int64)], st),
    }
    optional = {
        "tbsla_pagerank": ([P, C.POINTER(PageRankParams), _vp, C.POINTER(PageRankResult), _vp], st),
        "tbsla_pagerank_host": ([P, C.POINTER(PageRankParams), _vp, C.c_int64, C.POINTER(PageRankResult)],
                                st),
        "tbsla_personalized_pagerank_host": ([P, C.POINTER(PageRankParams), _vp, C.c_int, _vp, C.c_int64,
                                              C.POINTER(PageRankResult)], st),
        "tbsla_rmat_pagerank_matrix": ([C.c_int, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                        C.c_int, C.POINTER(P)], st),
        "tbsla_csr_download": ([P, _vp, _vp, _vp], st),
        "tbsla_spmv_transpose_ex": ([P, C.c_int, C.c_int, _vp, C.c_int, _vp, _vp], st),
        "tbsla_csr_grad_values": ([P, C.c_int, _vp, _vp, C.c_double, _vp, _vp], st),
        "tbsla_matrix_set_values": ([P, C.c_int, _vp, _vp], st),
        "tbsla_pagerank_teleport": ([P, C.POINTER(PageRankParams), _vp, _vp, C.POINTER(PageRankResult), _vp], st),
        "tbsla_pagerank_adjoint": ([P, C.POINTER(PageRankParams), _vp, _vp, _vp, _vp, _vp,
                                    C.POINTER(PageRankResult), _vp], st),
        "tbsla_batch_create": ([C.c_int, C.POINTER(_vp), C.POINTER(_vp)], st),
        "tbsla_batch_bind": ([_vp, C.c_int, C.POINTER(_vp), C.POINTER(_vp)], st),
        "tbsla_batch_set_mask": ([_vp, _vp], st),
        "tbsla_batch_tune": ([_vp, C.c_int], st),
        "tbsla_batch_spmv": ([_vp, _vp], st),
        "tbsla_batch_spmv_graph": ([_vp, _vp], st),
        "tbsla_batch_destroy": ([_vp], st),
        "tbsla_ppr_batched": ([P, C.POINTER(PageRankParams), C.c_int, _vp, _vp, C.c_int, _vp, _vp, _vp, _vp], st),
        "tbsla_ppr_batched_refined": ([P, C.POINTER(PageRankParams), C.c_int, _vp, _vp, C.c_int, _vp, _vp, _vp,
                                       _vp], st),
        "tbsla_autotune_spmv": ([P, C.c_int, C.POINTER(AutotuneResult)], st),
        "tbsla_matrix_read_file": ([C.c_char_p, C.c_int, C.c_int64, C.POINTER(P)], st),
        "tbsla_matrix_read_mm": ([C.c_char_p, C.c_int, C.POINTER(P)], st),
        "tbsla_coo_to_csr": ([P, C.c_int, C.POINTER(P)], st),
        "tbsla_coo_to_ell": ([P, C.c_int, C.POINTER(P)], st),
        "tbsla_coo_to_dense": ([P, C.c_int, C.POINTER(P)], st),
        "tbsla_coo_to_scoo": ([P, C.c_int, C.POINTER(P)], st),
        "tbsla_set_l2_fetch_granularity": ([C.c_int], st),
        "tbsla_get_l2_fetch_granularity": ([C.POINTER(C.c_int)], st),
        "tbsla_set_l2_persisting": ([C.c_size_t], st),
        "tbsla_get_l2_persisting": ([C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)], st),
        "tbsla_csr_normalize_columns": ([P, _vp], st),
        "tbsla_ell_download": ([P, _vp, _vp], st),
        "tbsla_dense_download": ([P, _vp], st),
        "tbsla_dense_spmm": ([P, C.c_int, C.c_int, _vp, C.c_int64, _vp, C.c_int64, _vp], st),
        "tbsla_spmm": ([P, C.c_int, C.c_int, _vp, C.c_int64, _vp, C.c_int64, _vp], st),
        "tbsla_autotune_batch": ([_vp, C.POINTER(AutotuneResult)], st),
        "tbsla_autotune_ppr": ([P, C.c_int, C.c_int, C.POINTER(AutotuneResult)], st),
    }
    for name, (args, res) in list(sig.items()) + list(optional.items()):
        if not hasattr(L, name):
            if name in sig:
                raise RuntimeError(f"{LIB_PATH} does not export {name}")
            continue
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _LIB = L
    return L


def check(status: int) -> None:
    if status != 0:
        raise TbslaError(status, lib().tbsla_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


@dataclass
class Generated:
    """A generated matrix in the reference's array layout."""
    fmt: str
    geom: list
    nnz: int
    values: np.ndarray = field(default_factory=lambda: np.zeros(0))
    idx0: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    idx1: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))

    @property
    def n_row(self):
        return self.geom[0]

    @property
    def n_col(self):
        return self.geom[1]

    @property
    def ln_row(self):
        return self.geom[2]

    @property
    def ln_col(self):
        return self.geom[3]

    @property
    def f_row(self):
        return self.geom[4]

    @property
    def f_col(self):
        return self.geom[5]

    @property
    def max_col(self):
        return self.geom[10]


def generate(fmt: str, gen: str, n_row: int, n_col: int, c: int, q: float = 0.0, seed_mult: int = 1,
             pr: int = 0, pc: int = 0, NR: int = 1, NC: int = 1) -> Generated:
    L = lib()
    sizes = (C.c_int64 * 3)()
    geom = (C.c_int * 11)()
    nnz = C.c_int64(0)
    args = (FMT[fmt], GEN[gen], n_row, n_col, c, q, seed_mult, pr, pc, NR, NC)
    check(L.tbsla_generate(*args, sizes, geom, C.byref(nnz), None, None, None))
    v = np.zeros(max(sizes[0], 1), np.float64)
    a = np.zeros(max(sizes[1], 1), np.int32)
    b = np.zeros(max(sizes[2], 1), np.int32)
    s2 = (C.c_int64 * 3)(v.size, a.size, b.size)
    check(L.tbsla_generate(*args, s2, geom, C.byref(nnz), _ptr(v), _ptr(a), _ptr(b)))
    return Generated(fmt, list(geom), nnz.value, v[: sizes[0]].copy(), a[: sizes[1]].copy(),
                     b[: sizes[2]].copy())


class DeviceMatrix:
    """Owns one tbsla_matrix_t handle."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        self.close()

    def close(self):
        if getattr(self, "h", None):
            lib().tbsla_matrix_destroy(self.h)
            self.h = None

    # -- construction -------------------------------------------------
    @classmethod
    def csr(cls, n_row, n_col, rowptr, colidx, values, f_col=0, stores=STORE_F64, rows=None):
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        colidx = np.ascontiguousarray(colidx, np.int32)
        values = np.ascontiguousarray(values, np.float64)
        rows = rowptr.size - 1 if rows is None else rows
        h = _vp()
        check(lib().tbsla_csr_create(n_row, n_col, f_col, max(rows, 0), _ptr(rowptr), _ptr(colidx),
                                     _ptr(values), stores, C.byref(h)))
        return cls(h)

    @classmethod
    def ell(cls, n_row, n_col, max_col, columns, values, f_col=0, stores=STORE_F64, rows=None):
        columns = np.ascontiguousarray(columns, np.int32)
        values = np.ascontiguousarray(values, np.float64)
        if rows is None:
            rows = min(n_row, values.size // max_col) if max_col else 0
        h = _vp()
        check(lib().tbsla_ell_create(n_row, n_col, f_col, rows, max_col, _ptr(columns), _ptr(values), stores,
                                     C.byref(h)))
        return cls(h)

    @classmethod
    def coo(cls, n_row, n_col, row, col, values, f_row=0, f_col=0, stores=STORE_F64):
        row = np.ascontiguousarray(row, np.int32)
        col = np.ascontiguousarray(col, np.int32)
        values = np.ascontiguousarray(values, np.float64)
        h = _vp()
        check(lib().tbsla_coo_create(n_row, n_col, f_row, f_col, values.size, _ptr(row), _ptr(col),
                                     _ptr(values), stores, C.byref(h)))
        return cls(h)

    @classmethod
    def dense(cls, n_row, n_col, ln_row, ln_col, values, stores=STORE_F64):
        values = np.ascontiguousarray(values, np.float64)
        h = _vp()
        check(lib().tbsla_dense_create(n_row, n_col, ln_row, ln_col, _ptr(values), stores, C.byref(h)))
        return cls(h)

    @classmethod
    def generate(cls, fmt: str, gen: str, n_row: int, n_col: int, c: int, q: float = 0.0, seed_mult: int = 1,
                 stores=STORE_F64):
        """One pass: generate on the host and upload (tbsla_generate_matrix)."""
        h = _vp()
        check(lib().tbsla_generate_matrix(FMT[fmt], GEN[gen], n_row, n_col, c, q, seed_mult, stores, C.byref(h)))
        return cls(h)

    @classmethod
    def generate_device(cls, fmt: str, gen: str, n_row: int, n_col: int, c: int, q: float = 0.0,
                        seed_mult: int = 1, pr: int = 0, pc: int = 0, NR: int = 1, NC: int = 1, stores=STORE_F64):
        """Generated on the device where the generator allows (tbsla_generate_device)."""
        h = _vp()
        check(lib().tbsla_generate_device(FMT[fmt], GEN[gen], n_row, n_col, c, q, seed_mult, pr, pc, NR, NC, stores,
                                          C.byref(h)))
        return cls(h)

    @classmethod
    def from_generated(cls, g: Generated, stores=STORE_F64):
        if g.fmt == "CSR":
            return cls.csr(g.n_row, g.n_col, g.idx0 if g.idx0.size else np.zeros(1, np.int32), g.idx1, g.values,
                           f_col=g.f_col, stores=stores, rows=max(g.idx0.size - 1, 0))
        if g.fmt == "ELL":
            return cls.ell(g.n_row, g.n_col, g.max_col, g.idx0, g.values, f_col=g.f_col, stores=stores,
                           rows=min(g.ln_row, g.values.size // g.max_col) if g.max_col else 0)
        if g.fmt == "COO":
            return cls.coo(g.n_row, g.n_col, g.idx0, g.idx1, g.values, stores=stores)
        if g.fmt == "SCOO":
            return cls.coo(g.n_row, g.n_col, g.idx0, g.idx1, g.values, f_row=g.f_row, f_col=g.f_col,
                           stores=stores)
        return cls.dense(g.n_row, g.n_col, g.ln_row if g.values.size else 0, g.ln_col, g.values, stores=stores)

    # -- queries --------------------------------------------------------
    def info(self) -> MatrixInfo:
        i = MatrixInfo()
        check(lib().tbsla_matrix_info(self.h, C.byref(i)))
        return i

    # -- products on host vectors -------------------------------------
    def spmv_host(self, x: np.ndarray, vect_incr: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(max(self.info().n_row, 1), np.float64)
        check(lib().tbsla_spmv_host(self.h, _ptr(x), x.size, _ptr(y), y.size, vect_incr))
        return y[: self.info().n_row]

    def a_axpx_host(self, x: np.ndarray, vect_incr: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        n = self.info().n_row
        y = np.zeros(max(n, 1), np.float64)
        check(lib().tbsla_a_axpx_host(self.h, _ptr(x), x.size, _ptr(y), y.size, vect_incr))
        return y[:n]

    # -- products on device pointers (ints, e.g. torch data_ptr) ------
    def spmv(self, d_x: int, d_y: int, vect_incr: int = 0, stream: int | None = None):
        check(lib().tbsla_spmv(self.h, d_x, d_y, vect_incr, stream))

    def spmv_ex(self, store: int, x_type: int, d_x: int, y_type: int, d_y: int, vect_incr: int = 0,
                stream: int | None = None):
        check(lib().tbsla_spmv_ex(self.h, store, x_type, d_x, y_type, d_y, vect_incr, stream))

    def a_axpx(self, d_x: int, d_r: int, d_tmp: int, vect_incr: int = 0, stream: int | None = None):
        check(lib().tbsla_a_axpx(self.h, d_x, d_r, d_tmp, vect_incr, stream))

    # -- PageRank --------------------------------------------------------
    def pagerank_host(self, beta=0.85, tol=1e-10, max_iter=10000, mode=PR_DANGLING, precision=F64,
                      check_every=0, accel=0):
        p = PageRankParams(beta, tol, max_iter, mode, precision, check_every, accel)
        r = PageRankResult()
        n = self.info().n_col
        out = np.zeros(max(n, 1), np.float64)
        check(lib().tbsla_pagerank_host(self.h, C.byref(p), _ptr(out), out.size, C.byref(r)))
        return out[:n], r

    def pagerank(self, d_out: int, beta=0.85, tol=1e-10, max_iter=10000, mode=PR_DANGLING, precision=F64,
                 check_every=0, stream: int | None = None, accel=0):
        p = PageRankParams(beta, tol, max_iter, mode, precision, check_every, accel)
        r = PageRankResult()
        check(lib().tbsla_pagerank(self.h, C.byref(p), d_out, C.byref(r), stream))
        return r

    def personalized_pagerank_host(self, nodes, beta=0.85, tol=1e-10, max_iter=10000):
        p = PageRankParams(beta, tol, max_iter, PR_REFERENCE, F64, 0)
        r = PageRankResult()
        nd = np.ascontiguousarray(nodes, np.int32)
        n = self.info().n_col
        out = np.zeros(max(n, 1), np.float64)
        check(lib().tbsla_personalized_pagerank_host(self.h, C.byref(p), _ptr(nd), nd.size, _ptr(out),
                                                     out.size, C.byref(r)))
        return out[:n], r

    # ---- differentiation (device pointers as ints, stream as int or None)
    def spmv_transpose_ex(self, store: int, x_type: int, d_x: int, y_type: int, d_y: int, stream=None):
        check(lib().tbsla_spmv_transpose_ex(self.h, store, x_type, d_x, y_type, d_y, stream))

    def grad_values(self, dtype: int, d_a: int, d_b: int, scale: float, d_out: int, stream=None):
        check(lib().tbsla_csr_grad_values(self.h, dtype, d_a, d_b, float(scale), d_out, stream))

    def set_values(self, dtype: int, d_values: int, stream=None):
        check(lib().tbsla_matrix_set_values(self.h, dtype, d_values, stream))

    def pagerank_teleport(self, d_v: int, d_out: int, beta=0.85, tol=1e-12, max_iter=10000, stream=None, accel=0):
        p = PageRankParams(beta, tol, max_iter, PR_TELEPORT, F64, 0, accel)
        r = PageRankResult()
        check(lib().tbsla_pagerank_teleport(self.h, C.byref(p), d_v, d_out, C.byref(r), stream))
        return r

    def pagerank_adjoint(self, d_v, d_x: int, d_w: int, d_grad_values, d_grad_v, beta=0.85, tol=1e-12,
                         max_iter=10000, stream=None, accel=0):
        p = PageRankParams(beta, tol, max_iter, PR_TELEPORT, F64, 0, accel)
        r = PageRankResult()
        check(lib().tbsla_pagerank_adjoint(self.h, C.byref(p), d_v, d_x, d_w, d_grad_values, d_grad_v,
                                           C.byref(r), stream))
        return r

    def tune(self, knob: int, value: float):
        check(lib().tbsla_matrix_tune(self.h, knob, float(value)))

    def autotune_spmv(self, store: int = F64) -> AutotuneResult:
        r = AutotuneResult()
        check(lib().tbsla_autotune_spmv(self.h, store, C.byref(r)))
        return r

    def autotune_ppr(self, k: int, precision: int = F64) -> AutotuneResult:
        r = AutotuneResult()
        check(lib().tbsla_autotune_ppr(self.h, k, precision, C.byref(r)))
        return r

    def set_variant(self, variant: int):
        check(lib().tbsla_matrix_set_variant(self.h, variant))

    def timing(self, enable: bool = True):
        check(lib().tbsla_kernel_timing_enable(self.h, int(enable)))

    def timing_read(self):
        ms, n = C.c_double(0), C.c_int64(0)
        check(lib().tbsla_kernel_timing_read(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def csr_download(self):
        i = self.info()
        rp = np.zeros(i.rows + 1, np.int32)
        ci = np.zeros(max(i.stored, 1), np.int32)
        vv = np.zeros(max(i.stored, 1), np.float64)
        check(lib().tbsla_csr_download(self.h, _ptr(rp), _ptr(ci), _ptr(vv)))
        return rp, ci[: i.stored], vv[: i.stored]

    def dense_spmm(self, store: int, k: int, d_X: int, ldx: int, d_Y: int, ldy: int, stream=None):
        check(lib().tbsla_dense_spmm(self.h, store, k, d_X, ldx, d_Y, ldy, stream))

    def device_status(self) -> int:
        """Nonzero when a kernel of this handle gave up a bounded wait
        (synchronises the device; clears the status)."""
        st = C.c_int(0)
        check(lib().tbsla_matrix_device_status(self.h, C.byref(st)))
        return st.value

    def spmm(self, store: int, k: int, d_X: int, ldx: int, d_Y: int, ldy: int, stream=None):
        """Y = A X for k row-major vectors (CSR, COO, SCOO)."""
        check(lib().tbsla_spmm(self.h, store, k, d_X, ldx, d_Y, ldy, stream))

    def to_csr(self, stores=STORE_F64):
        """CSR handle converted on the device from this COO / SCOO handle."""
        h = _vp()
        check(lib().tbsla_coo_to_csr(self.h, stores, C.byref(h)))
        return DeviceMatrix(h)

    def to_ell(self, stores=STORE_F64):
        """ELL handle converted on the device from this COO / SCOO handle."""
        h = _vp()
        check(lib().tbsla_coo_to_ell(self.h, stores, C.byref(h)))
        return DeviceMatrix(h)

    def to_dense(self, stores=STORE_F64):
        """DENSE handle converted on the device from this COO / SCOO handle."""
        h = _vp()
        check(lib().tbsla_coo_to_dense(self.h, stores, C.byref(h)))
        return DeviceMatrix(h)

    def to_scoo(self, stores=STORE_F64):
        """SCOO handle copied on the device from this COO / SCOO handle."""
        h = _vp()
        check(lib().tbsla_coo_to_scoo(self.h, stores, C.byref(h)))
        return DeviceMatrix(h)

    def normalize_columns(self, stream=None):
        """MatrixCSR::normalize_columns on the device (CSR handles)."""
        check(lib().tbsla_csr_normalize_columns(self.h, stream))

    def ell_download(self):
        """(columns, values) of an ELL handle, row-major rows x max_col."""
        i = self.info()
        cols = np.zeros(max(i.rows * i.max_col, 1), np.int32)
        vals = np.zeros(max(i.rows * i.max_col, 1), np.float64)
        check(lib().tbsla_ell_download(self.h, _ptr(cols), _ptr(vals)))
        return cols[: i.rows * i.max_col], vals[: i.rows * i.max_col]

    def dense_download(self):
        """values of a DENSE handle (stored entries, row-major)."""
        i = self.info()
        vals = np.zeros(max(i.stored, 1), np.float64)
        check(lib().tbsla_dense_download(self.h, _ptr(vals)))
        return vals[: i.stored]

    @classmethod
    def read_file(cls, path: str, fmt: str, seek: int = 0):
        h = _vp()
        check(lib().tbsla_matrix_read_file(path.encode(), FMT[fmt], seek, C.byref(h)))
        return cls(h)

    @classmethod
    def read_mm(cls, path: str, fmt: str):
        h = _vp()
        check(lib().tbsla_matrix_read_mm(path.encode(), FMT[fmt], C.byref(h)))
        return cls(h)

    @classmethod
    def rmat_pagerank(cls, scale, m, a=0.57, b=0.19, c=0.19, seed=1, stores=STORE_F64):
        h = _vp()
        check(lib().tbsla_rmat_pagerank_matrix(scale, m, a, b, c, seed, stores, C.byref(h)))
        return cls(h)


class Batch:
    """Several CSR DeviceMatrix objects multiplied in one launch (tbsla_batch_*)."""

    def __init__(self, members):
        self.members = list(members)  # kept alive while the batch exists
        arr = (_vp * len(self.members))(*[m.h for m in self.members])
        self.h = _vp()
        check(lib().tbsla_batch_create(len(self.members), arr, C.byref(self.h)))

    def bind(self, store: int, d_x, d_y):
        xs = (_vp * len(d_x))(*d_x)
        ys = (_vp * len(d_y))(*d_y)
        check(lib().tbsla_batch_bind(self.h, store, xs, ys))

    def set_mask(self, d_mask):
        check(lib().tbsla_batch_set_mask(self.h, d_mask))

    def tune(self, blocks_per_sm: int):
        check(lib().tbsla_batch_tune(self.h, blocks_per_sm))

    def autotune(self) -> "AutotuneResult":
        r = AutotuneResult()
        check(lib().tbsla_autotune_batch(self.h, C.byref(r)))
        return r

    def spmv(self, stream=None, graph=False):
        f = lib().tbsla_batch_spmv_graph if graph else lib().tbsla_batch_spmv
        check(f(self.h, stream))

    def close(self):
        if self.h:
            lib().tbsla_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ppr_batched(A, seed_sets, d_out: int, beta=0.85, tol=1e-12, max_iter=10000, precision=F64, tile=0,
                stream=None, check_every=0, refined=False, accel=0):
    """k personalized PageRank vectors of A solved together; returns (iterations, residuals).
    refined: FP32 sweeps with FP64 defect correction (tbsla_ppr_batched_refined);
    accel: 1 for Anderson-accelerated solves (per vector)."""
    k = len(seed_sets)
    offsets = np.zeros(k + 1, np.int32)
    offsets[1:] = np.cumsum([len(s) for s in seed_sets])
    nodes = np.ascontiguousarray(np.concatenate([np.asarray(s, np.int32) for s in seed_sets]), np.int32)
    its = np.zeros(k, np.int32)
    res = np.zeros(k, np.float64)
    p = PageRankParams(beta, tol, max_iter, PR_TELEPORT, precision, check_every, accel)
    fn = lib().tbsla_ppr_batched_refined if refined else lib().tbsla_ppr_batched
    check(fn(A.h, C.byref(p), k, _ptr(nodes), _ptr(offsets), tile, d_out, _ptr(its), _ptr(res), stream))
    return its, res
