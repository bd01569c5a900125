"""The allocation-free COO product (tbsla_coo_spmv_noalloc).

Callers whose device memory belongs to another allocator, or who cannot
afford the synchronisation of cudaMalloc/cudaFree, use this entry point: it
takes the caller's device buffers and keeps its scratch in a fixed array
inside the library.  The test calls it through the C ABI, twice in a row (the
array keeps the first call's contents), and compares with the allocating
path (tbsla_coo_create + tbsla_spmv_host) within the FP64 bound of the other
parity tests.  It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import assert_close

pytestmark = pytest.mark.gpu


class _Dev:
    def __init__(self, capi, a):
        self.capi = capi
        self.a = np.ascontiguousarray(a)
        self.p = C.c_void_p()
        L = capi.lib()
        capi.check(L.tbsla_device_alloc(C.byref(self.p), max(self.a.nbytes, 1)))
        capi.check(L.tbsla_memcpy_h2d(self.p, self.a.ctypes.data_as(C.c_void_p), self.a.nbytes, None))
        capi.check(L.tbsla_stream_sync(None))

    def get(self):
        out = np.empty_like(self.a)
        L = self.capi.lib()
        self.capi.check(L.tbsla_stream_sync(None))
        self.capi.check(L.tbsla_memcpy_d2h(out.ctypes.data_as(C.c_void_p), self.p, out.nbytes, None))
        self.capi.check(L.tbsla_stream_sync(None))
        return out

    def __del__(self):
        try:
            self.capi.lib().tbsla_device_free(self.p)
        except Exception:
            pass


def _noalloc(capi):
    L = capi.lib()
    f = L.tbsla_coo_spmv_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    f.restype = C.c_int
    return f


def test_no_alloc_coo_product_matches_allocating_path(gpu, orc):
    f = _noalloc(gpu)
    n = 30000
    # cqmat COO entries come in row order (MatrixCOO::fill_cqmat), as required
    g = gpu.generate("COO", "cqmat_stochastic", n, n, 12, 0.1, 1)
    assert np.all(np.diff(g.idx0) >= 0)
    rng = np.random.default_rng(21)
    rows, cols, vals = _Dev(gpu, g.idx0), _Dev(gpu, g.idx1), _Dev(gpu, g.values)
    m = gpu.DeviceMatrix.coo(n, n, g.idx0, g.idx1, g.values)
    scale_m = orc.from_arrays("COO", n, n, np.abs(g.values), g.idx0, g.idx1)
    for call in range(2):
        x = rng.uniform(-1, 1, n)
        dx, dy = _Dev(gpu, x), _Dev(gpu, np.full(n, np.nan))
        gpu.check(f(n, n, g.values.size, rows.p, cols.p, vals.p, dx.p, dy.p, None))
        y = dy.get()
        assert_close(y, m.spmv_host(x), scale_m.spmv(np.abs(x)), 1e-12, f"no-alloc call {call}")


def test_no_alloc_rejects_oversized_input(gpu):
    f = _noalloc(gpu)
    too_many = 16384 * 2304 + 1
    status = f(10, 10, too_many, None, None, None, None, None, None)
    assert status == 1  # TBSLA_ERR_INVALID_ARG, nothing launched
    assert b"exceeds" in gpu.lib().tbsla_last_error()
