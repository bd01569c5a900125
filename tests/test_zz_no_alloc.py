"""The allocation-free COO product (tbsla_coo_spmv_noalloc).

Callers whose device memory belongs to another allocator, or who cannot
afford the synchronisation of cudaMalloc/cudaFree, use this entry point: it
takes the caller's device buffers and keeps its scratch in a fixed array
inside the library.  The tests call it through the C ABI, twice in a row (the
array keeps the first call's contents), and compare with the allocating
path (tbsla_coo_create + tbsla_spmv_host) and with the oracle's COO product
within the FP64 bound of the other parity tests; then at exactly the array's
capacity followed by a smaller call (stale carries of the larger call must
not leak into it), with the device's free memory unchanged across warmed-up
calls.  They live in their own file, collected last.
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
    o = orc.from_arrays("COO", n, n, g.values, g.idx0, g.idx1)
    for call in range(2):
        x = rng.uniform(-1, 1, n)
        dx, dy = _Dev(gpu, x), _Dev(gpu, np.full(n, np.nan))
        gpu.check(f(n, n, g.values.size, rows.p, cols.p, vals.p, dx.p, dy.p, None))
        y = dy.get()
        scale = scale_m.spmv(np.abs(x))
        assert_close(y, m.spmv_host(x), scale, 1e-12, f"no-alloc call {call} vs allocating path")
        assert_close(y, o.spmv(x), scale, 1e-12, f"no-alloc call {call} vs oracle")


# the array's capacity: 16384 tiles of 2304 stored entries
CAP = 16384 * 2304


def _device_free_bytes():
    """Free device memory seen by the driver in the current context."""
    L = C.CDLL("libcuda.so.1")
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert L.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
    return free.value


def _banded_coo(n_row, n_col, per_row, seed):
    """Row-sorted triplets: per_row entries in each row, scattered columns."""
    rng = np.random.default_rng(seed)
    row = np.repeat(np.arange(n_row, dtype=np.int32), per_row)
    col = ((row.astype(np.int64) * 7 + rng.integers(0, n_col, row.size)) % n_col).astype(np.int32)
    val = rng.uniform(-1, 1, row.size)
    return row, col, val


def test_no_alloc_at_capacity_then_smaller(gpu, orc):
    f = _noalloc(gpu)
    rng = np.random.default_rng(5)
    big_rows = CAP // 16
    cases = [(big_rows, 1 << 20, 16, 1), (3001, 2000, 7, 2)]
    runs = []
    for (nr, nc, per_row, seed) in cases:
        row, col, val = _banded_coo(nr, nc, per_row, seed)
        runs.append((nr, nc, row, col, val, _Dev(gpu, row), _Dev(gpu, col), _Dev(gpu, val)))
    assert runs[0][2].size == CAP  # the last slot of every carry array is used
    # capacity, smaller, capacity again, smaller again
    for k, (nr, nc, row, col, val, drow, dcol, dval) in enumerate(runs + runs):
        x = rng.uniform(-1, 1, nc)
        dx, dy = _Dev(gpu, x), _Dev(gpu, np.full(nr, np.nan))
        free_before = _device_free_bytes()
        gpu.check(f(nr, nc, row.size, drow.p, dcol.p, dval.p, dx.p, dy.p, None))
        gpu.check(gpu.lib().tbsla_stream_sync(None))
        free_after = _device_free_bytes()
        if k >= 2:  # warmed up: the kernels are loaded, nothing else may take memory
            assert free_after == free_before, (k, free_before - free_after)
        y = dy.get()
        o = orc.from_arrays("COO", nr, nc, val, row, col)
        scale = orc.from_arrays("COO", nr, nc, np.abs(val), row, col).spmv(np.abs(x), threads=8)
        assert_close(y, o.spmv(x, threads=8), scale, 1e-12, f"no-alloc call {k} ({nr} rows) vs oracle")


def test_no_alloc_rejects_oversized_input(gpu):
    f = _noalloc(gpu)
    too_many = 16384 * 2304 + 1
    status = f(10, 10, too_many, None, None, None, None, None, None)
    assert status == 1  # TBSLA_ERR_INVALID_ARG, nothing launched
    assert b"exceeds" in gpu.lib().tbsla_last_error()


def test_no_alloc_checks_its_input(gpu):
    """Rows that decrease or leave [0, n_row), and columns outside [0, n_col),
    are caught by the call's input check: the product stands down before
    reading x, y is all NaN and tbsla_coo_spmv_noalloc_status reports 1; a
    valid call afterwards reports 0.  (x is allocated 64 entries longer than
    n_col, so that the out-of-range column stays inside the buffer.)"""
    f = _noalloc(gpu)
    L = gpu.lib()
    L.tbsla_coo_spmv_noalloc_status.argtypes = [C.POINTER(C.c_int), C.c_void_p]

    def status():
        bad = C.c_int(-1)
        gpu.check(L.tbsla_coo_spmv_noalloc_status(C.byref(bad), None))
        return bad.value

    nr, nc = 5000, 4000
    row, col, val = _banded_coo(nr, nc, 5, 11)
    x = np.random.default_rng(12).uniform(-1, 1, nc + 64)
    dx = _Dev(gpu, x)
    bad_rows = row.copy()
    bad_rows[1000], bad_rows[1001] = bad_rows[1001] + 1, bad_rows[1000]  # a decrease, rows in range
    bad_cols = col.copy()
    bad_cols[777] = nc  # one past the last column
    high_row = row.copy()
    high_row[-1] = nr  # one past the last row (the last row stays nondecreasing)
    for (r, c) in ((bad_rows, col), (row, bad_cols), (high_row, col)):
        drow, dcol, dval = _Dev(gpu, r), _Dev(gpu, c), _Dev(gpu, val)
        dy = _Dev(gpu, np.zeros(nr))
        gpu.check(f(nr, nc, r.size, drow.p, dcol.p, dval.p, dx.p, dy.p, None))
        assert status() == 1
        assert np.isnan(dy.get()).all()
    drow, dcol, dval = _Dev(gpu, row), _Dev(gpu, col), _Dev(gpu, val)
    dy = _Dev(gpu, np.zeros(nr))
    gpu.check(f(nr, nc, row.size, drow.p, dcol.p, dval.p, dx.p, dy.p, None))
    assert status() == 0
    y = dy.get()
    ref = np.zeros(nr)
    np.add.at(ref, row, val * x[col])
    assert np.allclose(y, ref, rtol=1e-12, atol=1e-12)
