"""Parity of the CUDA SpMV / a_axpx path with the oracle, through the C ABI.

Exact equality where the reference's own tests demand it (integer-valued
products: cqmat/cdiag with x = 0..n-1, test_spmv_cqmat.cpp:53-58 and
test_spmv_cdiag.cpp:22-26); otherwise the FP64 bound
|y - y_oracle| <= 1e-12 * sum_j |a_ij x_j| per row (rows split across
threads are summed in another order than the reference's sequential loop).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import assert_close
from test_oracle import BLOCKS, FORMATS

pytestmark = pytest.mark.gpu

RTOL64 = 1e-12


class Dev:
    """A device buffer allocated through the C ABI."""

    def __init__(self, capi, n, dtype=np.float64):
        self.capi, self.n, self.dtype = capi, n, np.dtype(dtype)
        self.p = C.c_void_p()
        capi.check(capi.lib().tbsla_device_alloc(C.byref(self.p), max(n, 1) * self.dtype.itemsize))

    @classmethod
    def of(cls, capi, a):
        a = np.ascontiguousarray(a)
        d = cls(capi, a.size, a.dtype)
        d.upload(a)
        return d

    def upload(self, a):
        L = self.capi.lib()
        self.capi.check(L.tbsla_memcpy_h2d(self.p, a.ctypes.data_as(C.c_void_p), a.nbytes, None))
        self.capi.check(L.tbsla_stream_sync(None))

    def get(self):
        out = np.zeros(max(self.n, 1), self.dtype)
        L = self.capi.lib()
        self.capi.check(L.tbsla_stream_sync(None))
        self.capi.check(L.tbsla_memcpy_d2h(out.ctypes.data_as(C.c_void_p), self.p, self.n * self.dtype.itemsize,
                                           None))
        self.capi.check(L.tbsla_stream_sync(None))
        return out[: self.n]

    @property
    def ptr(self):
        return self.p.value

    def __del__(self):
        try:
            self.capi.lib().tbsla_device_free(self.p)
        except Exception:
            pass


def oracle_of(orc, g):
    """The oracle matrix holding the same arrays as a generated one."""
    return orc.from_layout(g.fmt, g.geom, g.nnz, g.values, g.idx0, g.idx1)


def scale_of(orc, g, x):
    """sum_j |a_ij x_j| with the oracle (values and x in absolute value)."""
    from copy import copy
    ga = copy(g)
    ga.values = np.abs(g.values)
    return oracle_of(orc, ga).spmv(np.abs(x))


def gpu_spmv(capi, g, x, vect_incr=0):
    m = capi.DeviceMatrix.from_generated(g)
    return m.spmv_host(x, vect_incr)


def test_known_answer(gpu, golden):
    ka = golden["known_answer"]
    csr = gpu.DeviceMatrix.csr(5, 5, ka["rowptr"], ka["col"], ka["values"])
    coo = gpu.DeviceMatrix.coo(5, 5, ka["row"], ka["col"], ka["values"])
    assert csr.spmv_host(np.array(ka["x"])).tolist() == [20, 12, 10, 40, 85]
    assert coo.spmv_host(np.array(ka["x"])).tolist() == [20, 12, 10, 40, 85]


@pytest.mark.parametrize("fmt", FORMATS)
def test_reference_sweep_exact(gpu, orc, fmt):
    """Every format on the reference test shapes, x = 0..n-1: exact."""
    shapes = [(10, 5, 8), (5, 10, 7), (10, 10, 12), (10, 10, 3), (10, 5, 3), (10, 5, 6)]
    shapes += [(10, 10, i) for i in range(13)] + [(30, 30, 2 * i) for i in range(13)]
    shapes += [(20, 30, 2 * i) for i in range(0, 13, 3)] + [(30, 20, 2 * i) for i in range(0, 13, 3)]
    for (nr, nc, c) in shapes:
        x = np.arange(nc, dtype=np.float64)
        for s in (0, 1):
            for q in (0.0, 0.1, 0.5, 1.0):
                for blk in BLOCKS:
                    g = gpu.generate(fmt, "cqmat", nr, nc, c, q, s, *blk)
                    yo = oracle_of(orc, g).spmv(x)
                    y = gpu_spmv(gpu, g, x)
                    assert np.array_equal(y, yo), (fmt, nr, nc, c, q, s, blk, y, yo)
        for cd in range(0, 13, 2):
            g = gpu.generate(fmt, "cdiag", nr, nc, cd, 0.0, 0)
            y = gpu_spmv(gpu, g, x)
            assert np.array_equal(y, oracle_of(orc, g).spmv(x)), (fmt, "cdiag", nr, nc, cd)


@pytest.mark.parametrize("fmt", FORMATS)
def test_random_x(gpu, orc, fmt):
    rng = np.random.default_rng(11)
    for (nr, nc, c) in [(30, 30, 6), (300, 250, 17), (1000, 1000, 40), (257, 999, 3)]:
        for gen in ("cqmat", "cqmat_stochastic"):
            g = gpu.generate(fmt, gen, nr, nc, c, 0.3, 2)
            x = rng.uniform(-1, 1, nc)
            assert_close(gpu_spmv(gpu, g, x), oracle_of(orc, g).spmv(x), scale_of(orc, g, x), RTOL64,
                         f"{fmt} {gen} {nr}x{nc}")


@pytest.mark.parametrize("fmt", FORMATS)
def test_cfg1_all_formats(gpu, orc, fmt):
    """n=100000, c=10, q=0.1, seed 0 (the CPU-runnable headline case)."""
    g = gpu.generate(fmt, "cqmat", 100000, 100000, 10, 0.1, 0) if fmt != "DENSE" else \
        gpu.generate(fmt, "cqmat", 3000, 3000, 10, 0.1, 0)
    x = np.random.default_rng(0).random(g.n_col)
    o = oracle_of(orc, g)
    assert_close(gpu_spmv(gpu, g, x), o.spmv(x), scale_of(orc, g, x), RTOL64, fmt)
    if g.n_row == g.n_col:
        m = gpu.DeviceMatrix.from_generated(g)
        xa = np.abs(x)
        scale = scale_of(orc, g, scale_of(orc, g, xa) + xa)
        assert_close(m.a_axpx_host(x), o.a_axpx(x), scale, 1e-12, f"{fmt} a_axpx")


@pytest.mark.parametrize("fmt", FORMATS)
def test_cfg1_baseline_cqmat_all_formats(gpu, orc, fmt):
    """The benchmark's cqmat as configured (n = 100000, c = 10, q = 0.1,
    duplicates merged, values U(0,1], x U[0,1), seed 0; DENSE at n = 3000):
    every format's product and a_axpx_ against the oracle of the reference's
    array constructor MatrixCSR(n, n, values, rowptr, colidx)
    (MatrixCSR.cpp:13-27) and its spmv / a_axpx_."""
    from oracle.oracle import splitmix64_u01
    n = 100000 if fmt != "DENSE" else 3000
    rp, ci, va = orc.baseline_cqmat(n, n, 10, 0.1, 0)
    o = orc.from_arrays("CSR", n, n, va, rp, ci)
    oa = orc.from_arrays("CSR", n, n, np.abs(va), rp, ci)
    x = splitmix64_u01(0, 2, n)
    A = gpu.DeviceMatrix.generate(fmt, "cqmat_baseline", n, n, 10, 0.1, 0)
    if fmt in ("COO", "SCOO", "CSR"):
        assert A.info().stored == va.size
    assert_close(A.spmv_host(x), o.spmv(x), oa.spmv(x), RTOL64, f"{fmt} baseline-cqmat spmv")
    assert_close(A.a_axpx_host(x), o.a_axpx(x), oa.spmv(oa.spmv(x) + x), RTOL64, f"{fmt} baseline-cqmat a_axpx_")


def random_csr(rng, n_row, n_col, lengths):
    rowptr = np.zeros(n_row + 1, np.int64)
    rowptr[1:] = np.cumsum(lengths)
    nnz = int(rowptr[-1])
    colidx = rng.integers(0, n_col, nnz).astype(np.int32)
    values = rng.standard_normal(nnz)
    return rowptr.astype(np.int32), colidx, values


def test_csr_skewed_rows_and_tile_edges(gpu, orc):
    """Rows much longer than a tile, empty rows, and sizes around tile
    boundaries (rows + nnz = k * 2304 +- 1) exercise the carry paths."""
    rng = np.random.default_rng(3)
    cases = []
    lengths = rng.zipf(1.6, 5000).clip(0, 60000)
    lengths[:7] = 0
    lengths[-5:] = 0
    lengths[100] = 50000
    cases.append((5000, 7000, lengths))
    for total in (2303, 2304, 2305, 4607, 4608, 4609, 9216 * 3 + 1):
        n = 300
        base = rng.integers(0, 15, n)
        base[-1] = max(total - n - int(base[:-1].sum()), 0)
        cases.append((n, 500, base))
    cases.append((1, 10, np.array([0])))
    cases.append((3, 10, np.array([0, 0, 0])))
    cases.append((1, 100000, np.array([99999])))
    for (nr, nc, lens) in cases:
        rp, ci, va = random_csr(rng, nr, nc, lens)
        x = rng.uniform(-1, 1, nc)
        m = gpu.DeviceMatrix.csr(nr, nc, rp, ci, va)
        o = orc.from_arrays("CSR", nr, nc, va, rp, ci)
        so = orc.from_arrays("CSR", nr, nc, np.abs(va), rp, ci)
        assert_close(m.spmv_host(x), o.spmv(x), so.spmv(np.abs(x)), RTOL64, f"csr {nr}x{nc} nnz={ci.size}")


@pytest.mark.parametrize("variant", [0, 1])
def test_csr_kernel_variants(gpu, orc, variant):
    """Both CSR kernels (direct row bins, shared-memory row blocks) on
    uniform, skewed and huge-row matrices."""
    rng = np.random.default_rng(8)
    lens_skew = rng.zipf(1.5, 30000).clip(0, 40000)
    lens_skew[:3] = 0
    lens_skew[123] = 20000
    for (nr, nc, lens) in [(20000, 20000, np.full(20000, 16)), (30000, 40000, lens_skew),
                           (50, 300000, np.array([0, 9000, 33, 17000] + [5] * 46)), (40000, 9, np.full(40000, 2))]:
        rp, ci, va = random_csr(rng, nr, nc, lens)
        x = rng.uniform(-1, 1, nc)
        m = gpu.DeviceMatrix.csr(nr, nc, rp, ci, va)
        m.set_variant(variant)
        o = orc.from_arrays("CSR", nr, nc, va, rp, ci)
        so = orc.from_arrays("CSR", nr, nc, np.abs(va), rp, ci)
        assert_close(m.spmv_host(x), o.spmv(x), so.spmv(np.abs(x)), RTOL64, f"csr variant {variant} {nr}x{nc}")


def test_ell_kernel_variants(gpu, orc):
    """ELL warp tiles (variant 0: lane l of a warp sums rows l, l+32, ... of
    a tile of 32, 64 or 128 rows) and four consecutive rows per thread
    (variant 1) sum each row slot by slot: results are bit-identical and
    within the FP64 bound of the oracle.  Row counts that fill no tile, one row, padding
    slots, columns below f_col (read as x[0]), reduced-precision stores."""
    rng = np.random.default_rng(12)
    for (nr, nc, w, f_col) in [(1, 7, 3, 0), (127, 300, 5, 0), (129, 129, 16, 0), (5000, 4000, 9, 2),
                               (70001, 70001, 12, 0)]:
        cols = rng.integers(f_col, nc + f_col, (nr, w)).astype(np.int32)
        vals = rng.standard_normal((nr, w))
        cols[::7, -1] = 0  # padding slots (column 0, value 0)
        vals[::7, -1] = 0.0
        if f_col:
            cols[::5, 0] = 0  # below f_col: x[0]
        x = rng.uniform(-1, 1, nc)
        stores = gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16
        m = gpu.DeviceMatrix.ell(nr, nc, w, cols.ravel(), vals.ravel(), f_col=f_col, stores=stores)
        geom = (nr, nc, nr, nc, 0, f_col, 0, 0, 1, 1, w)
        o = orc.from_layout("ELL", geom, 0, vals.ravel(), cols.ravel(), np.zeros(0, np.int32))
        so = orc.from_layout("ELL", geom, 0, np.abs(vals).ravel(), cols.ravel(), np.zeros(0, np.int32))
        got = {}
        for variant in (0, 1):
            m.set_variant(variant)
            y = m.spmv_host(x)
            assert_close(y, o.spmv(x), so.spmv(np.abs(x)), RTOL64, f"ell variant {variant} {nr}x{nc}")
            x32 = Dev.of(gpu, x.astype(np.float32))
            outs = [y]
            for store in (gpu.F32, gpu.BF16):
                y32 = Dev(gpu, nr, np.float32)
                m.spmv_ex(store, gpu.F32, x32.ptr, gpu.F32, y32.ptr)
                outs.append(y32.get())
            got[variant] = outs
        for a, b in zip(got[0], got[1]):
            assert np.array_equal(a, b)
        # warp tiles with 1, 2 or 4 rows per thread (TBSLA_TUNE_SELL_ROWS):
        # the same bits
        m.set_variant(0)
        for rows_per_thread in (1, 4, 2):
            m.tune(gpu.TUNE_SELL_ROWS, rows_per_thread)
            assert np.array_equal(m.spmv_host(x), got[0][0]), rows_per_thread


def test_csr_tiny_rows_kernel(gpu, orc):
    """Rows of at most 4 entries, all in order: warp tiles (lane l taking
    rows l, l+32, ...) sum each row in stored order, one FMA per entry, so
    the default product equals one thread per row (TBSLA_TUNE_SHORT_ROWS 0)
    bit for bit, for every store; ragged rows (0 to 4 entries), row counts
    that fill no tile, and the FP64 bound against the oracle."""
    rng = np.random.default_rng(21)
    for (nr, nc, top) in [(1, 5, 2), (63, 70, 2), (129, 129, 2), (4097, 3000, 4), (200003, 150000, 3),
                          (70000, 90000, 1)]:
        lens = rng.integers(0, top + 1, nr)
        rp, ci, va = random_csr(rng, nr, nc, lens)
        x = rng.uniform(-1, 1, nc)
        stores = gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16
        m = gpu.DeviceMatrix.csr(nr, nc, rp, ci, va, stores=stores)
        ref = gpu.DeviceMatrix.csr(nr, nc, rp, ci, va, stores=stores)
        ref.tune(gpu.TUNE_SHORT_ROWS, 0)
        o = orc.from_arrays("CSR", nr, nc, va, rp, ci)
        so = orc.from_arrays("CSR", nr, nc, np.abs(va), rp, ci)
        y = m.spmv_host(x)
        assert_close(y, o.spmv(x), so.spmv(np.abs(x)), RTOL64, f"tiny rows {nr}x{nc}")
        assert np.array_equal(y, ref.spmv_host(x))
        assert np.array_equal(m.a_axpx_host(x[:nr]) if nr == nc else y, ref.a_axpx_host(x[:nr]) if nr == nc else y)
        x32 = Dev.of(gpu, x.astype(np.float32))
        for store in (gpu.F32, gpu.BF16):
            ya, yb = Dev(gpu, nr, np.float32), Dev(gpu, nr, np.float32)
            m.spmv_ex(store, gpu.F32, x32.ptr, gpu.F32, ya.ptr)
            ref.spmv_ex(store, gpu.F32, x32.ptr, gpu.F32, yb.ptr)
            assert np.array_equal(ya.get(), yb.get())


def test_autotune_tries_tiny_rows(gpu):
    """The SpMV autotuner times the tiny-row warp tiles (choice 4) next to
    one thread per row, row blocks, staged tiles and two lanes per row, each
    with four x-keep fractions; integer-valued products stay exact."""
    n = 1 << 16
    m = gpu.DeviceMatrix.from_generated(gpu.generate("CSR", "cdiag", n, n, 1, 0.0, 0))
    x = np.arange(n, dtype=np.float64)
    before = m.spmv_host(x)
    r = m.autotune_spmv(gpu.F64)
    # 4 keeps x (direct, staged, pairs, tiny) + 1 row-block run
    assert r.candidates == 17 and r.choice in (0, 1, 2, 3, 4)
    assert np.array_equal(m.spmv_host(x), before)


def test_autotune_tries_sliced_copy(gpu):
    """On a handle with the ELL-layout copy the SpMV autotuner also times the
    copy (choice 5, TBSLA_TUNE_SHORT_ROWS 3) with four x-keep fractions, next
    to one thread per row, row blocks, staged tiles and two lanes per row;
    integer-valued products stay exact whatever it keeps."""
    n = 70000
    m = gpu.DeviceMatrix.from_generated(gpu.generate("CSR", "cqmat", n, n, 12, 0.1, 3))
    assert m.info().slices > 0
    x = np.arange(n, dtype=np.float64)
    before = m.spmv_host(x)
    r = m.autotune_spmv(gpu.F64)
    # 4 keeps x (direct, staged, pairs, copy) + 1 row-block run
    assert r.candidates == 17 and r.choice in (0, 1, 2, 3, 5)
    assert np.array_equal(m.spmv_host(x), before)


def test_coo_unsorted_duplicates_and_shift(gpu, orc):
    rng = np.random.default_rng(4)
    for (nr, nc, nnz) in [(50, 40, 700), (1000, 800, 30000), (7, 7, 0), (1, 1, 5), (40000, 3, 90000)]:
        row = rng.integers(0, nr, nnz).astype(np.int32)
        col = rng.integers(0, nc, nnz).astype(np.int32)
        val = rng.standard_normal(nnz)
        x = rng.uniform(-1, 1, nc)
        m = gpu.DeviceMatrix.coo(nr, nc, row, col, val)
        o = orc.from_arrays("COO", nr, nc, val, row, col)
        so = orc.from_arrays("COO", nr, nc, np.abs(val), row, col)
        assert_close(m.spmv_host(x), o.spmv(x), so.spmv(np.abs(x)), RTOL64, f"coo {nr}x{nc}")
    # vect_incr shifts output rows (MatrixCOO.cpp:114)
    row = np.array([0, 1, 2, 2], np.int32)
    col = np.array([0, 1, 0, 2], np.int32)
    val = np.array([1.0, 2.0, 3.0, 4.0])
    m = gpu.DeviceMatrix.coo(4, 3, row, col, val)
    assert m.spmv_host(np.array([1.0, 1.0, 1.0]), vect_incr=1).tolist() == [0, 1, 2, 7]


def test_scoo_block_offsets(gpu, orc):
    """SCOO/CSR/ELL/DENSE blocks of a 2x3 grid: x indexed from f_col, y from f_row."""
    for fmt in ("SCOO", "CSR", "ELL", "DENSE"):
        for blk in [(1, 2, 2, 3), (0, 1, 2, 3), (1, 0, 2, 3)]:
            g = gpu.generate(fmt, "cqmat", 40, 45, 7, 0.2, 1, *blk)
            x = np.arange(g.ln_col, dtype=np.float64) + 1
            yo = oracle_of(orc, g).spmv(x)
            assert np.array_equal(gpu_spmv(gpu, g, x), yo), (fmt, blk)


def test_device_pointer_entry_points(gpu, orc):
    g = gpu.generate("CSR", "cqmat", 5000, 5000, 12, 0.1, 0)
    x = np.random.default_rng(9).uniform(-1, 1, 5000)
    m = gpu.DeviceMatrix.from_generated(g)
    dx, dy, dt = Dev.of(gpu, x), Dev(gpu, 5000), Dev(gpu, 5000)
    m.spmv(dx.ptr, dy.ptr)
    o = oracle_of(orc, g)
    assert_close(dy.get(), o.spmv(x), scale_of(orc, g, x), RTOL64, "device spmv")
    m.a_axpx(dx.ptr, dy.ptr, dt.ptr)
    xa = np.abs(x)
    assert_close(dy.get(), o.a_axpx(x), scale_of(orc, g, scale_of(orc, g, xa) + xa), RTOL64, "device a_axpx")


@pytest.mark.parametrize("fmt", ["CSR", "ELL", "COO", "DENSE"])
def test_reduced_precision_stores(gpu, orc, fmt):
    """F32 / BF16 value stores with FP32 accumulation against the FP64 oracle:
    |y - y64| <= rtol * sum|a x| with rtol 2e-6 (F32) and 8e-3 (BF16)."""
    n = 20000 if fmt != "DENSE" else 1500
    g = gpu.generate(fmt, "cqmat_stochastic", n, n, 16, 0.1, 0)
    m = gpu.DeviceMatrix.from_generated(g, stores=gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16)
    x = np.random.default_rng(2).random(n)
    yo = oracle_of(orc, g).spmv(x)
    sc = scale_of(orc, g, x)
    x32 = Dev.of(gpu, x.astype(np.float32))
    for store, rtol in ((gpu.F32, 2e-6), (gpu.BF16, 8e-3)):
        y32 = Dev(gpu, n, np.float32)
        m.spmv_ex(store, gpu.F32, x32.ptr, gpu.F32, y32.ptr)
        assert_close(y32.get().astype(np.float64), yo, sc, rtol, f"{fmt} store {store} f32 vectors")
        y64 = Dev(gpu, n)
        x64 = Dev.of(gpu, x)
        m.spmv_ex(store, gpu.F64, x64.ptr, gpu.F64, y64.ptr)
        assert_close(y64.get(), yo, sc, rtol, f"{fmt} store {store} f64 vectors")


def test_full_size_cqmat_exact_integers(gpu):
    """n = 2^24, c = 16, q = 0.1: with x_j = j mod 7 every product is a small
    integer, so y must equal the row sums computed exactly on the host."""
    n = 1 << 24
    g = gpu.generate("CSR", "cqmat", n, n, 16, 0.1, 0)
    x = (np.arange(n) % 7).astype(np.float64)
    m = gpu.DeviceMatrix.from_generated(g)
    y = m.spmv_host(x)
    gathered = x[g.idx1]
    expect = np.add.reduceat(gathered, g.idx0[:-1]) if gathered.size else np.zeros(n)
    expect[np.diff(g.idx0) == 0] = 0
    assert np.array_equal(y, expect)
    assert y.sum() == gathered.sum()
    # random x against the oracle (x of 128 MiB, 10 % random columns)
    from oracle.oracle import Oracle
    orc = Oracle()
    o = orc.from_layout("CSR", g.geom, g.nnz, g.values, g.idx0, g.idx1)
    oa = orc.from_layout("CSR", g.geom, g.nnz, np.abs(g.values), g.idx0, g.idx1)
    xr = np.random.default_rng(3).uniform(-1, 1, n)
    assert_close(m.spmv_host(xr), o.spmv(xr, threads=8), oa.spmv(np.abs(xr), threads=8), 1e-12, "cqmat 2^24")


def test_full_size_cdiag(gpu):
    """cdiag n = 2^26, c = 1 (the bandwidth sanity case): y_i = x_{i-1} + x_{i+1}."""
    n = 1 << 26
    m = gpu.DeviceMatrix.generate("CSR", "cdiag", n, n, 1)
    x = (np.arange(n) % 1000).astype(np.float64)
    y = m.spmv_host(x)
    expect = np.zeros(n)
    expect[1:] += x[:-1]
    expect[:-1] += x[1:]
    assert np.array_equal(y, expect)


def test_invalid_arguments_are_reported(gpu):
    with pytest.raises(gpu.TbslaError):
        gpu.DeviceMatrix.csr(3, 3, [0, 2, 1, 3], [0, 1, 2], [1.0, 1.0, 1.0])  # rowptr not monotone
    with pytest.raises(gpu.TbslaError):
        gpu.DeviceMatrix.csr(3, 3, [0, 1, 2, 3], [0, 1, 5], [1.0, 1.0, 1.0])  # column out of range
    with pytest.raises(gpu.TbslaError):
        gpu.DeviceMatrix.coo(3, 3, [0, 3], [0, 0], [1.0, 1.0])  # row out of range
    m = gpu.DeviceMatrix.csr(3, 3, [0, 1, 2, 3], [0, 1, 2], [1.0, 1.0, 1.0])
    with pytest.raises(gpu.TbslaError):
        m.spmv_ex(gpu.F32, gpu.F64, 0, gpu.F64, 0)  # no F32 store


@pytest.mark.parametrize("variant", [0, 1])
def test_coo_variants(gpu, orc, variant):
    """COO / SCOO through the direct CSR kernels over the derived row pointer
    (variant 0) and through the merge path (variant 1): unsorted triplets
    with repeated entries, empty rows, a hub row, SCOO offsets, row shifts."""
    rng = np.random.default_rng(17 + variant)
    n_row, n_col, nnz = 4000, 3000, 50000
    # rows in [2, n_row - 4): the shifted products below stay inside y (the
    # reference writes r[row + vect_incr] unchecked)
    row = rng.integers(2, n_row - 4, nnz).astype(np.int32)
    row[:9000] = 7  # one row longer than the chunk size of the direct kernels
    row[row % 13 == 0] = 5  # rows multiple of 13 stay empty
    col = rng.integers(0, n_col, nnz).astype(np.int32)
    val = rng.standard_normal(nnz)
    for (f_row, f_col) in ((0, 0), (100, 50)):
        m = gpu.DeviceMatrix.coo(n_row, n_col, row + f_row, col + f_col, val, f_row=f_row, f_col=f_col)
        m.set_variant(variant)
        o = orc.from_arrays("COO", n_row, n_col, val, row, col)
        so = orc.from_arrays("COO", n_row, n_col, np.abs(val), row, col)
        x = rng.uniform(-1, 1, n_col)
        for incr in (0, 3, -2):
            assert_close(m.spmv_host(x, incr), o.spmv(x, incr), so.spmv(np.abs(x), incr), RTOL64,
                         f"coo variant {variant} offsets {f_row},{f_col} shift {incr}")


def test_csr_staged_kernel(gpu, orc):
    """The staged kernel (every row at most 32 entries, 32-row tiles copied to
    shared memory) sums each row in stored order with one FMA per entry, as
    the direct kernel does: results are bit-identical to it and within the
    FP64 bound of the oracle.  Uniform, ragged (empty rows, row counts that
    are not a multiple of 32), full (32-entry rows: the largest tile) and
    reduced-precision stores; a_axpx and the PageRank sweep epilogue."""
    rng = np.random.default_rng(31)
    cases = [(20000, 20000, np.full(20000, 16)), (20011, 5000, rng.integers(0, 33, 20011)),
             (4133, 70000, np.full(4133, 32)), (33, 40, rng.integers(0, 4, 33)), (1, 7, np.array([5]))]
    for (nr, nc, lens) in cases:
        rp, ci, va = random_csr(rng, nr, nc, lens)
        x = rng.uniform(-1, 1, nc)
        m = gpu.DeviceMatrix.csr(nr, nc, rp, ci, va, stores=gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16)
        m.tune(gpu.TUNE_SHORT_ROWS, 0)
        y0 = m.spmv_host(x)
        m.tune(gpu.TUNE_SHORT_ROWS, 1)
        y1 = m.spmv_host(x)
        assert np.array_equal(y0, y1), f"staged {nr}x{nc}: not bit-identical"
        o = orc.from_arrays("CSR", nr, nc, va, rp, ci)
        so = orc.from_arrays("CSR", nr, nc, np.abs(va), rp, ci)
        assert_close(y1, o.spmv(x), so.spmv(np.abs(x)), RTOL64, f"staged {nr}x{nc}")
        for store in (gpu.F32, gpu.BF16):
            outs = []
            for mode in (0, 1):
                m.tune(gpu.TUNE_SHORT_ROWS, mode)
                xs = Dev.of(gpu, x.astype(np.float32))
                ys = Dev(gpu, nr, np.float32)
                m.spmv_ex(store, gpu.F32, xs.ptr, gpu.F32, ys.ptr)
                outs.append(ys.get())
            assert np.array_equal(outs[0], outs[1]), f"staged store {store} {nr}x{nc}"
        if nr == nc:
            m.tune(gpu.TUNE_SHORT_ROWS, 0)
            r0 = m.a_axpx_host(x)
            m.tune(gpu.TUNE_SHORT_ROWS, 1)
            assert np.array_equal(r0, m.a_axpx_host(x)), "staged a_axpx"
    # PageRank sweeps (reducing epilogue) on a column-stochastic cqmat
    g = gpu.generate("CSR", "cqmat_stochastic", 50000, 50000, 12, 0.1, 2)
    m = gpu.DeviceMatrix.from_generated(g)
    m.tune(gpu.TUNE_SHORT_ROWS, 0)
    x0, r0 = m.pagerank_host(beta=0.85, tol=1e-12, max_iter=500, mode=gpu.PR_DANGLING)
    m.tune(gpu.TUNE_SHORT_ROWS, 1)
    x1, r1 = m.pagerank_host(beta=0.85, tol=1e-12, max_iter=500, mode=gpu.PR_DANGLING)
    # the per-block partial sums group rows differently: equal to rounding
    assert abs(r0.iterations - r1.iterations) <= 1 and r1.converged
    assert float(np.abs(x0 - x1).sum()) <= 1e-11


def test_l2_fetch_granularity(gpu):
    """The process-wide L2 fetch granularity is set and read back; products
    do not depend on it (32-byte fetches with 256-byte prefetched rows)."""
    L = gpu.lib()
    v = C.c_int()
    g = gpu.generate("CSR", "cqmat", 30000, 30000, 16, 0.1, 0)
    m = gpu.DeviceMatrix.from_generated(g)
    x = np.random.default_rng(4).uniform(-1, 1, 30000)
    ys = []
    for b in (32, 64, 128):
        gpu.check(L.tbsla_set_l2_fetch_granularity(b))
        gpu.check(L.tbsla_get_l2_fetch_granularity(C.byref(v)))
        assert v.value == b
        ys.append(m.spmv_host(x))
    assert np.array_equal(ys[0], ys[1]) and np.array_equal(ys[0], ys[2])
    assert L.tbsla_set_l2_fetch_granularity(48) != 0


def test_csr_pair_kernel(gpu, orc):
    """Two lanes per short row (TBSLA_TUNE_SHORT_ROWS = 2): each lane sums half
    the row in stored order, the row is the halves' sum -- within the FP64
    bound of the oracle on uniform, ragged and skewed matrices (short rows
    listed among long ones), for reduced-precision stores, a_axpx and the
    PageRank sweep epilogue."""
    rng = np.random.default_rng(41)
    skew = rng.zipf(1.5, 30000).clip(0, 20000)
    skew[:5] = 0
    cases = [(20000, 20000, np.full(20000, 16)), (20011, 5000, rng.integers(0, 33, 20011)),
             (30000, 30000, skew), (33, 40, rng.integers(0, 4, 33)), (1, 7, np.array([5]))]
    for (nr, nc, lens) in cases:
        rp, ci, va = random_csr(rng, nr, nc, lens)
        x = rng.uniform(-1, 1, nc)
        m = gpu.DeviceMatrix.csr(nr, nc, rp, ci, va, stores=gpu.STORE_F64 | gpu.STORE_F32)
        m.tune(gpu.TUNE_SHORT_ROWS, 2)
        o = orc.from_arrays("CSR", nr, nc, va, rp, ci)
        so = orc.from_arrays("CSR", nr, nc, np.abs(va), rp, ci)
        sc = so.spmv(np.abs(x))
        assert_close(m.spmv_host(x), o.spmv(x), sc, RTOL64, f"pairs {nr}x{nc}")
        xs = Dev.of(gpu, x.astype(np.float32))
        ys = Dev(gpu, nr, np.float32)
        m.spmv_ex(gpu.F32, gpu.F32, xs.ptr, gpu.F32, ys.ptr)
        assert_close(ys.get().astype(np.float64), o.spmv(x), sc, 2e-6, f"pairs F32 {nr}x{nc}")
        if nr == nc:
            assert_close(m.a_axpx_host(x), o.a_axpx(x), so.spmv(sc + np.abs(x)), RTOL64, "pairs a_axpx")
    g = gpu.generate("CSR", "cqmat_stochastic", 50000, 50000, 12, 0.1, 2)
    m = gpu.DeviceMatrix.from_generated(g)
    x0, r0 = m.pagerank_host(beta=0.85, tol=1e-12, max_iter=500, mode=gpu.PR_DANGLING)
    m.tune(gpu.TUNE_SHORT_ROWS, 2)
    x1, r1 = m.pagerank_host(beta=0.85, tol=1e-12, max_iter=500, mode=gpu.PR_DANGLING)
    assert abs(r0.iterations - r1.iterations) <= 1 and r1.converged
    assert float(np.abs(x0 - x1).sum()) <= 1e-11


def test_l2_persisting_setaside(gpu):
    """The process's persisting L2 set-aside is set, read back (rounded by the
    device, within its maximum) and restored; products do not depend on it or
    on the evict-last fraction of x."""
    L = gpu.lib()
    cur, mx = C.c_size_t(), C.c_size_t()
    gpu.check(L.tbsla_get_l2_persisting(C.byref(cur), C.byref(mx)))
    assert mx.value > 0
    g = gpu.generate("CSR", "cqmat", 30000, 30000, 16, 0.1, 0)
    m = gpu.DeviceMatrix.from_generated(g)
    x = np.random.default_rng(5).uniform(-1, 1, 30000)
    y0 = m.spmv_host(x)
    for want in (0, 32 << 20, mx.value):
        gpu.check(L.tbsla_set_l2_persisting(want))
        got = C.c_size_t()
        gpu.check(L.tbsla_get_l2_persisting(C.byref(got), None))
        assert got.value <= mx.value and (want == 0) == (got.value == 0)
        for keep in (0.0, 1.0):
            m.tune(gpu.TUNE_X_L2_KEEP, keep)
            assert np.array_equal(m.spmv_host(x), y0)
    gpu.check(L.tbsla_set_l2_persisting(cur.value))


def test_csr_sliced_copy(gpu, orc):
    """The ELL-layout copy of short-row CSR / row-sorted COO handles
    (csr_sell_kernel, TBSLA_TUNE_SHORT_ROWS -1 or 3): built only when every
    row has at most 32 entries, rows average 4 or more and padding adds at
    most 1/32 slots; each row summed in stored order, so every store's
    product equals one thread per row (mode 0) bit for bit, and the oracle
    within the FP64 bound; a_axpx through it; refreshed by set_values; rows
    past `rows` and the output shift of COO unchanged; every rows-per-thread
    setting (TBSLA_TUNE_SELL_ROWS) gives the same bits; no copy below 2^16
    rows."""
    rng = np.random.default_rng(77)
    n = 70000
    lens = np.full(n, 12)
    lens[rng.choice(n, 300, replace=False)] = 11  # a few padded slots
    rp, ci, va = random_csr(rng, n, n, lens)
    x = rng.uniform(-1, 1, n)
    m = gpu.DeviceMatrix.csr(n, n, rp, ci, va, stores=gpu.STORE_F64 | gpu.STORE_F32 | gpu.STORE_BF16)
    assert m.info().slices == (n + 127) // 128
    o = orc.from_arrays("CSR", n, n, va, rp, ci)
    so = orc.from_arrays("CSR", n, n, np.abs(va), rp, ci)
    sc = so.spmv(np.abs(x))
    y_sliced = m.spmv_host(x)
    assert_close(y_sliced, o.spmv(x), sc, RTOL64, "sliced")
    assert_close(m.a_axpx_host(x), o.a_axpx(x), so.spmv(sc + np.abs(x)), RTOL64, "sliced a_axpx")
    for store, xt, tol in ((gpu.F32, np.float32, 2e-6), (gpu.BF16, np.float32, 2e-2)):
        xs = Dev.of(gpu, x.astype(xt))
        ys, y0 = Dev(gpu, n, np.float32), Dev(gpu, n, np.float32)
        m.tune(gpu.TUNE_SHORT_ROWS, 3)
        m.spmv_ex(store, gpu.F32, xs.ptr, gpu.F32, ys.ptr)
        m.tune(gpu.TUNE_SHORT_ROWS, 0)
        m.spmv_ex(store, gpu.F32, xs.ptr, gpu.F32, y0.ptr)
        assert np.array_equal(ys.get(), y0.get()), store
        assert_close(ys.get().astype(np.float64), o.spmv(x), sc, tol, f"sliced store {store}")
    y_mode0 = m.spmv_host(x)
    assert np.array_equal(y_sliced, y_mode0)
    m.tune(gpu.TUNE_SHORT_ROWS, -1)
    for rows_per_thread in (1, 2, 4):
        m.tune(gpu.TUNE_SELL_ROWS, rows_per_thread)
        assert np.array_equal(m.spmv_host(x), y_mode0), rows_per_thread
    m.tune(gpu.TUNE_SELL_ROWS, 0)
    # new values: the copy follows
    va2 = rng.uniform(-2, 2, va.size)
    d_va2 = Dev.of(gpu, va2)
    m.set_values(gpu.F64, d_va2.ptr)
    o2 = orc.from_arrays("CSR", n, n, va2, rp, ci)
    y2 = m.spmv_host(x)
    m.tune(gpu.TUNE_SHORT_ROWS, 0)
    assert np.array_equal(y2, m.spmv_host(x))
    assert_close(y2, o2.spmv(x), orc.from_arrays("CSR", n, n, np.abs(va2), rp, ci).spmv(np.abs(x)), RTOL64,
                 "sliced after set_values")
    # below 2^16 rows: no copy
    small = gpu.DeviceMatrix.csr(50000, n, rp[:50001], ci[: rp[50000]], va[: rp[50000]])
    assert small.info().slices == 0
    # the same entries as COO (row-sorted on the device), the last three rows
    # empty so that the output shift of vect_incr stays inside y (the
    # reference's Ax writes r[row + vect_incr] unchecked): the copy as well
    keep = rp[n - 3]
    rows_of = np.repeat(np.arange(n, dtype=np.int32), np.diff(rp))[:keep]
    mc = gpu.DeviceMatrix.coo(n, n, rows_of, ci[:keep], va[:keep])
    assert mc.info().slices > 0
    oc = orc.from_arrays("COO", n, n, va[:keep], rows_of, ci[:keep])
    sc3 = orc.from_arrays("COO", n, n, np.abs(va[:keep]), rows_of, ci[:keep]).spmv(np.abs(x))
    for incr in (0, 3):
        bound = np.zeros(n)
        bound[incr:] = sc3[: n - incr]
        assert_close(mc.spmv_host(x, incr), oc.spmv(x, incr), bound, RTOL64, f"COO {incr}")
    # rows below n_row (rows past them give 0)
    part = n - 1003
    mp = gpu.DeviceMatrix.csr(n, n, rp[: part + 1], ci[: rp[part]], va[: rp[part]], rows=part)
    assert mp.info().slices > 0
    yp = mp.spmv_host(x)
    assert np.array_equal(yp[part:], np.zeros(n - part)) and np.array_equal(yp[:part], y_sliced[:part])
    # dropped on request: the memory returns, the products read the CSR arrays
    held = m.info().device_bytes
    m.tune(gpu.TUNE_DROP_SLICED_COPY, 1)
    assert m.info().slices == 0 and m.info().device_bytes < held
    assert np.array_equal(m.spmv_host(x), y2)
    # not built: a row longer than 32 entries; padding above 1/32; short rows
    for bad in (np.r_[np.full(n - 1, 12), 40], np.r_[np.full(n // 2, 12), np.full(n - n // 2, 6)],
                np.full(n, 3)):
        rpb, cib, vab = random_csr(rng, n, n, bad)
        mb = gpu.DeviceMatrix.csr(n, n, rpb, cib, vab)
        assert mb.info().slices == 0
        ob = orc.from_arrays("CSR", n, n, vab, rpb, cib)
        assert_close(mb.spmv_host(x), ob.spmv(x), orc.from_arrays("CSR", n, n, np.abs(vab), rpb, cib).spmv(np.abs(x)),
                     RTOL64, "no copy")
