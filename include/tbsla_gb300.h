/*
 * tbsla_gb300.h -- C ABI of the GB300 (sm_103a) implementation of TBSLA's
 * SpMV / a_axpx_ / PageRank path.
 *
 * The entry points replace the compute behind TBSLA's tbsla::cpp::Matrix*
 * classes (src/cpp/include/tbsla/cpp/Matrix.hpp:9-47) and the C_CPP_* C ABI
 * (src/cpp/interface/c/include/tbsla/cpp/MatrixCSR.h and its siblings).  A
 * matrix handle owns device copies of one matrix in the layout its kernels
 * want (CSR with rows binned by length, column-major ELL, row-sorted COO,
 * row-major DENSE).  Plain
 * pointers and sizes only: no C++ or CUDA types cross this boundary; a
 * stream is passed as `void*` (a cudaStream_t, NULL for the legacy stream).
 *
 * Errors: every call returns a tbsla_status_t; no exception crosses the ABI.
 * tbsla_last_error() gives a readable message for the calling thread's last
 * failure.  On TBSLA_ERR_CUDA the handle stays valid only if the CUDA context
 * does.
 *
 * Threading: a handle may be used from several threads for reads (spmv on
 * device pointers); the *_host entry points use the handle's own stream and
 * staging buffers and must not run concurrently on one handle.
 */
#ifndef TBSLA_GB300_H
#define TBSLA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TBSLA_OK = 0,
  TBSLA_ERR_INVALID_ARG = 1,
  TBSLA_ERR_CUDA = 2,
  TBSLA_ERR_OOM = 3,
  TBSLA_ERR_NOT_CONVERGED = 4,
  TBSLA_ERR_TIMEOUT = 5,
  TBSLA_ERR_UNSUPPORTED = 6
} tbsla_status_t;

/* the reference's five storage formats */
typedef enum {
  TBSLA_FMT_COO = 0,
  TBSLA_FMT_SCOO = 1,
  TBSLA_FMT_CSR = 2,
  TBSLA_FMT_ELL = 3,
  TBSLA_FMT_DENSE = 4
} tbsla_format_t;

/* element types of stored matrix values and of vectors */
typedef enum { TBSLA_F64 = 0, TBSLA_F32 = 1, TBSLA_BF16 = 2 } tbsla_dtype_t;

/* value-store flags for *_create: which copies of the values to keep on the
 * device.  F64 is the drop-in; F32 / BF16 are the reduced-precision stores
 * (products accumulated in FP32). */
enum { TBSLA_STORE_F64 = 1, TBSLA_STORE_F32 = 2, TBSLA_STORE_BF16 = 4 };

typedef struct tbsla_matrix tbsla_matrix_t;

typedef struct {
  int format;          /* tbsla_format_t */
  int n_row, n_col;    /* global shape (Matrix::get_n_row/get_n_col)       */
  int f_row, f_col;    /* first row / column of the stored block           */
  int rows;            /* rows the kernels visit (rows past it give 0)     */
  int max_col;         /* ELL width                                        */
  int64_t stored;      /* stored entries (ELL: rows*max_col, DENSE: rows*cols) */
  int stores;          /* TBSLA_STORE_* bits present                       */
  int64_t device_bytes;/* device memory held by the handle                 */
  int kernels;         /* kernel launches of one tbsla_spmv call           */
  int slices;          /* CSR / row-sorted COO: 128-row tiles of the
                          ELL-layout copy that plain F64 / F32 products read
                          (TBSLA_TUNE_SHORT_ROWS 3); 0 without one         */
} tbsla_matrix_info_t;

/* ---------------------------------------------------------------- misc */
const char *tbsla_last_error(void);
const char *tbsla_status_string(tbsla_status_t s);
int tbsla_version(void);
/* device the library uses for new handles (default: current device) */
tbsla_status_t tbsla_set_device(int device);
/* The device's name (into name, name_len bytes, NUL-terminated), its
 * theoretical HBM rate in GB/s (memory clock x bus width, double data rate)
 * and its SM count; NULL pointers skip a field.  For reports such as the
 * driver programs' roofline fraction. */
tbsla_status_t tbsla_device_describe(int device, char *name, int name_len, double *hbm_gbs, int *sms);
/* The current device's L2 fetch granularity for this process (the CUDA
 * context limit cudaLimitMaxL2FetchGranularity; 32, 64 or 128 bytes): how
 * much a missing load brings from DRAM.  The kernels ask for 256-byte
 * prefetches on their streamed row data, so at 32 bytes the random gathers
 * of x stop bringing unused sectors while the streams stay wide (cqmat 2^24
 * FP64, one thread per row: 4396 GB/s at 32 against 4283 at the context's
 * default; ELL 4741 against 4102).  The setting is the caller's,
 * process-wide, and ends with it. */
tbsla_status_t tbsla_set_l2_fetch_granularity(int bytes);
tbsla_status_t tbsla_get_l2_fetch_granularity(int *bytes);
/* The current device's persisting L2 set-aside for this process (the CUDA
 * context limit cudaLimitPersistingL2CacheSize; the device rounds it, and
 * reports its maximum in *max_bytes).  Lines loaded with an evict-last
 * policy -- the gathered x, TBSLA_TUNE_X_L2_KEEP -- stay there ahead of the
 * streamed matrix.  cqmat 2^24 FP64 with all of x evict-last: 5085 GB/s at
 * 64 MiB against 4811 at the context's default (25 MB here); with the first
 * 45 % of x's addresses (TBSLA_TUNE_X_L2_RANGE): 5191.  The maximum (84 MB)
 * leaves the streams too little L2 (2920 GB/s), and R-MAT PageRank sweeps
 * lose 2 % at 64 MiB.  Setting it first returns every persisting
 * line to normal (cudaCtxResetPersistingL2Cache).  Process-wide, the
 * caller's to set and restore. */
tbsla_status_t tbsla_set_l2_persisting(size_t bytes);
tbsla_status_t tbsla_get_l2_persisting(size_t *bytes, size_t *max_bytes);

/* ------------------------------------------------------------ matrices */
/* CSR from host arrays.  Replaces MatrixCSR(n_row, n_col, values, rowptr,
 * colidx) (src/cpp/include/tbsla/cpp/MatrixCSR.hpp:15, MatrixCSR.cpp:13-27)
 * and the storage behind MatrixCSR::spmv (MatrixCSR.cpp:123-140).  rowptr has
 * rows+1 entries; its first entry is the base subtracted from every other
 * entry (the reference's rowptr.front()).  colidx holds global columns; the
 * kernel reads x[colidx - f_col].  rows may be below n_row (rows past it give
 * y = 0, as when the reference's rowptr is shorter than n_row+1). */
tbsla_status_t tbsla_csr_create(int n_row, int n_col, int f_col, int rows, const int *rowptr,
                                const int *colidx, const double *values, int stores,
                                tbsla_matrix_t **out);

/* ELL from host arrays in the reference's row-major layout
 * (values[i*max_col + j], columns[i*max_col + j], MatrixELL.hpp:33-35).
 * rows = min(ln_row, values.size()/max_col) as MatrixELL::Ax visits
 * (MatrixELL.cpp:101-114); padding is (column 0, value 0) and a column below
 * f_col is read as x[0], exactly as the reference clamps it.  Stored on the
 * device column-major. */
tbsla_status_t tbsla_ell_create(int n_row, int n_col, int f_col, int rows, int max_col,
                                const int *columns, const double *values, int stores,
                                tbsla_matrix_t **out);

/* COO / SCOO from host triplets.  Replaces MatrixCOO(n_row, n_col, values,
 * row, col) (MatrixCOO.hpp:14, MatrixCOO.cpp:30-44) and MatrixSCOO's
 * (MatrixSCOO.hpp:15); spmv adds values[k]*x[col[k]-f_col] into
 * y[row[k]-f_row] as MatrixCOO::Ax / MatrixSCOO::Ax do (MatrixCOO.cpp:107-116,
 * MatrixSCOO.cpp:114-123).  COO passes f_row = f_col = 0.  Entries are put in
 * row order (stable) at creation; entries whose output row falls outside
 * [0, n_row) are rejected with TBSLA_ERR_INVALID_ARG. */
tbsla_status_t tbsla_coo_create(int n_row, int n_col, int f_row, int f_col, int64_t nnz,
                                const int *row, const int *col, const double *values, int stores,
                                tbsla_matrix_t **out);

/* DENSE row-major ln_row x ln_col block (MatrixDENSE.hpp:33, Ax at
 * MatrixDENSE.cpp:64-73); y has n_row entries, rows past ln_row give 0. */
tbsla_status_t tbsla_dense_create(int n_row, int n_col, int ln_row, int ln_col,
                                  const double *values, int stores, tbsla_matrix_t **out);

tbsla_status_t tbsla_matrix_destroy(tbsla_matrix_t *A);
/* Kernel choice for a format with several (CSR: 0 = direct row bins, the
 * default; 1 = shared-memory row blocks.  COO / SCOO: 0 = direct kernels
 * over a derived row pointer, 1 = merge path.  ELL: 0 = warp tiles of 128
 * rows, lane l taking rows l, l+32, l+64, l+96, the default; 1 = four
 * consecutive rows per thread, bit-identical results).  Results agree within
 * the FP64 bound of the parity tests; the choice only changes speed. */
tbsla_status_t tbsla_matrix_set_variant(tbsla_matrix_t *A, int variant);

/* Tunable knobs of a handle's kernels (what the autotuner sets); results do
 * not depend on them.
 *   TBSLA_TUNE_X_L2_KEEP  fraction in [0, 1] of the gathered vector x that the
 *                         CSR product loads with L2 evict-last priority (the
 *                         rest with normal priority); default 0.6.
 *   TBSLA_TUNE_X_L2_RANGE 1: the kept fraction is the leading part of x by
 *                         address (the same lines on every load: an L2
 *                         range policy); 0 (default): a fraction of the
 *                         lines touched.
 *   TBSLA_TUNE_SHORT_ROWS the kernel for rows of at most 32 entries:
 *                         -1 (default) for plain products: the sliced copy
 *                         (3) when the handle has one; else when every row
 *                         has at most 4 entries, warp tiles of 64 or 128
 *                         rows, lane l taking rows l, l+32, ... (one thread
 *                         per row's arithmetic, bit-identical to 0); else 2
 *                         for FP64 values when the short rows average 8
 *                         entries or more; 0 otherwise (and for PageRank
 *                         sweeps);
 *                         0 one thread per row, summed in stored
 *                         order; 1 (every row short) each 32-row tile's
 *                         entries staged in shared memory with coalesced
 *                         loads, rows summed from there in stored order
 *                         (bit-identical to 0); 2 two lanes per row, each
 *                         summing half the row in stored order, row = first
 *                         half + second half (rounds differently from 0);
 *                         3 the sliced copy (tbsla_matrix_info_t.slices):
 *                         a copy of the entries in ELL layout (slot j of
 *                         every row stored together, rows padded to a
 *                         multiple of 128, padding marked by column -1),
 *                         built at creation for matrices of at least 2^16
 *                         rows when every row has at most 32 entries, rows
 *                         average 4 or more and padding adds at most 1/32
 *                         slots; kept for the F64 and F32 stores (BF16
 *                         products read the CSR arrays); one thread per row
 *                         summing in stored order (bit-identical to 0).
 *                         Without the copy, 3 acts as -1.
 *   TBSLA_TUNE_SELL_ROWS  rows per thread of the sliced copy's kernel and of
 *                         the ELL warp tiles: 1, 2 or 4 (a warp takes 32, 64
 *                         or 128 rows); 0 (default): 2, the fastest or within
 *                         3 % from 7e4 to 1.6e7 rows (cqmat 2^24 FP64: CSR
 *                         copy 0.625 ms, 4 rows 0.646 ms; ELL 0.629 against
 *                         0.649 ms).  Results do not depend on it.
 *   TBSLA_TUNE_DROP_SLICED_COPY  1: frees the handle's ELL-layout copy (the
 *                         copy doubles the device memory of the entries);
 *                         products then read the CSR arrays.  Waits for the
 *                         device; the copy is not rebuilt.
 *   TBSLA_TUNE_PR_RELABEL PageRank on a copy of a CSR graph relabelled in
 *                         decreasing out-degree order (built on first use,
 *                         kept with the handle): 1 on, 0 off, -1 (default)
 *                         when the graph is square, has at least 2^20
 *                         vertices, is not banded and its top tenth of
 *                         vertices holds half of the entries.  Results are
 *                         returned in the original labels.  The dangling and
 *                         mixed-precision modes only: TBSLA_PR_REFERENCE
 *                         (page_rank, personalized_page_rank) always sweeps
 *                         the handle itself, so its iteration count follows
 *                         the reference's summation order at every size.
 *   TBSLA_TUNE_TC_SPLIT   DENSE tensor-core product (tbsla_dense_spmm, F32 /
 *                         BF16 stores): the number of parts K is split into,
 *                         1, 2, 4, 8 or 16, or 0 (default) to choose per call
 *                         from the shape and the SM count. */
typedef enum {
  TBSLA_TUNE_X_L2_KEEP = 0,
  TBSLA_TUNE_PR_RELABEL = 1,
  TBSLA_TUNE_X_L2_RANGE = 2,
  TBSLA_TUNE_SHORT_ROWS = 3,
  TBSLA_TUNE_TC_SPLIT = 4,
  TBSLA_TUNE_SELL_ROWS = 5,
  TBSLA_TUNE_DROP_SLICED_COPY = 6
} tbsla_tune_knob_t;
tbsla_status_t tbsla_matrix_tune(tbsla_matrix_t *A, int knob, double value);
tbsla_status_t tbsla_matrix_info(const tbsla_matrix_t *A, tbsla_matrix_info_t *info);

/* --------------------------------------------------------------- SpMV */
/* y[0:n_row] = A x on device pointers, ordered on `stream`; FP64 vectors and
 * FP64 values.  x has n_col - f_col... entries addressed as x[col - f_col]
 * (the reference's v[colidx - f_col]).  Replaces Matrix::spmv
 * (Matrix.hpp:12) / Ax (Matrix.hpp:13).  vect_incr shifts COO/SCOO output
 * rows (MatrixCOO.cpp:114); rows shifted outside [0, n_row) are dropped.  */
tbsla_status_t tbsla_spmv(const tbsla_matrix_t *A, const double *d_x, double *d_y, int vect_incr,
                          void *stream);

/* General form: values read from the `store` copy (TBSLA_F64/F32/BF16);
 * x and y in x_type / y_type (TBSLA_F64 or TBSLA_F32).  Products accumulate
 * in FP64 for the F64 store and in FP32 for the F32/BF16 stores. */
tbsla_status_t tbsla_spmv_ex(const tbsla_matrix_t *A, tbsla_dtype_t store, tbsla_dtype_t x_type,
                             const void *d_x, tbsla_dtype_t y_type, void *d_y, int vect_incr,
                             void *stream);

/* Synchronous host-vector form used by the drop-in classes
 * (std::vector<double> in, std::vector<double> out): x (nx entries) goes to
 * the device (copy engine from pinned memory, an SM copy from pageable
 * memory the device reads coherently), then tbsla_spmv.  When the product
 * writes every row and y (ny >= n_row entries) is pinned or coherently
 * reachable pageable memory, the product writes y in place over NVLink-C2C;
 * otherwise y is copied back. */
tbsla_status_t tbsla_spmv_host(tbsla_matrix_t *A, const double *x, int64_t nx, double *y,
                               int64_t ny, int vect_incr);

/* y = A^T x (CSR handles): the gradient of y = A x with respect to x.  x has
 * n_row entries, y n_col entries (indexed col - f_col).  The transpose is
 * built on the first call (host sort of the entries by column, stable) and
 * kept with the handle; store / types as tbsla_spmv_ex.  No reference
 * counterpart. */
tbsla_status_t tbsla_spmv_transpose_ex(const tbsla_matrix_t *A, tbsla_dtype_t store, tbsla_dtype_t x_type,
                                       const void *d_x, tbsla_dtype_t y_type, void *d_y, void *stream);

/* out[k] = scale * a[row(k)] * b[col(k) - f_col] for every stored entry k of
 * a CSR handle, in its entry order: the gradient of y = A x with respect to
 * the values (a = dL/dy, b = x, scale = 1).  a, b and out are FP64 for
 * type TBSLA_F64, FP32 for TBSLA_F32.  No reference counterpart. */
tbsla_status_t tbsla_csr_grad_values(const tbsla_matrix_t *A, tbsla_dtype_t type, const void *d_a,
                                     const void *d_b, double scale, void *d_out, void *stream);

/* Replaces the values of a CSR handle (entry order of its creation arrays,
 * nnz entries of `type` on the device) and re-derives its reduced-precision
 * stores; the transposed copy follows and cached PageRank state is rebuilt
 * on next use.  No reference counterpart. */
tbsla_status_t tbsla_matrix_set_values(tbsla_matrix_t *A, tbsla_dtype_t type, const void *d_values,
                                       void *stream);

/* Y = A X for a DENSE handle and k vectors, each column of Y one
 * MatrixDENSE::Ax (src/cpp/matrix/MatrixDENSE.cpp:64-73): X column-major
 * ln_col x k (leading dimension ldx), Y column-major n_row x k (ldy); rows
 * past ln_row give 0.  FP64 vectors for the F64 store (cuBLAS DGEMM on the
 * FP64 pipe), FP32 for F32 and BF16, which run on the tensor cores in this
 * library's own kernel (tcgen05 MMA, operands staged by TMA, FP32
 * accumulation in TMEM): the F32 store as TF32 with X read as TF32, the BF16
 * store with X rounded to BF16.  K is split into parts when the row tiles
 * alone do not fill the GPU (TBSLA_TUNE_TC_SPLIT); the parts are summed in
 * part order, so results are reproducible.  Rows of A and vectors of X that
 * do not start on 16-byte boundaries are copied to padded buffers first
 * (ln_col a multiple of 8 for BF16, 4 for F32, and such an ldx avoid it).
 * Work buffers come from the stream-ordered allocator (cudaMallocAsync).
 * A kernel whose bounded wait gave up raises the handle's device status
 * (tbsla_matrix_device_status). */
tbsla_status_t tbsla_dense_spmm(const tbsla_matrix_t *A, tbsla_dtype_t store, int k, const void *d_X,
                                int64_t ldx, void *d_Y, int64_t ldy, void *stream);
/* Synchronises the handle's device and returns in *status, then clears, the
 * handle's device status: nonzero when one of its kernels gave up a bounded
 * wait (its results are then not valid).  No reference counterpart. */
tbsla_status_t tbsla_matrix_device_status(const tbsla_matrix_t *A, int *status);

/* Y = A X for k vectors of a CSR or COO / SCOO handle, X and Y row-major
 * (vector index fastest: X[j*ldx + c] is entry j of vector c, ldx, ldy >= k;
 * X has x_extent rows, Y n_row rows).  FP64 vectors for the F64 store, FP32
 * for F32 and BF16.  Vectors go in panels of up to 32, a group of lanes per
 * row with lane c on vector c: one gather brings a row of X for the panel,
 * and the matrix is streamed once per panel.  FP32 panels of 4, 8 or 12
 * vectors of a handle with the ELL-layout copy (TBSLA_TUNE_SHORT_ROWS 3) are
 * multiplied over the copy instead, one thread per row, when ldx, ldy and
 * the blocks' addresses allow 16-byte loads.  Column c equals the one-vector
 * product of vector c summed in stored order (bit for bit for rows of at most
 * 32 entries with TBSLA_TUNE_SHORT_ROWS = 0).  No reference counterpart (the
 * reference multiplies one vector at a time). */
tbsla_status_t tbsla_spmm(const tbsla_matrix_t *A, tbsla_dtype_t store, int k, const void *d_X, int64_t ldx,
                          void *d_Y, int64_t ldy, void *stream);

/* r = A (A x + x): Matrix::a_axpx_ (Matrix.cpp:6-11), square matrices; the
 * "+ x" is fused into the first product.  d_tmp: n_row doubles of device
 * scratch (required: the call is stream-ordered and holds no handle lock). */
tbsla_status_t tbsla_a_axpx(const tbsla_matrix_t *A, const double *d_x, double *d_r,
                            double *d_tmp, int vect_incr, void *stream);
tbsla_status_t tbsla_a_axpx_host(tbsla_matrix_t *A, const double *x, int64_t nx, double *r,
                                 int64_t nr, int vect_incr);

/* y = A x for row-sorted COO triplets already on the device, without
 * allocating any memory.  This entry point has no counterpart in the
 * reference.  It is for callers that cannot call cudaMalloc: their device
 * memory is owned by another allocator (a framework's caching pool or a
 * fixed arena), or they cannot afford the device-wide synchronisation that
 * cudaMalloc / cudaFree may cause.  Inputs and outputs are the caller's
 * device buffers: d_row (nondecreasing rows in [0, n_row)), d_col (columns in
 * [0, n_col)), d_values, d_x (n_col), d_y (n_row, cleared by the call).  The
 * product's only scratch is a fixed array inside the library (344 KiB per
 * device, held until exit), which limits nnz to 37,748,736 stored entries;
 * larger nnz returns TBSLA_ERR_INVALID_ARG without launching anything.  The
 * first call on a device looks the array up (cudaGetSymbolAddress) and
 * should come before any stream capture on that device.  All calls share the
 * array: calls that overlap on the GPU race and must be ordered by the
 * caller.  The inputs are checked on the device, without waiting: rows that
 * decrease or leave [0, n_row), or columns outside [0, n_col), stop the
 * product before it reads x, and y is filled with NaN. */
tbsla_status_t tbsla_coo_spmv_noalloc(int n_row, int n_col, int64_t nnz, const int *d_row, const int *d_col,
                                      const double *d_values, const double *d_x, double *d_y, void *stream);
/* Waits for `stream` and reports the input check of the device's last
 * tbsla_coo_spmv_noalloc call: *bad = 1 when it failed (y is NaN), else 0. */
tbsla_status_t tbsla_coo_spmv_noalloc_status(int *bad, void *stream);

/* -------------------------------------------------------------- batches */
/* Many CSR handles multiplied together: y_m = A_m x_m for every member in
 * ONE kernel launch (a persistent grid walking row items of every member
 * with a fixed stride, so sums are deterministic; members that keep the
 * ELL-layout copy, TBSLA_TUNE_SHORT_ROWS 3, are read from it for the F64 and
 * F32 stores).  No reference counterpart (the reference multiplies one
 * matrix per call). */
typedef struct tbsla_batch tbsla_batch_t;
/* members: count CSR handles on one device, kept alive by the caller */
tbsla_status_t tbsla_batch_create(int count, const tbsla_matrix_t *const *members, tbsla_batch_t **out);
/* Binds device vectors (host arrays of count device pointers; FP64 for
 * TBSLA_F64, FP32 for the F32 / BF16 stores) and the value store to use. */
tbsla_status_t tbsla_batch_bind(tbsla_batch_t *B, tbsla_dtype_t store, const void *const *d_x, void *const *d_y);
/* d_mask: count ints on the device, members with 0 are skipped (their y is
 * left as it is); NULL: every member.  For iterative callers that stop
 * members independently. */
tbsla_status_t tbsla_batch_set_mask(tbsla_batch_t *B, const int *d_mask);
/* persistent grid of 152 x blocks_per_sm blocks (default 6) */
tbsla_status_t tbsla_batch_tune(tbsla_batch_t *B, int blocks_per_sm);
/* Enqueues the one launch on `stream`: no allocation, no synchronisation. */
tbsla_status_t tbsla_batch_spmv(tbsla_batch_t *B, void *stream);
/* The same launch replayed from a CUDA graph built on the first call (it
 * reads the member table, so later tbsla_batch_bind calls apply to it). */
tbsla_status_t tbsla_batch_spmv_graph(tbsla_batch_t *B, void *stream);
tbsla_status_t tbsla_batch_destroy(tbsla_batch_t *B);

/* ------------------------------------------------------------ autotune */
/* Tuners: each times its candidates with CUDA events on the caller's data
 * and keeps the fastest in the handle (results never change, only times).
 * No reference counterpart. */
typedef struct {
  int candidates;   /* candidates timed                         */
  float best_ms;    /* time of the kept one                     */
  int choice;       /* spmv: 0 direct, 1 row blocks, 2 staged short rows,
                       3 two lanes per short row, 4 warp tiles of tiny
                       rows (every row at most 4 entries), 5 the
                       ELL-layout copy (TBSLA_TUNE_SHORT_ROWS 3);
                       batch: blocks per SM; ppr: tile */
  double value;     /* spmv: x L2-keep fraction; otherwise = choice */
} tbsla_autotune_result_t;
/* CSR kernel variant, TBSLA_TUNE_SHORT_ROWS and TBSLA_TUNE_X_L2_KEEP for the
 * `store` product (COO / SCOO: the staged kernel and the keep fraction) */
tbsla_status_t tbsla_autotune_spmv(tbsla_matrix_t *A, tbsla_dtype_t store, tbsla_autotune_result_t *res);
/* persistent grid of a bound batch */
tbsla_status_t tbsla_autotune_batch(tbsla_batch_t *B, tbsla_autotune_result_t *res);
/* tile width of tbsla_ppr_batched for k vectors (used when it gets tile 0) */
tbsla_status_t tbsla_autotune_ppr(tbsla_matrix_t *A, int k, tbsla_dtype_t precision, tbsla_autotune_result_t *res);

/* ----------------------------------------------------------- PageRank */
typedef enum {
  /* Matrix::page_rank (Matrix.cpp:13-61): b0 = 1; b = beta*A b + (1-beta)/n *
   * sum(b_prev); b /= max(b); stop when sum|b - b_prev| < tol; finally
   * b /= sum(b).  No dangling term. */
  TBSLA_PR_REFERENCE = 0,
  /* x0 = 1/n; x = beta*A x + (beta*dangling(x) + (1-beta)*sum(x))/n, where
   * dangling(x) sums x over columns of A with no stored entry; stop when
   * ||x - x_prev||_1 < tol.  Result sums to 1. */
  TBSLA_PR_DANGLING = 1,
  /* The same fixed point with a teleport vector v (tbsla_pagerank_teleport):
   * x0 = v; x = beta*A x + (beta*dangling(x) + (1-beta)) v; stop when
   * ||x - x_prev||_1 < tol.  This is the affine form of TBSLA_PR_DANGLING (for
   * a column-stochastic A and v = 1/n they agree) and the function that
   * tbsla_pagerank_adjoint differentiates.  FP64 only; no normalisation. */
  TBSLA_PR_TELEPORT = 2
} tbsla_pr_mode_t;

typedef struct {
  double beta;        /* damping, the reference's beta                     */
  double tol;         /* stopping threshold, the reference's epsilon       */
  int max_iter;       /* the reference's max_iteration                     */
  int mode;           /* tbsla_pr_mode_t                                   */
  int precision;      /* TBSLA_F64: plain FP64 sweeps.  TBSLA_F32 / TBSLA_BF16:
                         low-precision sweeps on that value store with FP32
                         vectors, corrected by FP64 residual refinement
                         (TBSLA_PR_DANGLING only; needs TBSLA_STORE_F64 too) */
  int check_every;    /* sweeps per convergence check (0: library default) */
  int accel;          /* dangling and teleport modes, and the adjoint:
                         0 power iteration; 1 Anderson acceleration over
                         the last two differences (the next sweep starts
                         from the combination of the last three sweep
                         outputs whose residual combination is smallest in
                         the 2-norm); same stopping rule, same fixed point,
                         fewer sweeps.  With precision TBSLA_F32 / TBSLA_BF16
                         the low-precision correction solves are the
                         accelerated ones (FP32 vectors; an F32 store is
                         then solved to 1e-4 of ||r|| per correction, BF16
                         to 0.05) */
} tbsla_pagerank_params_t;

typedef struct {
  int iterations;     /* sweeps done (FP64 + low precision)                */
  int iterations_f64; /* of which FP64 sweeps                              */
  double residual;    /* last stopping quantity                            */
  int converged;      /* 1 if tol was reached                              */
} tbsla_pagerank_result_t;

/* d_out: n_col doubles on the device.  Returns TBSLA_OK also when max_iter
 * is hit without convergence (as the reference does); check
 * result->converged. */
tbsla_status_t tbsla_pagerank(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p,
                              double *d_out, tbsla_pagerank_result_t *result, void *stream);
tbsla_status_t tbsla_pagerank_host(tbsla_matrix_t *A, const tbsla_pagerank_params_t *p,
                                   double *out, int64_t n_out, tbsla_pagerank_result_t *result);

/* TBSLA_PR_TELEPORT with the teleport vector d_v (n_col doubles on the
 * device); p->mode is ignored.  No reference counterpart. */
tbsla_status_t tbsla_pagerank_teleport(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p,
                                       const double *d_v, double *d_out, tbsla_pagerank_result_t *result,
                                       void *stream);

/* Gradients of L(x*) through the TBSLA_PR_TELEPORT fixed point x* of A
 * (square CSR).  With d the dangling columns of A and w = dL/dx* (d_w), the
 * adjoint lambda solves lambda = beta*A^T lambda + beta*d*(v . lambda) + w
 * (sweeps on the transpose, stopped when ||lambda - lambda_prev||_1 < p->tol
 * or after p->max_iter sweeps); then
 *   dL/dvalues[k] = beta * lambda[row(k)] * x*[col(k)]   (d_grad_values, nnz
 *                   doubles in the handle's entry order; NULL to skip)
 *   dL/dv         = (beta * d . x* + 1 - beta) * lambda  (d_grad_v, n; NULL
 *                   to skip)
 * d_v: the teleport vector of the forward solve (NULL: uniform 1/n); d_x: x*.
 * The dangling set is structural (columns with no stored entry).  No
 * reference counterpart. */
tbsla_status_t tbsla_pagerank_adjoint(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p,
                                      const double *d_v, const double *d_x, const double *d_w,
                                      double *d_grad_values, double *d_grad_v,
                                      tbsla_pagerank_result_t *result, void *stream);

/* k personalized PageRank vectors of one square CSR graph solved together
 * (TBSLA_PR_TELEPORT form): vector c teleports uniformly to its seed set
 * nodes[offsets[c] .. offsets[c+1]) (repeated seeds count once), and stops on
 * its own when its L1 change is below p->tol or after p->max_iter sweeps;
 * stopped vectors are frozen while the others continue.  The iterates are
 * multiplied in tiles of `tile` vectors (2, 4, 8, 16 or 32; 0 picks one) as one
 * multi-vector product per tile.  Every p->check_every sweeps (0: 4) the
 * stopped vectors are written out and the running ones repacked into as few
 * tiles as hold them; each result equals the vector solved alone bit for
 * bit.  p->precision: TBSLA_F64, or TBSLA_F32
 * (F32 value store and FP32 iterates).  p->accel = 1: each vector's solve is
 * Anderson-accelerated (the combination of its last three sweep outputs
 * whose residual combination is smallest, as in tbsla_pagerank; same
 * stopping rule and fixed point, fewer sweeps).  d_out: n*k doubles, vector
 * c at d_out + c*n; iterations / residuals: k host entries each, or NULL.
 * Allocates its work buffers per call: 2 n k values of the precision, 7 n k
 * with acceleration (iterate, three outputs, three residuals).  No reference
 * counterpart. */
tbsla_status_t tbsla_ppr_batched(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p, int k,
                                 const int *nodes, const int *offsets, int tile, double *d_out, int *iterations,
                                 double *residuals, void *stream);

/* As tbsla_ppr_batched with p->precision = TBSLA_F32, corrected to FP64
 * accuracy (the F64 and F32 value stores are needed): the FP32 batched solve
 * (stopped at max(p->tol, 1e-6)), then rounds of r = G(x) - x by one FP64
 * sweep of every vector; when every ||r_c||_1 < p->tol the result is G(x),
 * else the FP32 batched correction solve e = beta A e + beta (d.e) v_c + r_c
 * (from e = r_c, to ||e_j+1 - e_j||_1 < 1e-3 ||r_c||_1, 1e-4 with
 * p->accel = 1, whose FP32 solves are accelerated) and x += e, at most
 * 8 rounds.  FP64 is used only for the residual sweeps, the L1 norms and the
 * update.  iterations: FP32 and FP64 sweeps together; residuals: the last
 * ||r_c||_1.  Allocates 2 n k doubles of work space per call (stream
 * ordered).  No reference counterpart. */
tbsla_status_t tbsla_ppr_batched_refined(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p, int k,
                                         const int *nodes, const int *offsets, int tile, double *d_out,
                                         int *iterations, double *residuals, void *stream);

/* Matrix::personalized_page_rank (Matrix.cpp:63-114): as TBSLA_PR_REFERENCE
 * with b0 = 0.25 and the teleport term (1-beta)*sum(b_prev)/n_nodes added only
 * to the listed nodes (a node listed twice counts once but n_nodes is the
 * list length, as std::find over the list gives). */
tbsla_status_t tbsla_personalized_pagerank_host(tbsla_matrix_t *A, const tbsla_pagerank_params_t *p,
                                                const int *nodes, int n_nodes, double *out,
                                                int64_t n_out, tbsla_pagerank_result_t *result);

/* COO / SCOO handle -> CSR handle, on the device: MatrixCSR(const
 * MatrixCOO&) (MatrixCSR.cpp:29-74) with entries ordered by (row, column),
 * equal pairs in input order (the host conversion's arrays, bit for bit).
 * stores: the value stores of the new handle (the COO handle needs F64). */
tbsla_status_t tbsla_coo_to_csr(const tbsla_matrix_t *coo, int stores, tbsla_matrix_t **out);
/* COO / SCOO handle -> ELL handle on the device: MatrixELL(const MatrixCOO&)
 * (MatrixELL.cpp:12-53): max_col = the longest row, row i's entries in
 * (row, column) order in slots 0..len-1, padding slots column 0 / value 0.
 * The handle equals tbsla_ell_create on the host conversion's arrays. */
tbsla_status_t tbsla_coo_to_ell(const tbsla_matrix_t *coo, int stores, tbsla_matrix_t **out);
/* COO / SCOO handle -> DENSE handle (n_row x n_col) on the device:
 * MatrixDENSE(const MatrixCOO&) (MatrixDENSE.cpp:11-28), repeated (row,
 * column) pairs added to 0 in input order.  Stored columns must lie below
 * n_col (the reference indexes the dense row with them). */
tbsla_status_t tbsla_coo_to_dense(const tbsla_matrix_t *coo, int stores, tbsla_matrix_t **out);
/* COO handle -> SCOO handle: MatrixSCOO(const MatrixCOO&) (MatrixSCOO.cpp:
 * 53-68) copies the arrays; here a device-to-device copy of the handle. */
tbsla_status_t tbsla_coo_to_scoo(const tbsla_matrix_t *coo, int stores, tbsla_matrix_t **out);
/* MatrixCSR::normalize_columns (MatrixCSR.cpp:423-435) on the device: each
 * value divided by its column's sum, the sums accumulated in the reference's
 * order (bit-identical values).  Derived stores and copies are refreshed. */
tbsla_status_t tbsla_csr_normalize_columns(tbsla_matrix_t *A, void *stream);
/* host copies in the reference's layouts: ELL columns / values row-major
 * (rows x max_col, MatrixELL::get_columns / get_values); DENSE values
 * (rows x ln_col).  Either pointer may be NULL. */
tbsla_status_t tbsla_ell_download(const tbsla_matrix_t *A, int *columns, double *values);
tbsla_status_t tbsla_dense_download(const tbsla_matrix_t *A, double *values);

/* ---------------------------------------------------------------- files */
/* A handle (F64 store) from a file in the reference's binary matrix layout
 * of `format`, starting at byte `seek`: what Matrix*::read reads
 * (MatrixCSR.cpp:206-232 and the matching read of each format).  Files the
 * reference's write produced load as they are. */
tbsla_status_t tbsla_matrix_read_file(const char *path, int format, int64_t seek, tbsla_matrix_t **out);
/* A handle (F64 store) of `format` from a Matrix Market file: "matrix
 * coordinate real general|symmetric" as MatrixCOO::readMM reads it
 * (MatrixCOO.cpp:230-292, including its echo of the banner and size lines to
 * stdout), converted as MatrixCSR(COO) / MatrixELL(COO) / MatrixSCOO(COO) /
 * MatrixDENSE(COO) do.  Other kinds: TBSLA_ERR_UNSUPPORTED. */
tbsla_status_t tbsla_matrix_read_mm(const char *path, int format, tbsla_matrix_t **out);

/* ---------------------------------------------------------- generators */
/* Host-side builders of the reference's synthetic matrices, in the
 * reference's own array layout, so that the drop-in classes and the C_CPP_*
 * ABI return exactly the reference's arrays.  Two-call protocol: call with
 * NULL arrays to get the sizes in *sizes, allocate, call again.
 *   sizes[0] = values length, sizes[1] = idx0 length (row / rowptr /
 *   columns), sizes[2] = idx1 length (col / colidx)
 *   geom[0..10] = n_row, n_col, ln_row, ln_col, f_row, f_col, pr, pc, NR, NC,
 *   max_col;  *nnz = the reference's nnz field.
 * gen: 0 = cqmat (Matrix*::fill_cqmat), 1 = cdiag (fill_cdiag),
 *      2 = cqmat_stochastic (fill_cqmat_stochastic),
 *      3 = cqmat_baseline: the cqmat pattern of fill_cqmat with duplicates
 *          merged (each row's columns sorted, repeats kept once) and values
 *          uniform in (0, 1]: value k in (row, column) order is 1 - u_k with
 *          u_k = (splitmix64(((uint64_t)1 << 32 | seed_mult) + (k+1) *
 *          0x9e3779b97f4a7c15) >> 11) * 2^-53 (SplitMix64, Steele, Lea and
 *          Flood 2014); whole matrix only (pr,pc,NR,NC = 0,0,1,1).  ELL and
 *          DENSE arrays are those of MatrixELL(COO) / MatrixDENSE(COO).  No
 *          reference counterpart beyond the pattern: it is the benchmark's
 *          cqmat with merged duplicates and random values. */
tbsla_status_t tbsla_generate(int format, int gen, int n_row, int n_col, int c, double q,
                              unsigned int seed_mult, int pr, int pc, int NR, int NC,
                              int64_t sizes[3], int geom[11], int64_t *nnz, double *values,
                              int *idx0, int *idx1);

/* One-pass form: builds the block (pr,pc,NR,NC) = (0,0,1,1) of the chosen
 * generator and uploads it as a handle of `format` with the given value
 * stores (the matrices tbsla_perf times, src/cpp/apps/tbsla_perf.cpp:111-119). */
tbsla_status_t tbsla_generate_matrix(int format, int gen, int n_row, int n_col, int c, double q,
                                     unsigned int seed_mult, int stores, tbsla_matrix_t **out);

/* tbsla_generate_matrix built on the device, for the block (pr, pc, NR, NC):
 * gen 1 (cdiag) for CSR, ELL and DENSE is generated on the device (closed
 * form per row: the arrays of MatrixCSR / MatrixELL / MatrixDENSE::fill_cdiag,
 * src/cpp/matrix/MatrixCSR.cpp:234-297, MatrixELL.cpp:192-260,
 * MatrixDENSE.cpp:137-190, bit for bit); gen 2 (cqmat_stochastic) for CSR,
 * ELL and DENSE takes fill_cqmat's pattern and the column sums of the global
 * generator from the host (glibc rand_r draws) and divides on the device
 * (MatrixCSR.cpp:411-421, MatrixELL.cpp:394-404, MatrixDENSE.cpp:273-286).
 * Other formats and generators: the host path, whole matrix only. */
tbsla_status_t tbsla_generate_device(int format, int gen, int n_row, int n_col, int c, double q,
                                     unsigned int seed_mult, int pr, int pc, int NR, int NC, int stores,
                                     tbsla_matrix_t **out);

/* R-MAT digraph with 2^scale nodes and m edge draws (Chakrabarti, Zhan,
 * Faloutsos 2004), generated on the device with counter-based draws, as the
 * column-stochastic PageRank matrix: row = destination, column = source,
 * repeated edges merged, value 1/outdeg(source).  The product is a CSR
 * handle with the requested value stores. */
tbsla_status_t tbsla_rmat_pagerank_matrix(int scale, int64_t m, double a, double b, double c,
                                          uint64_t seed, int stores, tbsla_matrix_t **out);
/* host copy of a CSR handle's arrays (rowptr rows+1, colidx/values nnz) */
tbsla_status_t tbsla_csr_download(const tbsla_matrix_t *A, int *rowptr, int *colidx,
                                  double *values);

/* ---------------------------------------------------------- utilities */
/* sizes of device buffers; simple wrappers so that C callers need no CUDA
 * headers */
tbsla_status_t tbsla_device_alloc(void **ptr, size_t bytes);
tbsla_status_t tbsla_device_free(void *ptr);
tbsla_status_t tbsla_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream);
tbsla_status_t tbsla_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream);
tbsla_status_t tbsla_stream_sync(void *stream);
/* page-locked host buffers (fast host<->device copies for the *_host calls) */
tbsla_status_t tbsla_host_alloc(void **ptr, size_t bytes);
tbsla_status_t tbsla_host_free(void *ptr);

/* Kernel timing: when enabled, every product launched on A records CUDA
 * events around its main kernel on the launching stream; the accumulated
 * device time and launch count are read (synchronising on the events) and
 * reset with tbsla_kernel_timing_read. */
tbsla_status_t tbsla_kernel_timing_enable(tbsla_matrix_t *A, int enable);
tbsla_status_t tbsla_kernel_timing_read(tbsla_matrix_t *A, double *total_ms, int64_t *launches);

#ifdef __cplusplus
}
#endif
#endif
