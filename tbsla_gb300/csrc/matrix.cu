// matrix.cu -- matrix handles of the C ABI: creation from host arrays in the
// reference's layouts, device layouts, SpMV / a_axpx dispatch.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
#include "product.cuh"

namespace tbsla {

// ------------------------------------------------------------- errors
static thread_local std::string g_err;
static int g_device = -1;

tbsla_status_t fail(tbsla_status_t s, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return s;
}

tbsla_status_t cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  const tbsla_status_t s = e == cudaErrorMemoryAllocation ? TBSLA_ERR_OOM : TBSLA_ERR_CUDA;
  return fail(s, "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

int current_device() {
  int d = 0;
  if (g_device >= 0) return g_device;
  cudaGetDevice(&d);
  return d;
}

tbsla_status_t dev_alloc(tbsla_matrix *A, void **p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  // 64 spare bytes: vector loads and 16-byte aligned bulk copies of a
  // ragged end stay inside the allocation
  cudaError_t e = cudaMalloc(p, bytes + 64);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(TBSLA_ERR_OOM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
  }
  if (A) A->device_bytes += (int64_t)bytes + 64;
  return TBSLA_OK;
}

KernelTimer::KernelTimer(const tbsla_matrix *A_, cudaStream_t s_) : A(const_cast<tbsla_matrix *>(A_)), s(s_) {
  if (!A || !A->timing) return;
  if (!A->free_events.empty()) {
    e0 = A->free_events.back().first;
    e1 = A->free_events.back().second;
    A->free_events.pop_back();
  } else if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    e0 = e1 = nullptr;
    return;
  }
  cudaEventRecord(e0, s);
}

void KernelTimer::stop() {
  if (!e0) return;
  cudaEventRecord(e1, s);
  A->pending_events.emplace_back(e0, e1);
  e0 = e1 = nullptr;
}

template <typename T> static tbsla_status_t alloc_n(tbsla_matrix *A, T **p, int64_t n) {
  return dev_alloc(A, reinterpret_cast<void **>(p), (size_t)std::max<int64_t>(n, 1) * sizeof(T));
}

tbsla_status_t ensure_host_buffers(tbsla_matrix *A, int64_t nx, int64_t ny, int64_t nt) {
  if (!A->stream) TB_CUDA(cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking));
  if (nx > A->cap_x) {
    if (A->d_x) cudaFree(A->d_x);
    A->d_x = nullptr;
    TB_TRY(alloc_n(A, &A->d_x, nx));
    A->cap_x = nx;
  }
  if (ny > A->cap_y) {
    if (A->d_y) cudaFree(A->d_y);
    A->d_y = nullptr;
    TB_TRY(alloc_n(A, &A->d_y, ny));
    A->cap_y = ny;
  }
  if (nt > A->cap_t) {
    if (A->d_t) cudaFree(A->d_t);
    A->d_t = nullptr;
    TB_TRY(alloc_n(A, &A->d_t, nt));
    A->cap_t = nt;
  }
  return TBSLA_OK;
}

// ------------------------------------------------------- value stores
__global__ void f64_to_f32_kernel(const double *in, float *out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __double2float_rn(in[i]);
}
__global__ void f64_to_bf16_kernel(const double *in, __nv_bfloat16 *out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __double2bfloat16(in[i]);
}

__global__ void f32_to_f64_kernel(const float *in, double *out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}

static int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 32);
}

// Uploads n FP64 values and derives the requested reduced stores on the
// device.  `host` may hold the values in any order the caller prepared.
static tbsla_status_t upload_values(tbsla_matrix *A, const double *host, int64_t n, int stores) {
  if (!(stores & (TBSLA_STORE_F64 | TBSLA_STORE_F32 | TBSLA_STORE_BF16)))
    return fail(TBSLA_ERR_INVALID_ARG, "no value store requested");
  double *d64 = nullptr;
  TB_TRY(alloc_n(A, &d64, n));
  if (n) TB_CUDA(cudaMemcpy(d64, host, n * sizeof(double), cudaMemcpyHostToDevice));
  if (stores & TBSLA_STORE_F32) {
    float *d = nullptr;
    TB_TRY(alloc_n(A, &d, n));
    if (n) f64_to_f32_kernel<<<grid_for(n, 256), 256>>>(d64, d, n);
    A->values[1] = d;
  }
  if (stores & TBSLA_STORE_BF16) {
    __nv_bfloat16 *d = nullptr;
    TB_TRY(alloc_n(A, &d, n));
    if (n) f64_to_bf16_kernel<<<grid_for(n, 256), 256>>>(d64, d, n);
    A->values[2] = d;
  }
  TB_CUDA(cudaGetLastError());
  if (stores & TBSLA_STORE_F64) {
    A->values[0] = d64;
  } else {
    TB_CUDA(cudaDeviceSynchronize());
    cudaFree(d64);
    A->device_bytes -= (int64_t)std::max<int64_t>(n, 1) * 8 + 64;
  }
  A->stores = stores & (TBSLA_STORE_F64 | TBSLA_STORE_F32 | TBSLA_STORE_BF16);
  return TBSLA_OK;
}

// The sliced copies of A's value stores (csr_sell_kernel) from the stores
static tbsla_status_t sell_refresh(tbsla_matrix *A, cudaStream_t s) {
  if (!A->sell_width) return TBSLA_OK;
  const int *rp = A->format == TBSLA_FMT_CSR ? A->idx0 : A->coo_rowptr;
  const int grid = grid_for(A->rows, 256);
  if (A->values[0])
    sell_scatter_kernel<double><<<grid, 256, 0, s>>>(rp, A->sell_stride, A->rows,
                                                     static_cast<const double *>(A->values[0]),
                                                     static_cast<double *>(A->sell_vals[0]));
  if (A->values[1])
    sell_scatter_kernel<float><<<grid, 256, 0, s>>>(rp, A->sell_stride, A->rows,
                                                    static_cast<const float *>(A->values[1]),
                                                    static_cast<float *>(A->sell_vals[1]));
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

// The F32 / BF16 stores of A recomputed from its F64 store (and the sliced
// copies of all stores)
tbsla_status_t rederive_stores(tbsla_matrix *A, cudaStream_t s) {
  const int64_t n = A->format == TBSLA_FMT_ELL ? (int64_t)A->rows_pad * A->max_col : A->stored;
  if (!A->values[0] || n == 0) return TBSLA_OK;
  const double *v = static_cast<const double *>(A->values[0]);
  if (A->values[1]) f64_to_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(v, static_cast<float *>(A->values[1]), n);
  if (A->values[2])
    f64_to_bf16_kernel<<<grid_for(n, 256), 256, 0, s>>>(v, static_cast<__nv_bfloat16 *>(A->values[2]), n);
  TB_CUDA(cudaGetLastError());
  return sell_refresh(A, s);
}

tbsla_status_t transpose_refresh(tbsla_matrix *A, cudaStream_t s);

// As upload_values, from FP64 values already on the device (d_src, n)
tbsla_status_t store_values_device(tbsla_matrix *A, const double *d_src, int64_t n, int stores, cudaStream_t s) {
  if (!(stores & (TBSLA_STORE_F64 | TBSLA_STORE_F32 | TBSLA_STORE_BF16)))
    return fail(TBSLA_ERR_INVALID_ARG, "no value store requested");
  double *d64 = nullptr;
  TB_TRY(alloc_n(A, &d64, n));
  if (n) TB_CUDA(cudaMemcpyAsync(d64, d_src, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  A->values[0] = d64;
  A->stores = stores & (TBSLA_STORE_F64 | TBSLA_STORE_F32 | TBSLA_STORE_BF16);
  if (stores & TBSLA_STORE_F32) {
    float *d = nullptr;
    TB_TRY(alloc_n(A, &d, n));
    A->values[1] = d;
  }
  if (stores & TBSLA_STORE_BF16) {
    __nv_bfloat16 *d = nullptr;
    TB_TRY(alloc_n(A, &d, n));
    A->values[2] = d;
  }
  TB_TRY(rederive_stores(A, s));
  TB_CUDA(cudaStreamSynchronize(s));
  if (!(stores & TBSLA_STORE_F64)) {
    cudaFree(d64);
    A->values[0] = nullptr;
    A->device_bytes -= (int64_t)std::max<int64_t>(n, 1) * 8 + 64;
  }
  return TBSLA_OK;
}

tbsla_matrix *new_matrix(int format);
void free_matrix(tbsla_matrix *A);

tbsla_status_t alloc_carries(tbsla_matrix *A) {
  const int nt = std::max(A->num_tiles, 1);
  TB_TRY(alloc_n(A, &A->tile_head_row, nt));
  TB_TRY(alloc_n(A, &A->tile_head_val, nt));
  TB_TRY(alloc_n(A, &A->tile_tail_val, nt));
  TB_TRY(alloc_n(A, &A->tile_emitted, nt));
  TB_TRY(alloc_n(A, &A->tile_head_val32, nt));
  TB_TRY(alloc_n(A, &A->tile_tail_val32, nt));
  TB_TRY(alloc_n(A, &A->d_err, 1));
  TB_CUDA(cudaMemset(A->d_err, 0, sizeof(int)));
  return TBSLA_OK;
}

tbsla_status_t csr_bins(tbsla_matrix *A, const std::vector<int> &rp);

static tbsla_matrix *new_handle(int format) {
  tbsla_matrix *A = new (std::nothrow) tbsla_matrix();
  if (!A) return nullptr;
  A->format = format;
  A->device = current_device();
  cudaSetDevice(A->device);
  return A;
}

static void free_handle(tbsla_matrix *A) {
  if (!A) return;
  cudaSetDevice(A->device);
  if (A->pr_work && A->pr_work_free) A->pr_work_free(A->pr_work);
  if (A->ppr_plan && A->ppr_plan_free) A->ppr_plan_free(A->ppr_plan);
  if (A->pr_relabel) free_handle(A->pr_relabel);
  if (A->transpose) free_handle(A->transpose);
  for (void *p : A->values) if (p) cudaFree(p);
  void *ptrs[] = {A->idx0, A->idx1, A->row_blocks, A->huge_rows, A->huge_partials, A->huge_partials32,
                  A->short_rows, A->warp_items, A->chunk_rows, A->chunk_partials, A->chunk_partials32,
                  A->tile_start, A->tile_head_row, A->tile_head_val,
                  A->tile_tail_val, A->tile_emitted, A->tile_head_val32, A->tile_tail_val32,
                  A->dangling, A->pr_scratch, A->d_x, A->d_y, A->d_t, A->d_err, A->pr_newid, A->pr_out,
                  A->transpose_perm, A->coo_rowptr, A->sell_cols, A->sell_vals[0], A->sell_vals[1],
                  A->sell_vals[2]};
  for (void *p : ptrs) if (p) cudaFree(p);
  if (A->stream) cudaStreamDestroy(A->stream);
  for (auto &e : A->pending_events) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  for (auto &e : A->free_events) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  delete A;
}

// The short-row list back in row order, without the tiny head: for copies
// whose rows are already grouped by length (the degree-relabelled PageRank
// graph), where the one-thread-per-row kernel over the whole list measured
// faster (R-MAT 2^24 FP64 solve 44.7 ms against 47.4 ms with the split).
tbsla_status_t csr_unsplit_tiny(tbsla_matrix *A) {
  if (A->n_tiny == 0 || !A->short_rows) return TBSLA_OK;
  std::vector<int> rows((size_t)A->n_short);
  TB_CUDA(cudaMemcpy(rows.data(), A->short_rows, rows.size() * sizeof(int), cudaMemcpyDeviceToHost));
  std::sort(rows.begin(), rows.end());
  TB_CUDA(cudaMemcpy(A->short_rows, rows.data(), rows.size() * sizeof(int), cudaMemcpyHostToDevice));
  A->n_tiny = 0;
  return TBSLA_OK;
}

tbsla_matrix *new_matrix(int format) { return new_handle(format); }
void free_matrix(tbsla_matrix *A) { free_handle(A); }
tbsla_status_t alloc_ints(tbsla_matrix *A, int **p, int64_t n) { return alloc_n(A, p, n); }

tbsla_status_t axpy_inplace(double *y, const double *x, int64_t n, cudaStream_t s);

// y rows the format never writes are zeroed first: COO/SCOO rows without
// entries, CSR/ELL/DENSE rows past A->rows, and everything when the
// reference's early exits apply
static tbsla_status_t zero_unwritten(const tbsla_matrix *A, void *y, size_t elt, int vect_incr,
                                     cudaStream_t s) {
  if (A->n_row <= 0) return TBSLA_OK;
  if (A->format == TBSLA_FMT_COO || A->format == TBSLA_FMT_SCOO) {
    // the direct kernels write every row (empty rows as 0) unless rows are shifted
    if (A->coo_rowptr && A->csr_variant == 0 && vect_incr == 0 && A->stored > 0) return TBSLA_OK;
    TB_CUDA(cudaMemsetAsync(y, 0, (size_t)A->n_row * elt, s));
    return TBSLA_OK;
  }
  (void)vect_incr;
  int written = A->rows;
  if (A->format == TBSLA_FMT_ELL && A->max_col == 0) written = 0;
  if (A->format == TBSLA_FMT_DENSE && A->cols == 0) written = 0;
  if (A->format == TBSLA_FMT_CSR && A->stored == 0) written = 0;
  written = std::min(written, A->n_row);
  if (written < A->n_row)
    TB_CUDA(cudaMemsetAsync(static_cast<char *>(y) + (size_t)written * elt, 0,
                            (size_t)(A->n_row - written) * elt, s));
  return TBSLA_OK;
}

static int out_shift(const tbsla_matrix *A, int vect_incr) {
  if (A->format == TBSLA_FMT_COO || A->format == TBSLA_FMT_SCOO) return vect_incr - A->f_row;
  return 0;
}

template <typename V, typename XT, typename YT>
static tbsla_status_t spmv_typed(const tbsla_matrix *A, const V *vals, const XT *x, YT *y,
                                 int vect_incr, cudaStream_t s) {
  using Acc = typename AccOf<V>::type;
  TB_TRY(zero_unwritten(A, y, sizeof(YT), vect_incr, s));
  if (A->format == TBSLA_FMT_CSR && A->stored == 0) return TBSLA_OK;  // MatrixCSR.cpp:130-131
  StoreEpi<YT, Acc> epi{y, A->n_row, out_shift(A, vect_incr)};
  return launch_product<V, XT>(A, vals, x, epi, s);
}

tbsla_status_t spmv_dispatch(const tbsla_matrix *A, tbsla_dtype_t store, tbsla_dtype_t xt,
                             const void *x, tbsla_dtype_t yt, void *y, int vect_incr,
                             cudaStream_t s) {
  const int si = store_index(store);
  const void *vals = A->values[si];
  if (!vals) return fail(TBSLA_ERR_INVALID_ARG, "value store %d not present in this handle", (int)store);
  if (xt != TBSLA_F64 && xt != TBSLA_F32) return fail(TBSLA_ERR_INVALID_ARG, "x type must be F64 or F32");
  if (yt != TBSLA_F64 && yt != TBSLA_F32) return fail(TBSLA_ERR_INVALID_ARG, "y type must be F64 or F32");
#define TB_SPMV_CASE(VT)                                                                          \
  {                                                                                               \
    const VT *v = static_cast<const VT *>(vals);                                                  \
    if (xt == TBSLA_F64 && yt == TBSLA_F64)                                                       \
      return spmv_typed(A, v, static_cast<const double *>(x), static_cast<double *>(y), vect_incr, s); \
    if (xt == TBSLA_F32 && yt == TBSLA_F32)                                                       \
      return spmv_typed(A, v, static_cast<const float *>(x), static_cast<float *>(y), vect_incr, s); \
    if (xt == TBSLA_F64 && yt == TBSLA_F32)                                                       \
      return spmv_typed(A, v, static_cast<const double *>(x), static_cast<float *>(y), vect_incr, s); \
    return spmv_typed(A, v, static_cast<const float *>(x), static_cast<double *>(y), vect_incr, s); \
  }
  if (si == 0) TB_SPMV_CASE(double)
  if (si == 1) TB_SPMV_CASE(float)
  TB_SPMV_CASE(__nv_bfloat16)
#undef TB_SPMV_CASE
}

tbsla_status_t a_axpx_dispatch(const tbsla_matrix *A, const double *x, double *r, double *tmp,
                               int vect_incr, cudaStream_t s) {
  const double *vals = static_cast<const double *>(A->values[0]);
  if (!vals) return fail(TBSLA_ERR_INVALID_ARG, "a_axpx needs the F64 value store");
  // tmp = A x + x (rows never written by the product stay x, as r(0)+v)
  TB_TRY(zero_unwritten(A, tmp, sizeof(double), vect_incr, s));
  const bool empty = (A->format == TBSLA_FMT_CSR && A->stored == 0);
  if (A->format == TBSLA_FMT_COO || A->format == TBSLA_FMT_SCOO || empty || A->rows < A->n_row ||
      (A->format == TBSLA_FMT_ELL && A->max_col == 0) || (A->format == TBSLA_FMT_DENSE && A->cols == 0)) {
    // rows without a product still get "+ x": run the plain product, then add
    if (!empty) {
      StoreEpi<double, double> epi{tmp, A->n_row, out_shift(A, vect_incr)};
      TB_TRY(launch_product<double, double>(A, vals, x, epi, s));
    }
    // tmp += x
    TB_TRY(axpy_inplace(tmp, x, A->n_row, s));
  } else {
    AddXEpi<double> epi{tmp, x, A->n_row, out_shift(A, vect_incr)};
    TB_TRY(launch_product<double, double>(A, vals, x, epi, s));
  }
  return spmv_typed<double, double, double>(A, vals, tmp, r, vect_incr, s);
}

__global__ void axpy_kernel(double *y, const double *x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += x[i];
}
tbsla_status_t axpy_inplace(double *y, const double *x, int64_t n, cudaStream_t s) {
  if (n <= 0) return TBSLA_OK;
  axpy_kernel<<<grid_for(n, 256), 256, 0, s>>>(y, x, n);
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

// ------------------------------------------------------------ creation
// Cuts rows [0, rows) into blocks of csr_rows_kernel: at most kRowsMax rows,
// kRowsMax segments (of at most kSeg nonzeros) and kRowsCap nonzeros per
// block; a row longer than kRowsCap is huge and gets one block per chunk.
static void plan_row_blocks(const std::vector<int> &rp, std::vector<int4> &blocks,
                            std::vector<int2> &huge, int *n_partials) {
  const int rows = (int)rp.size() - 1;
  int slot = 0, cur_r0 = 0, cur_rows = 0, cur_segs = 0, cur_nnz = 0;
  auto close = [&](int r_end) {
    if (cur_rows > 0) blocks.push_back(make_int4(cur_r0, r_end, rp[cur_r0], -1));
    cur_rows = 0;
    cur_segs = 0;
    cur_nnz = 0;
  };
  for (int r = 0; r < rows; ++r) {
    const int len = rp[r + 1] - rp[r];
    const int nseg = len > kSeg ? (len + kSeg - 1) / kSeg : 1;
    if (len > kRowsCap) {
      close(r);
      huge.push_back(make_int2(r, slot));
      for (int c = 0; c < len; c += kRowsCap) blocks.push_back(make_int4(r, r + 1, rp[r] + c, slot++));
      cur_r0 = r + 1;
      continue;
    }
    if (cur_rows + 1 > kRowsMax || cur_segs + nseg > kRowsMax || cur_nnz + len > kRowsCap) {
      close(r);
      cur_r0 = r;
    }
    if (cur_rows == 0) cur_r0 = r;
    ++cur_rows;
    cur_segs += nseg;
    cur_nnz += len;
  }
  close(rows);
  huge.push_back(make_int2(-1, slot));
  *n_partials = slot;
}

static tbsla_status_t build_csr(tbsla_matrix *A, const int *rowptr, const int *colidx,
                                const double *values, int stores) {
  const int rows = A->rows;
  const int base = rowptr[0];
  const int64_t nnz = (int64_t)rowptr[rows] - base;
  if (nnz < 0 || nnz > INT_MAX) return fail(TBSLA_ERR_INVALID_ARG, "bad rowptr range");
  if ((int64_t)rows + nnz > INT_MAX) return fail(TBSLA_ERR_INVALID_ARG, "rows + nnz exceeds the 32-bit index range");
  std::vector<int> rp((size_t)rows + 1);
  rp[0] = 0;
  for (int i = 0; i < rows; ++i) {
    if (rowptr[i + 1] < rowptr[i]) return fail(TBSLA_ERR_INVALID_ARG, "rowptr is not monotone at row %d", i);
    rp[i + 1] = rowptr[i + 1] - base;
  }
  int cmax = -1;
  for (int64_t k = 0; k < nnz; ++k) {
    const int c = colidx[k] - A->f_col;
    if (c < 0 || c >= A->n_col) return fail(TBSLA_ERR_INVALID_ARG, "colidx[%lld]=%d outside the column block", (long long)k, colidx[k]);
    cmax = std::max(cmax, c);
  }
  A->x_extent = cmax + 1;
  A->stored = nnz;
  TB_TRY(alloc_n(A, &A->idx0, (int64_t)rows + 1));
  TB_TRY(alloc_n(A, &A->idx1, nnz));
  TB_CUDA(cudaMemcpy(A->idx0, rp.data(), ((size_t)rows + 1) * sizeof(int), cudaMemcpyHostToDevice));
  if (nnz) TB_CUDA(cudaMemcpy(A->idx1, colidx, nnz * sizeof(int), cudaMemcpyHostToDevice));
  TB_TRY(upload_values(A, values, nnz, stores));
  return csr_bins(A, rp);
}

// The row bins of the direct kernels and the row blocks of variant 1 from the
// host copy of rowptr (base removed); idx0 / idx1 / values already on the device.
tbsla_status_t csr_bins(tbsla_matrix *A, const std::vector<int> &rp) {
  const int rows = A->rows;
  // direct bins: short rows by thread, long rows by warp, huge rows by chunk
  {
    std::vector<int> shorts;
    std::vector<int4> cls[kGroupClasses];
    std::vector<int2> chunk_rows;
    int slot = 0;
    bool all_short = true;
    int64_t short_nnz = 0;
    int short_max = 0;
    for (int r = 0; r < rows; ++r) {
      const int len = rp[r + 1] - rp[r];
      if (len <= kShortRow) {
        shorts.push_back(r);
        short_nnz += len;
        short_max = std::max(short_max, len);
        continue;
      }
      all_short = false;
      if (len <= kChunk) {
        int c = 0;
        while (len > kGroupLimit[c]) ++c;
        cls[c].push_back(make_int4(r, rp[r], rp[r + 1], -1));
        continue;
      }
      chunk_rows.push_back(make_int2(r, slot));
      for (int c = rp[r]; c < rp[r + 1]; c += kChunk)
        cls[kGroupClasses - 1].push_back(make_int4(r, c, std::min(c + kChunk, rp[r + 1]), slot++));
    }
    std::vector<int4> items;
    for (int c = 0; c < kGroupClasses; ++c) {
      A->item_class_start[c] = (int)items.size();
      items.insert(items.end(), cls[c].begin(), cls[c].end());
    }
    A->item_class_start[kGroupClasses] = (int)items.size();
    A->n_short = (int)shorts.size();
    A->short_nnz = short_nnz;
    A->short_max = short_max;
    // staged kernel (all rows short): entries of the largest 32-row tile,
    // rounded up to the 16-entry swizzle group
    A->stage_cap = 0;
    if (all_short && rows > 0) {
      int cap = 0;
      for (int r = 0; r < rows; r += 32) cap = std::max(cap, rp[std::min(r + 32, rows)] - rp[r]);
      A->stage_cap = std::max(16, (cap + 15) / 16 * 16);
    }
    // Rows of at most kTinyRow entries first, when they are a large part of
    // the short rows (power-law graphs: R-MAT 2^22 has 52 % empty rows and
    // 27 % of 1-4 entries); the order within each part is the rows' order.
    A->n_tiny = 0;
    if (!all_short && !shorts.empty()) {
      int64_t tiny = 0;
      for (int r : shorts) tiny += rp[r + 1] - rp[r] <= kTinyRow;
      if (tiny >= 1024 && 8 * tiny >= (int64_t)shorts.size()) {
        std::stable_partition(shorts.begin(), shorts.end(), [&](int r) { return rp[r + 1] - rp[r] <= kTinyRow; });
        A->n_tiny = (int)tiny;
      }
    }
    if (!all_short && !shorts.empty()) {
      TB_TRY(alloc_n(A, &A->short_rows, (int64_t)shorts.size()));
      TB_CUDA(cudaMemcpy(A->short_rows, shorts.data(), shorts.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    // the sliced copy (csr_sell_kernel): every row short, rows of at least 4
    // entries on average, at most 1/32 more slots than entries
    A->sell_width = 0;
    if (all_short && rows >= (1 << 16)) {
      int width = 0;
      for (int r = 0; r < rows; ++r) width = std::max(width, rp[r + 1] - rp[r]);
      const int64_t stride = ((int64_t)rows + kSellRows - 1) / kSellRows * kSellRows;
      const int64_t total = stride * width;
      const int64_t nnz = rp[rows];
      if (nnz >= 4ll * rows && total <= nnz + nnz / 32) {
        // best effort: without the device memory for it the handle keeps the
        // CSR arrays alone (the copy doubles the entries' memory)
        const size_t esz[3] = {4, 8, 4};  // columns, F64 and F32 values (BF16 products read the CSR arrays)
        void **bufs[3] = {(void **)&A->sell_cols, &A->sell_vals[0], &A->sell_vals[1]};
        bool ok = true;
        for (int k = 0; k < 3 && ok; ++k)
          if (k == 0 || A->values[k - 1]) ok = dev_alloc(A, bufs[k], (size_t)total * esz[k]) == TBSLA_OK;
        if (!ok) {
          for (int k = 0; k < 3; ++k)
            if (*bufs[k]) {
              cudaFree(*bufs[k]);
              *bufs[k] = nullptr;
              A->device_bytes -= total * (int64_t)esz[k] + 64;
            }
          g_err.clear();
        } else {
          const int *rpd = A->format == TBSLA_FMT_CSR ? A->idx0 : A->coo_rowptr;
          TB_CUDA(cudaMemset(A->sell_cols, 0xff, (size_t)total * sizeof(int)));  // padding: column -1
          for (int k = 0; k < 2; ++k)
            if (A->sell_vals[k]) TB_CUDA(cudaMemset(A->sell_vals[k], 0, (size_t)total * esz[k + 1]));
          sell_scatter_kernel<int><<<grid_for(rows, 256), 256>>>(rpd, stride, rows, A->idx1, A->sell_cols);
          A->sell_stride = stride;
          A->sell_width = width;
          TB_TRY(sell_refresh(A, 0));
        }
      }
    }
    A->n_warp_items = (int)items.size();
    if (!items.empty()) {
      TB_TRY(alloc_n(A, &A->warp_items, (int64_t)items.size()));
      TB_CUDA(cudaMemcpy(A->warp_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    }
    A->n_chunk_rows = (int)chunk_rows.size();
    chunk_rows.push_back(make_int2(-1, slot));
    TB_TRY(alloc_n(A, &A->chunk_rows, (int64_t)chunk_rows.size()));
    TB_CUDA(cudaMemcpy(A->chunk_rows, chunk_rows.data(), chunk_rows.size() * sizeof(int2), cudaMemcpyHostToDevice));
    TB_TRY(alloc_n(A, &A->chunk_partials, std::max(slot, 1)));
    TB_TRY(alloc_n(A, &A->chunk_partials32, std::max(slot, 1)));
  }
  std::vector<int4> blocks;
  std::vector<int2> huge;
  int n_partials = 0;
  plan_row_blocks(rp, blocks, huge, &n_partials);
  A->num_blocks = (int)blocks.size();
  A->num_huge = (int)huge.size() - 1;
  TB_TRY(alloc_n(A, &A->row_blocks, std::max<int64_t>((int64_t)blocks.size(), 1)));
  TB_TRY(alloc_n(A, &A->huge_rows, (int64_t)huge.size()));
  TB_TRY(alloc_n(A, &A->huge_partials, std::max(n_partials, 1)));
  TB_TRY(alloc_n(A, &A->huge_partials32, std::max(n_partials, 1)));
  if (!blocks.empty())
    TB_CUDA(cudaMemcpy(A->row_blocks, blocks.data(), blocks.size() * sizeof(int4), cudaMemcpyHostToDevice));
  TB_CUDA(cudaMemcpy(A->huge_rows, huge.data(), huge.size() * sizeof(int2), cudaMemcpyHostToDevice));
  TB_CUDA(cudaDeviceSynchronize());
  return TBSLA_OK;
}

}  // namespace tbsla

using namespace tbsla;

extern "C" {

const char *tbsla_last_error(void) { return g_err.c_str(); }

const char *tbsla_status_string(tbsla_status_t s) {
  switch (s) {
  case TBSLA_OK: return "ok";
  case TBSLA_ERR_INVALID_ARG: return "invalid argument";
  case TBSLA_ERR_CUDA: return "CUDA error";
  case TBSLA_ERR_OOM: return "out of device memory";
  case TBSLA_ERR_NOT_CONVERGED: return "not converged";
  case TBSLA_ERR_TIMEOUT: return "timeout";
  case TBSLA_ERR_UNSUPPORTED: return "unsupported";
  }
  return "unknown status";
}

int tbsla_version(void) { return 100; }

tbsla_status_t tbsla_set_l2_fetch_granularity(int bytes) {
  TB_CHECK(bytes == 32 || bytes == 64 || bytes == 128, "L2 fetch granularity %d not 32, 64 or 128", bytes);
  TB_CUDA(cudaSetDevice(current_device()));
  TB_CUDA(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)bytes));
  return TBSLA_OK;
}

tbsla_status_t tbsla_get_l2_fetch_granularity(int *bytes) {
  TB_CHECK(bytes, "bytes is NULL");
  TB_CUDA(cudaSetDevice(current_device()));
  size_t v = 0;
  TB_CUDA(cudaDeviceGetLimit(&v, cudaLimitMaxL2FetchGranularity));
  *bytes = (int)v;
  return TBSLA_OK;
}

tbsla_status_t tbsla_set_l2_persisting(size_t bytes) {
  TB_CUDA(cudaSetDevice(current_device()));
  TB_CUDA(cudaCtxResetPersistingL2Cache());
  TB_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, bytes));
  return TBSLA_OK;
}

tbsla_status_t tbsla_get_l2_persisting(size_t *bytes, size_t *max_bytes) {
  TB_CUDA(cudaSetDevice(current_device()));
  if (bytes) TB_CUDA(cudaDeviceGetLimit(bytes, cudaLimitPersistingL2CacheSize));
  if (max_bytes) {
    int v = 0;
    TB_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxPersistingL2CacheSize, current_device()));
    *max_bytes = (size_t)v;
  }
  return TBSLA_OK;
}

tbsla_status_t tbsla_set_device(int device) {
  int n = 0;
  TB_CUDA(cudaGetDeviceCount(&n));
  TB_CHECK(device >= 0 && device < n, "device %d out of range (%d devices)", device, n);
  g_device = device;
  TB_CUDA(cudaSetDevice(device));
  return TBSLA_OK;
}

tbsla_status_t tbsla_device_describe(int device, char *name, int name_len, double *hbm_gbs, int *sms) {
  int n = 0;
  TB_CUDA(cudaGetDeviceCount(&n));
  TB_CHECK(device >= 0 && device < n, "device %d out of range (%d devices)", device, n);
  cudaDeviceProp prop{};
  TB_CUDA(cudaGetDeviceProperties(&prop, device));
  if (name && name_len > 0) {
    std::snprintf(name, (size_t)name_len, "%s", prop.name);
  }
  if (hbm_gbs) {
    int khz = 0, bits = 0;
    TB_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrMemoryClockRate, device));
    TB_CUDA(cudaDeviceGetAttribute(&bits, cudaDevAttrGlobalMemoryBusWidth, device));
    *hbm_gbs = 2.0 * khz * 1e3 * (bits / 8.0) / 1e9;  // double data rate
  }
  if (sms) *sms = prop.multiProcessorCount;
  return TBSLA_OK;
}

tbsla_status_t tbsla_csr_create(int n_row, int n_col, int f_col, int rows, const int *rowptr,
                                const int *colidx, const double *values, int stores,
                                tbsla_matrix_t **out) {
  TB_CHECK(out, "out is NULL");
  *out = nullptr;
  TB_CHECK(n_row >= 0 && n_col >= 0 && rows >= 0 && f_col >= 0, "negative size");
  TB_CHECK(rows <= n_row || n_row == 0, "rows %d > n_row %d", rows, n_row);
  TB_CHECK(rowptr || rows == 0, "rowptr is NULL");
  tbsla_matrix *A = new_handle(TBSLA_FMT_CSR);
  if (!A) return fail(TBSLA_ERR_OOM, "host allocation failed");
  A->n_row = n_row; A->n_col = n_col; A->f_col = f_col; A->rows = std::min(rows, n_row);
  static const int zero = 0;
  const tbsla_status_t s = build_csr(A, rows ? rowptr : &zero, colidx, values, stores);
  if (s != TBSLA_OK) { free_handle(A); return s; }
  *out = A;
  return TBSLA_OK;
}

tbsla_status_t tbsla_ell_create(int n_row, int n_col, int f_col, int rows, int max_col,
                                const int *columns, const double *values, int stores,
                                tbsla_matrix_t **out) {
  TB_CHECK(out, "out is NULL");
  *out = nullptr;
  TB_CHECK(n_row >= 0 && n_col >= 0 && rows >= 0 && max_col >= 0 && f_col >= 0, "negative size");
  rows = std::min(rows, n_row);
  const int64_t slots = (int64_t)rows * max_col;
  TB_CHECK(slots == 0 || (columns && values), "NULL arrays");
  int cmax = slots > 0 ? 0 : -1;  // padding reads x[0]
  for (int64_t k = 0; k < slots; ++k) {
    int c = columns[k] - f_col;
    if (c < 0) c = 0;  // the reference's clamp (MatrixELL.cpp:108-109)
    if (c >= n_col)
      return fail(TBSLA_ERR_INVALID_ARG, "columns[%lld]=%d outside the column block", (long long)k, columns[k]);
    cmax = std::max(cmax, c);
  }
  tbsla_matrix *A = new_handle(TBSLA_FMT_ELL);
  if (!A) return fail(TBSLA_ERR_OOM, "host allocation failed");
  A->x_keep = 0.3f;  // ELL measured best at 0.2-0.4 (cqmat 2^24), CSR at 0.6
  A->n_row = n_row; A->n_col = n_col; A->f_col = f_col; A->rows = rows; A->max_col = max_col;
  A->rows_pad = (rows + 3) / 4 * 4;
  A->x_extent = cmax + 1;
  A->stored = slots;
  // transpose to slot-major with rows padded to a multiple of four
  const int64_t padded = (int64_t)A->rows_pad * max_col;
  std::vector<int> cm((size_t)std::max<int64_t>(padded, 1), f_col);
  std::vector<double> vm((size_t)std::max<int64_t>(padded, 1), 0.0);
  for (int i = 0; i < rows; ++i)
    for (int s = 0; s < max_col; ++s) {
      cm[(size_t)s * A->rows_pad + i] = columns[(int64_t)i * max_col + s];
      vm[(size_t)s * A->rows_pad + i] = values[(int64_t)i * max_col + s];
    }
  tbsla_status_t st = alloc_n(A, &A->idx0, padded);
  if (st == TBSLA_OK && padded)
    if (cudaMemcpy(A->idx0, cm.data(), padded * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
      st = fail(TBSLA_ERR_CUDA, "upload failed");
  if (st == TBSLA_OK) st = upload_values(A, vm.data(), padded, stores);
  if (st == TBSLA_OK && cudaDeviceSynchronize() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "sync failed");
  if (st != TBSLA_OK) { free_handle(A); return st; }
  *out = A;
  return TBSLA_OK;
}

tbsla_status_t tbsla_coo_create(int n_row, int n_col, int f_row, int f_col, int64_t nnz,
                                const int *row, const int *col, const double *values, int stores,
                                tbsla_matrix_t **out) {
  TB_CHECK(out, "out is NULL");
  *out = nullptr;
  TB_CHECK(n_row >= 0 && n_col >= 0 && nnz >= 0 && f_row >= 0 && f_col >= 0, "negative size");
  TB_CHECK(nnz == 0 || (row && col && values), "NULL arrays");
  TB_CHECK(nnz <= INT_MAX, "nnz %lld exceeds the 32-bit index range", (long long)nnz);
  // stable counting sort by row so that each row is a contiguous run in
  // input order
  std::vector<int64_t> cnt((size_t)n_row + 1, 0);
  int cmax = -1;
  for (int64_t k = 0; k < nnz; ++k) {
    const int r = row[k] - f_row, c = col[k] - f_col;
    if (r < 0 || r >= n_row) return fail(TBSLA_ERR_INVALID_ARG, "row[%lld]=%d outside the row block", (long long)k, row[k]);
    if (c < 0 || c >= n_col) return fail(TBSLA_ERR_INVALID_ARG, "col[%lld]=%d outside the column block", (long long)k, col[k]);
    cnt[r + 1]++;
    cmax = std::max(cmax, c);
  }
  for (int i = 0; i < n_row; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> sr((size_t)std::max<int64_t>(nnz, 1)), sc((size_t)std::max<int64_t>(nnz, 1));
  std::vector<double> sv((size_t)std::max<int64_t>(nnz, 1));
  for (int64_t k = 0; k < nnz; ++k) {
    const int64_t p = cnt[row[k] - f_row]++;
    sr[p] = row[k] - f_row;  // stored relative to f_row
    sc[p] = col[k];
    sv[p] = values[k];
  }
  tbsla_matrix *A = new_handle(f_row == 0 && f_col == 0 ? TBSLA_FMT_COO : TBSLA_FMT_SCOO);
  if (!A) return fail(TBSLA_ERR_OOM, "host allocation failed");
  A->n_row = n_row; A->n_col = n_col; A->f_row = f_row; A->f_col = f_col;
  A->rows = n_row; A->stored = nnz; A->x_extent = cmax + 1;
  A->num_tiles = (int)((nnz + kMergeTile - 1) / kMergeTile);
  tbsla_status_t st = alloc_n(A, &A->idx0, nnz);
  if (st == TBSLA_OK) st = alloc_n(A, &A->idx1, nnz);
  if (st == TBSLA_OK && nnz) {
    if (cudaMemcpy(A->idx0, sr.data(), nnz * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(A->idx1, sc.data(), nnz * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
      st = fail(TBSLA_ERR_CUDA, "upload failed");
  }
  if (st == TBSLA_OK) st = upload_values(A, sv.data(), nnz, stores);
  if (st == TBSLA_OK) st = alloc_carries(A);
  // the entries are row-sorted: a row pointer makes them CSR for the direct
  // kernels (cnt[r] is now the end of row r)
  if (st == TBSLA_OK && n_row > 0) {
    std::vector<int> rp((size_t)n_row + 1);
    rp[0] = 0;
    for (int r = 0; r < n_row; ++r) rp[(size_t)r + 1] = (int)cnt[(size_t)r];
    st = alloc_n(A, &A->coo_rowptr, (int64_t)n_row + 1);
    if (st == TBSLA_OK && cudaMemcpy(A->coo_rowptr, rp.data(), ((size_t)n_row + 1) * sizeof(int),
                                     cudaMemcpyHostToDevice) != cudaSuccess)
      st = fail(TBSLA_ERR_CUDA, "upload failed");
    if (st == TBSLA_OK) st = csr_bins(A, rp);
  }
  if (st == TBSLA_OK && cudaDeviceSynchronize() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "sync failed");
  if (st != TBSLA_OK) { free_handle(A); return st; }
  // COO rows are stored relative to f_row: output row = row + vect_incr
  A->f_row = 0;
  *out = A;
  return TBSLA_OK;
}

tbsla_status_t tbsla_dense_create(int n_row, int n_col, int ln_row, int ln_col,
                                  const double *values, int stores, tbsla_matrix_t **out) {
  TB_CHECK(out, "out is NULL");
  *out = nullptr;
  TB_CHECK(n_row >= 0 && n_col >= 0 && ln_row >= 0 && ln_col >= 0, "negative size");
  const int64_t n = (int64_t)ln_row * ln_col;
  TB_CHECK(n == 0 || values, "values is NULL");
  tbsla_matrix *A = new_handle(TBSLA_FMT_DENSE);
  if (!A) return fail(TBSLA_ERR_OOM, "host allocation failed");
  A->n_row = n_row; A->n_col = n_col; A->rows = std::min(ln_row, n_row); A->cols = ln_col;
  A->stored = n;
  A->x_extent = A->rows > 0 ? ln_col : 0;
  tbsla_status_t st = upload_values(A, values, n, stores);
  if (st == TBSLA_OK && cudaDeviceSynchronize() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "sync failed");
  if (st != TBSLA_OK) { free_handle(A); return st; }
  *out = A;
  return TBSLA_OK;
}

tbsla_status_t tbsla_matrix_set_variant(tbsla_matrix_t *A, int variant) {
  TB_CHECK(A, "matrix is NULL");
  if (A->format == TBSLA_FMT_CSR) {
    TB_CHECK(variant == 0 || variant == 1, "CSR kernel variant %d unknown (0 direct, 1 row blocks)", variant);
    A->csr_variant = variant;
    return TBSLA_OK;
  }
  if (A->format == TBSLA_FMT_COO || A->format == TBSLA_FMT_SCOO) {
    TB_CHECK(variant == 0 || variant == 1, "COO kernel variant %d unknown (0 direct, 1 merge path)", variant);
    A->csr_variant = variant;
    return TBSLA_OK;
  }
  if (A->format == TBSLA_FMT_ELL) {
    TB_CHECK(variant == 0 || variant == 1, "ELL kernel variant %d unknown (0 warp tiles, 1 four rows per thread)",
             variant);
    A->csr_variant = variant;
    return TBSLA_OK;
  }
  TB_CHECK(variant == 0, "format %d has a single kernel", A->format);
  return TBSLA_OK;
}

tbsla_status_t tbsla_matrix_tune(tbsla_matrix_t *A, int knob, double value) {
  TB_CHECK(A, "matrix is NULL");
  switch (knob) {
  case TBSLA_TUNE_X_L2_KEEP:
    TB_CHECK(value >= 0.0 && value <= 1.0, "x L2 keep fraction %g outside [0, 1]", value);
    A->x_keep = (float)value;
    if (A->pr_relabel) A->pr_relabel->x_keep = (float)value;
    return TBSLA_OK;
  case TBSLA_TUNE_PR_RELABEL:
    TB_CHECK(value == -1.0 || value == 0.0 || value == 1.0, "PageRank relabel mode %g not -1, 0 or 1", value);
    A->pr_relabel_mode = (int)value;
    return TBSLA_OK;
  case TBSLA_TUNE_SHORT_ROWS:
    TB_CHECK(value == -1.0 || value == 0.0 || value == 1.0 || value == 2.0 || value == 3.0,
             "short-row kernel mode %g not -1, 0, 1, 2 or 3", value);
    A->short_mode = (int)value;
    if (A->pr_relabel) A->pr_relabel->short_mode = (int)value;
    return TBSLA_OK;
  case TBSLA_TUNE_TC_SPLIT:
    TB_CHECK(value == 0.0 || value == 1.0 || value == 2.0 || value == 4.0 || value == 8.0 || value == 16.0,
             "tensor-core K split %g not 0, 1, 2, 4, 8 or 16", value);
    A->tc_split = (int)value;
    return TBSLA_OK;
  case TBSLA_TUNE_SELL_ROWS:
    TB_CHECK(value == 0.0 || value == 1.0 || value == 2.0 || value == 4.0,
             "rows per thread %g not 0, 1, 2 or 4", value);
    A->sell_rows = (int)value;
    return TBSLA_OK;
  case TBSLA_TUNE_DROP_SLICED_COPY:
    TB_CHECK(value == 1.0, "drop the sliced copy: value %g not 1", value);
    if (A->sell_width) {
      TB_CUDA(cudaSetDevice(A->device));
      TB_CUDA(cudaDeviceSynchronize());  // no product may still read it
      const int64_t slots = A->sell_stride * A->sell_width;
      const size_t esz[3] = {4, 8, 4};  // columns, F64, F32 values
      void *bufs[3] = {A->sell_cols, A->sell_vals[0], A->sell_vals[1]};
      for (int k = 0; k < 3; ++k)
        if (bufs[k]) {
          cudaFree(bufs[k]);
          A->device_bytes -= slots * (int64_t)esz[k] + 64;
        }
      A->sell_cols = nullptr;
      A->sell_vals[0] = A->sell_vals[1] = A->sell_vals[2] = nullptr;
      A->sell_width = 0;
      A->sell_stride = 0;
    }
    return TBSLA_OK;
  case TBSLA_TUNE_X_L2_RANGE:
    TB_CHECK(value == 0.0 || value == 1.0, "x L2 range mode %g not 0 or 1", value);
    A->x_keep_range = (int)value;
    if (A->pr_relabel) A->pr_relabel->x_keep_range = (int)value;
    if (A->transpose) A->transpose->x_keep_range = (int)value;
    return TBSLA_OK;
  default:
    return fail(TBSLA_ERR_INVALID_ARG, "unknown tuning knob %d", knob);
  }
}

tbsla_status_t tbsla_matrix_set_values(tbsla_matrix_t *A, tbsla_dtype_t type, const void *d_values, void *stream) {
  TB_CHECK(A, "matrix is NULL");
  TB_CHECK(A->format == TBSLA_FMT_CSR, "tbsla_matrix_set_values needs a CSR handle");
  TB_CHECK(A->values[0], "tbsla_matrix_set_values needs the F64 value store");
  TB_CHECK(A->stored == 0 || d_values, "values is NULL");
  TB_CHECK(type == TBSLA_F64 || type == TBSLA_F32, "type must be TBSLA_F64 or TBSLA_F32");
  TB_CUDA(cudaSetDevice(A->device));
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n = A->stored;
  if (n) {
    if (type == TBSLA_F64)
      TB_CUDA(cudaMemcpyAsync(A->values[0], d_values, (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
    else
      f32_to_f64_kernel<<<grid_for(n, 256), 256, 0, s>>>(static_cast<const float *>(d_values),
                                                         static_cast<double *>(A->values[0]), n);
  }
  TB_TRY(rederive_stores(A, s));
  TB_TRY(transpose_refresh(A, s));
  TB_CUDA(cudaStreamSynchronize(s));
  // PageRank state derived from the values: rebuilt on next use
  if (A->pr_work && A->pr_work_free) A->pr_work_free(A->pr_work);
  A->pr_work = nullptr;
  if (A->pr_relabel) free_handle(A->pr_relabel);
  A->pr_relabel = nullptr;
  if (A->pr_newid) cudaFree(A->pr_newid);
  A->pr_newid = nullptr;
  A->pr_newid_host.clear();
  A->pr_relabel_state = 0;
  return TBSLA_OK;
}

tbsla_status_t tbsla_matrix_destroy(tbsla_matrix_t *A) {
  free_handle(A);
  return TBSLA_OK;
}

tbsla_status_t tbsla_matrix_info(const tbsla_matrix_t *A, tbsla_matrix_info_t *info) {
  TB_CHECK(A && info, "NULL argument");
  info->format = A->format;
  info->n_row = A->n_row; info->n_col = A->n_col;
  info->f_row = A->f_row; info->f_col = A->f_col;
  info->rows = A->rows; info->max_col = A->max_col;
  info->stored = A->stored; info->stores = A->stores;
  info->device_bytes = A->device_bytes;
  int k = 0;
  switch (A->format) {
  case TBSLA_FMT_CSR:
    if (A->rows > 0 && A->stored > 0) {
      if (A->csr_variant == 0) {
        k = (A->n_short > 0) + (A->n_chunk_rows > 0);
        for (int c = 0; c < kGroupClasses; ++c) k += A->item_class_start[c + 1] > A->item_class_start[c];
      }
      else k = 1 + (A->num_huge > 0);
    }
    break;
  case TBSLA_FMT_COO:
  case TBSLA_FMT_SCOO:
    if (A->stored > 0 && A->coo_rowptr && A->csr_variant == 0) {
      k = (A->n_short > 0) + (A->n_chunk_rows > 0);
      for (int c = 0; c < kGroupClasses; ++c) k += A->item_class_start[c + 1] > A->item_class_start[c];
    } else {
      k = A->stored > 0 ? 2 : 0;
    }
    break;
  case TBSLA_FMT_ELL: k = (A->rows > 0 && A->max_col > 0) ? 1 : 0; break;
  default: k = (A->rows > 0 && A->cols > 0) ? 1 : 0; break;
  }
  info->kernels = k;
  info->slices = A->sell_width ? (int)(A->sell_stride / kSellRows) : 0;
  return TBSLA_OK;
}

tbsla_status_t tbsla_spmv(const tbsla_matrix_t *A, const double *d_x, double *d_y, int vect_incr,
                          void *stream) {
  TB_CHECK(A, "matrix is NULL");
  TB_CHECK(d_y || A->n_row == 0, "y is NULL");
  return spmv_dispatch(A, TBSLA_F64, TBSLA_F64, d_x, TBSLA_F64, d_y, vect_incr, (cudaStream_t)stream);
}

tbsla_status_t tbsla_spmv_ex(const tbsla_matrix_t *A, tbsla_dtype_t store, tbsla_dtype_t x_type,
                             const void *d_x, tbsla_dtype_t y_type, void *d_y, int vect_incr,
                             void *stream) {
  TB_CHECK(A, "matrix is NULL");
  return spmv_dispatch(A, store, x_type, d_x, y_type, d_y, vect_incr, (cudaStream_t)stream);
}

}  // extern "C"

namespace tbsla {
namespace {

// whether the device reads and writes pageable host memory coherently (the
// NVLink-C2C / address-translation path of Grace-Blackwell), per device
bool pageable_access(int dev) {
  static int cache[64];
  static std::once_flag once[64];
  if (dev < 0 || dev >= 64) return false;
  std::call_once(once[dev], [dev] {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    cache[dev] = v;
  });
  return cache[dev] != 0;
}

// The pointer a kernel uses for host memory p: the device alias of pinned
// memory, p itself for pageable memory the device reaches coherently,
// nullptr otherwise (or for memory that is not host memory).
void *device_alias(void *p, int dev) {
  if (!p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost) return a.devicePointer;
  if (a.type == cudaMemoryTypeUnregistered && pageable_access(dev)) return p;
  return nullptr;
}

// host -> device copy of n doubles by the SMs, for pageable sources the
// device reads coherently (the copy engines would stage them through a
// pinned bounce buffer)
__global__ void __launch_bounds__(256) host_read2_kernel(const double2 *__restrict__ src, double2 *__restrict__ dst,
                                                        int64_t n2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
__global__ void __launch_bounds__(256) host_read1_kernel(const double *__restrict__ src, double *__restrict__ dst,
                                                        int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

tbsla_status_t stage_x(tbsla_matrix *A, const double *x, int64_t nx) {
  if (!nx) return TBSLA_OK;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, x) != cudaSuccess) {
    cudaGetLastError();
    a.type = cudaMemoryTypeUnregistered;
  }
  if (a.type == cudaMemoryTypeUnregistered && pageable_access(A->device)) {
    const int grid = 152 * 4;
    if ((reinterpret_cast<uintptr_t>(x) & 15) == 0) {
      host_read2_kernel<<<grid, 256, 0, A->stream>>>(reinterpret_cast<const double2 *>(x),
                                                     reinterpret_cast<double2 *>(A->d_x), nx / 2);
      if (nx & 1) host_read1_kernel<<<1, 32, 0, A->stream>>>(x + nx - 1, A->d_x + nx - 1, 1);
    } else {
      host_read1_kernel<<<grid, 256, 0, A->stream>>>(x, A->d_x, nx);
    }
    TB_CUDA(cudaGetLastError());
    return TBSLA_OK;
  }
  TB_CUDA(cudaMemcpyAsync(A->d_x, x, nx * sizeof(double), cudaMemcpyHostToDevice, A->stream));
  return TBSLA_OK;
}

}  // namespace

// whether the product writes every row of y itself (zero_unwritten would
// leave y alone), so y may be written in place wherever it lives
bool writes_all_rows(const tbsla_matrix *A, int vect_incr) {
  if (A->n_row <= 0) return false;
  if (A->format == TBSLA_FMT_COO || A->format == TBSLA_FMT_SCOO)
    return A->coo_rowptr && A->csr_variant == 0 && vect_incr == 0 && A->stored > 0;
  if (A->format == TBSLA_FMT_ELL && A->max_col == 0) return false;
  if (A->format == TBSLA_FMT_DENSE && A->cols == 0) return false;
  if (A->format == TBSLA_FMT_CSR && A->stored == 0) return false;
  return A->rows >= A->n_row;
}

}  // namespace tbsla

extern "C" {

// Host vectors: x is staged into the handle's device buffer (a copy-engine
// copy from pinned memory, an SM copy from pageable memory the device reads
// coherently); when the product writes every row, y is written in place in
// host memory by the product itself (pinned or coherent pageable memory),
// so no device-to-host copy follows and y's traffic leaves HBM to the matrix.
tbsla_status_t tbsla_spmv_host(tbsla_matrix_t *A, const double *x, int64_t nx, double *y,
                               int64_t ny, int vect_incr) {
  TB_CHECK(A, "matrix is NULL");
  TB_CHECK(ny >= A->n_row, "y has %lld entries, n_row is %d", (long long)ny, A->n_row);
  TB_CHECK(nx >= A->x_extent, "x has %lld entries, the matrix reads %lld", (long long)nx, (long long)A->x_extent);
  TB_CHECK(nx == 0 || x, "x is NULL");
  std::lock_guard<std::mutex> lk(A->host_mu);
  TB_CUDA(cudaSetDevice(A->device));
  double *y_dev = writes_all_rows(A, vect_incr) ? static_cast<double *>(device_alias(y, A->device)) : nullptr;
  TB_TRY(ensure_host_buffers(A, std::max<int64_t>(nx, 1), y_dev ? 1 : std::max<int64_t>(ny, 1), 0));
  TB_TRY(stage_x(A, x, nx));
  TB_TRY(spmv_dispatch(A, TBSLA_F64, TBSLA_F64, A->d_x, TBSLA_F64, y_dev ? y_dev : A->d_y, vect_incr, A->stream));
  if (!y_dev && A->n_row)
    TB_CUDA(cudaMemcpyAsync(y, A->d_y, (size_t)A->n_row * sizeof(double), cudaMemcpyDeviceToHost, A->stream));
  TB_CUDA(cudaStreamSynchronize(A->stream));
  return TBSLA_OK;
}

tbsla_status_t tbsla_a_axpx(const tbsla_matrix_t *A, const double *d_x, double *d_r,
                            double *d_tmp, int vect_incr, void *stream) {
  TB_CHECK(A, "matrix is NULL");
  TB_CHECK(A->n_row == A->n_col, "a_axpx needs a square matrix (%d x %d)", A->n_row, A->n_col);
  TB_CHECK(d_tmp, "d_tmp is NULL (device pointer form needs caller scratch)");
  return a_axpx_dispatch(A, d_x, d_r, d_tmp, vect_incr, (cudaStream_t)stream);
}

tbsla_status_t tbsla_a_axpx_host(tbsla_matrix_t *A, const double *x, int64_t nx, double *r,
                                 int64_t nr, int vect_incr) {
  TB_CHECK(A, "matrix is NULL");
  TB_CHECK(A->n_row == A->n_col, "a_axpx needs a square matrix (%d x %d)", A->n_row, A->n_col);
  TB_CHECK(nx >= A->n_col && nr >= A->n_row && nx >= A->x_extent, "vector too short");
  std::lock_guard<std::mutex> lk(A->host_mu);
  TB_CUDA(cudaSetDevice(A->device));
  // r is written in place by the second product when it writes every row
  double *r_dev = writes_all_rows(A, vect_incr) ? static_cast<double *>(device_alias(r, A->device)) : nullptr;
  TB_TRY(ensure_host_buffers(A, std::max<int64_t>(nx, 1), r_dev ? 1 : std::max<int64_t>(nr, 1), std::max(A->n_row, 1)));
  TB_TRY(stage_x(A, x, nx));
  TB_TRY(a_axpx_dispatch(A, A->d_x, r_dev ? r_dev : A->d_y, A->d_t, vect_incr, A->stream));
  if (!r_dev && A->n_row)
    TB_CUDA(cudaMemcpyAsync(r, A->d_y, (size_t)A->n_row * sizeof(double), cudaMemcpyDeviceToHost, A->stream));
  TB_CUDA(cudaStreamSynchronize(A->stream));
  return TBSLA_OK;
}

tbsla_status_t tbsla_device_alloc(void **ptr, size_t bytes) {
  TB_CHECK(ptr, "ptr is NULL");
  return dev_alloc(nullptr, ptr, bytes);
}
tbsla_status_t tbsla_device_free(void *ptr) {
  if (ptr) TB_CUDA(cudaFree(ptr));
  return TBSLA_OK;
}
tbsla_status_t tbsla_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream) {
  if (bytes) TB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  return TBSLA_OK;
}
tbsla_status_t tbsla_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream) {
  if (bytes) TB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  return TBSLA_OK;
}
tbsla_status_t tbsla_stream_sync(void *stream) {
  TB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return TBSLA_OK;
}

tbsla_status_t tbsla_host_alloc(void **ptr, size_t bytes) {
  TB_CHECK(ptr, "ptr is NULL");
  *ptr = nullptr;
  TB_CUDA(cudaMallocHost(ptr, bytes ? bytes : 16));
  return TBSLA_OK;
}

tbsla_status_t tbsla_host_free(void *ptr) {
  if (ptr) TB_CUDA(cudaFreeHost(ptr));
  return TBSLA_OK;
}

tbsla_status_t tbsla_kernel_timing_enable(tbsla_matrix_t *A, int enable) {
  TB_CHECK(A, "matrix is NULL");
  A->timing = enable != 0;
  return TBSLA_OK;
}

tbsla_status_t tbsla_kernel_timing_read(tbsla_matrix_t *A, double *total_ms, int64_t *launches) {
  TB_CHECK(A, "matrix is NULL");
  for (auto &e : A->pending_events) {
    TB_CUDA(cudaEventSynchronize(e.second));
    float ms = 0;
    TB_CUDA(cudaEventElapsedTime(&ms, e.first, e.second));
    A->timed_ms += ms;
    A->timed_launches += 1;
    A->free_events.push_back(e);
  }
  A->pending_events.clear();
  if (total_ms) *total_ms = A->timed_ms;
  if (launches) *launches = A->timed_launches;
  A->timed_ms = 0;
  A->timed_launches = 0;
  return TBSLA_OK;
}

}  // extern "C"
