// transpose.cu -- the CSR differentiation helpers: the transposed copy
// (A^T x), the gradient of y = A x with respect to the values (the outer
// product a b^T sampled on the sparsity pattern), and value replacement.
//
// The transposed copy is an ordinary CSR handle (so A^T x runs the same
// kernels as A x).  It is built once on the host: entries sorted by column,
// stably, so that row j of the copy lists column j's entries in increasing
// row order.  transpose_perm maps its entries back to A's, so new values of A
// reach the copy by a gather on the device.
#include <vector>

#include "product.cuh"

namespace tbsla {

tbsla_status_t spmv_dispatch(const tbsla_matrix *A, tbsla_dtype_t store, tbsla_dtype_t xt, const void *x,
                             tbsla_dtype_t yt, void *y, int vect_incr, cudaStream_t s);
tbsla_status_t rederive_stores(tbsla_matrix *A, cudaStream_t s);

namespace {

// out[k] = scale * a[row] * b[col - f_col] over the short rows (one thread each)
template <typename T>
__global__ void __launch_bounds__(256) grad_short_kernel(const int *__restrict__ rows, int n_rows,
                                                        const int *__restrict__ rowptr,
                                                        const int *__restrict__ colidx, int f_col,
                                                        const T *__restrict__ a, const T *__restrict__ b, T scale,
                                                        T *__restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n_rows; t += stride) {
    const int r = rows ? rows[t] : (int)t;
    const T ar = scale * a[r];
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) out[k] = ar * b[colidx[k] - f_col];
  }
}

// All rows short and consecutive (b, the gathered vector, read with the
// handle's L2 policy for x, TBSLA_TUNE_X_L2_KEEP): a warp takes 32 rows [r0, r0 + 32) and
// strides its lanes over the segment's entries, so index loads and gradient
// stores are coalesced; a lane finds the row of its entry by a binary search
// over the 32 row starts held one per lane (shuffles).  Four strides of the
// warp go together (128 entries: their index loads, then their gathers, in
// flight at once; eight measured the same).  The entry loop runs in whole warps (inactive lanes
// search too, then store nothing), as the full-mask shuffles require.
template <typename T>
__global__ void __launch_bounds__(256) grad_segment_kernel(int rows, const int *__restrict__ rowptr,
                                                          const int *__restrict__ colidx, int f_col,
                                                          const T *__restrict__ a, const T *__restrict__ b,
                                                          T scale, T *__restrict__ out, XKeep b_keep) {
  constexpr int U = 4;
  const int lane = threadIdx.x & 31;
  const uint64_t keep = policy_keep(b_keep, b);
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 32 < rows; w += nwarps) {
    const int r0 = (int)(w * 32);
    const int mine = min(r0 + lane, rows);
    const int start = __ldg(rowptr + mine);                    // row start of row r0 + lane
    const T ar = r0 + lane < rows ? scale * a[r0 + lane] : T(0);
    const int first = __shfl_sync(0xffffffffu, start, 0);
    const int end = __ldg(rowptr + min(r0 + 32, rows));
    for (int e0 = first; e0 < end; e0 += 32 * U) {
      int col[U];
      T bv[U];
      #pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = e0 + 32 * u + lane;
        col[u] = e < end ? ld_stream(colidx + e) : f_col;
      }
      #pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = e0 + 32 * u + lane;
        bv[u] = e < end ? ld_keep(b + (col[u] - f_col), keep) : T(0);
      }
      #pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = e0 + 32 * u + lane;
        int j = 0;  // largest lane index with start <= e
        #pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
          const int cand = j + step;
          const int v = __shfl_sync(0xffffffffu, start, cand & 31);
          if (cand < 32 && v <= e) j = cand;
        }
        const T arow = __shfl_sync(0xffffffffu, ar, j);
        if (e < end) __stcs(out + e, arow * bv[u]);
      }
    }
  }
}

// the same over the long-row items, L lanes per item
template <int L, typename T>
__global__ void __launch_bounds__(256) grad_group_kernel(const int4 *__restrict__ items, int n_items,
                                                        const int *__restrict__ colidx, int f_col,
                                                        const T *__restrict__ a, const T *__restrict__ b, T scale,
                                                        T *__restrict__ out) {
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / L;
  const int lane = threadIdx.x & (L - 1);
  for (int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / L; g < n_items; g += ng) {
    const int4 it = items[g];
    const T ar = scale * a[it.x];
    for (int k = it.y + lane; k < it.z; k += L) out[k] = ar * b[colidx[k] - f_col];
  }
}

// dst[k'] = src[perm[k']]
__global__ void permute_values_kernel(const double *__restrict__ src, const int *__restrict__ perm, int64_t n,
                                      double *__restrict__ dst) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    dst[k] = src[perm[k]];
}

bool csr_direct(const tbsla_matrix *A) { return A && A->format == TBSLA_FMT_CSR && A->csr_variant == 0; }

template <typename T>
tbsla_status_t grad_values(const tbsla_matrix *A, const T *a, const T *b, T scale, T *out, cudaStream_t s) {
  if (A->stored == 0 || A->rows == 0) return TBSLA_OK;
  if (A->short_rows == nullptr && A->n_short == A->rows) {  // every row short, in order
    const int warps = (A->rows + 31) / 32;
    grad_segment_kernel<T><<<(int)std::min<int64_t>(((int64_t)warps + 7) / 8, 152 * 64), 256, 0, s>>>(
        A->rows, A->idx0, A->idx1, A->f_col, a, b, scale, out, xkeep_of<T>(A));
    TB_CUDA(cudaGetLastError());
    return TBSLA_OK;
  }
  if (A->n_short > 0)
    grad_short_kernel<T><<<(int)(((int64_t)A->n_short + 255) / 256), 256, 0, s>>>(
        A->short_rows, A->n_short, A->idx0, A->idx1, A->f_col, a, b, scale, out);
  for (int c = 0; c < kGroupClasses; ++c) {
    const int first = A->item_class_start[c], count = A->item_class_start[c + 1] - first;
    if (count == 0) continue;
    const int grid = group_grid(count, kGroupLanes[c], false);
    const int4 *items = A->warp_items + first;
    switch (kGroupLanes[c]) {
    case 4: grad_group_kernel<4, T><<<grid, 256, 0, s>>>(items, count, A->idx1, A->f_col, a, b, scale, out); break;
    case 8: grad_group_kernel<8, T><<<grid, 256, 0, s>>>(items, count, A->idx1, A->f_col, a, b, scale, out); break;
    case 16: grad_group_kernel<16, T><<<grid, 256, 0, s>>>(items, count, A->idx1, A->f_col, a, b, scale, out); break;
    default: grad_group_kernel<32, T><<<grid, 256, 0, s>>>(items, count, A->idx1, A->f_col, a, b, scale, out); break;
    }
  }
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

}  // namespace

// The transposed copy of a CSR handle, built on first use.
tbsla_status_t ensure_transpose(tbsla_matrix *A, tbsla_matrix **T) {
  if (A->transpose) {
    *T = A->transpose;
    return TBSLA_OK;
  }
  TB_CHECK(A->format == TBSLA_FMT_CSR, "the transpose needs a CSR handle");
  TB_CHECK(A->values[0], "the transpose needs the F64 value store");
  TB_CUDA(cudaSetDevice(A->device));
  const int rows = A->rows, ncol = A->n_col;
  const int64_t nnz = A->stored;
  std::vector<int> rp((size_t)rows + 1), ci((size_t)std::max<int64_t>(nnz, 1));
  std::vector<double> va((size_t)std::max<int64_t>(nnz, 1));
  TB_TRY(tbsla_csr_download(A, rp.data(), ci.data(), va.data()));
  std::vector<int> tp((size_t)ncol + 1, 0);
  for (int64_t k = 0; k < nnz; ++k) ++tp[(size_t)(ci[(size_t)k] - A->f_col) + 1];
  for (int j = 0; j < ncol; ++j) tp[(size_t)j + 1] += tp[(size_t)j];
  std::vector<int> next(tp.begin(), tp.end() - 1), tci((size_t)std::max<int64_t>(nnz, 1)),
      perm((size_t)std::max<int64_t>(nnz, 1));
  std::vector<double> tva((size_t)std::max<int64_t>(nnz, 1));
  for (int i = 0; i < rows; ++i)
    for (int k = rp[(size_t)i]; k < rp[(size_t)i + 1]; ++k) {
      const int d = next[(size_t)(ci[(size_t)k] - A->f_col)]++;
      tci[(size_t)d] = i;
      tva[(size_t)d] = va[(size_t)k];
      perm[(size_t)d] = k;
    }
  tbsla_matrix_t *B = nullptr;
  TB_TRY(tbsla_csr_create(ncol, A->n_row, 0, ncol, tp.data(), tci.data(), tva.data(), A->stores, &B));
  B->x_keep = A->x_keep;
  B->x_keep_range = A->x_keep_range;
  B->short_mode = A->short_mode;
  int *d_perm = nullptr;
  if (cudaMalloc(&d_perm, (size_t)std::max<int64_t>(nnz, 1) * sizeof(int)) != cudaSuccess ||
      (nnz && cudaMemcpy(d_perm, perm.data(), (size_t)nnz * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)) {
    cudaGetLastError();
    if (d_perm) cudaFree(d_perm);
    tbsla_matrix_destroy(B);
    return fail(TBSLA_ERR_OOM, "transpose map (%lld ints)", (long long)nnz);
  }
  A->transpose = B;
  A->transpose_perm = d_perm;
  *T = B;
  return TBSLA_OK;
}

// After A's F64 values changed: the copy's values follow
tbsla_status_t transpose_refresh(tbsla_matrix *A, cudaStream_t s) {
  if (!A->transpose) return TBSLA_OK;
  tbsla_matrix *T = A->transpose;
  if (A->stored)
    permute_values_kernel<<<152 * 8, 256, 0, s>>>(static_cast<const double *>(A->values[0]), A->transpose_perm,
                                                 A->stored, static_cast<double *>(T->values[0]));
  TB_CUDA(cudaGetLastError());
  return rederive_stores(T, s);
}

tbsla_status_t grad_values_f64(const tbsla_matrix *A, const double *a, const double *b, double scale, double *out,
                               cudaStream_t s) {
  return grad_values<double>(A, a, b, scale, out, s);
}

}  // namespace tbsla

using namespace tbsla;

extern "C" {

tbsla_status_t tbsla_spmv_transpose_ex(const tbsla_matrix_t *A, tbsla_dtype_t store, tbsla_dtype_t x_type,
                                       const void *d_x, tbsla_dtype_t y_type, void *d_y, void *stream) {
  TB_CHECK(A, "matrix is NULL");
  TB_CHECK(A->format == TBSLA_FMT_CSR, "tbsla_spmv_transpose_ex needs a CSR handle");
  tbsla_matrix *T = nullptr;
  TB_TRY(ensure_transpose(const_cast<tbsla_matrix *>(A), &T));
  return spmv_dispatch(T, store, x_type, d_x, y_type, d_y, 0, (cudaStream_t)stream);
}

tbsla_status_t tbsla_csr_grad_values(const tbsla_matrix_t *A, tbsla_dtype_t type, const void *d_a, const void *d_b,
                                     double scale, void *d_out, void *stream) {
  TB_CHECK(A, "matrix is NULL");
  TB_CHECK(csr_direct(A), "tbsla_csr_grad_values needs a CSR handle (default kernel variant)");
  TB_CHECK(A->stored == 0 || (d_a && d_b && d_out), "NULL vector");
  TB_CUDA(cudaSetDevice(A->device));
  if (type == TBSLA_F64)
    return grad_values<double>(A, static_cast<const double *>(d_a), static_cast<const double *>(d_b), scale,
                               static_cast<double *>(d_out), (cudaStream_t)stream);
  TB_CHECK(type == TBSLA_F32, "type must be TBSLA_F64 or TBSLA_F32");
  return grad_values<float>(A, static_cast<const float *>(d_a), static_cast<const float *>(d_b), (float)scale,
                            static_cast<float *>(d_out), (cudaStream_t)stream);
}

}  // extern "C"

// ------------------------------------------------------- normalize_columns
// MatrixCSR::normalize_columns (src/cpp/matrix/MatrixCSR.cpp:423-435) on the
// device: column sums accumulated from 0 in the order of the reference's
// loop (rows ascending, then stored order) -- the transposed copy lists each
// column's entries in exactly that order, so one thread per column repeats
// the reference's additions -- then every value divided by its column's sum
// (IEEE division, as the host's).  The values then go through
// tbsla_matrix_set_values, which refreshes every derived copy.
namespace tbsla {
namespace {

__global__ void colsum_kernel(const int *__restrict__ tp, const double *__restrict__ tv, int ncol,
                              double *__restrict__ sum) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ncol; j += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = tp[j]; k < tp[j + 1]; ++k) s += tv[k];
    sum[j] = s;
  }
}

__global__ void divide_kernel(const double *__restrict__ v, const int *__restrict__ ci, int f_col, int64_t n,
                              const double *__restrict__ sum, double *__restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    out[k] = v[k] / sum[ci[k] - f_col];
}

}  // namespace
}  // namespace tbsla

extern "C" tbsla_status_t tbsla_csr_normalize_columns(tbsla_matrix_t *A, void *stream) {
  TB_CHECK(A, "matrix is NULL");
  TB_CHECK(A->format == TBSLA_FMT_CSR, "tbsla_csr_normalize_columns needs a CSR handle");
  TB_CHECK(A->values[0], "the F64 value store is needed");
  TB_CUDA(cudaSetDevice(A->device));
  if (A->stored == 0) return TBSLA_OK;
  tbsla_matrix *T = nullptr;
  TB_TRY(ensure_transpose(A, &T));
  cudaStream_t s = (cudaStream_t)stream;
  double *sum = nullptr, *out = nullptr;
  const int ncol = std::max(A->n_col, 1);
  if (cudaMalloc(&sum, (size_t)ncol * 8) != cudaSuccess || cudaMalloc(&out, (size_t)A->stored * 8) != cudaSuccess) {
    cudaGetLastError();
    if (sum) cudaFree(sum);
    return fail(TBSLA_ERR_OOM, "normalize_columns scratch");
  }
  tbsla_status_t st = TBSLA_OK;
  colsum_kernel<<<std::max(1, std::min((T->rows + 255) / 256, 152 * 16)), 256, 0, s>>>(
      T->idx0, static_cast<const double *>(T->values[0]), T->rows, sum);
  divide_kernel<<<152 * 8, 256, 0, s>>>(static_cast<const double *>(A->values[0]), A->idx1, A->f_col, A->stored, sum,
                                       out);
  if (cudaGetLastError() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "normalize_columns kernels failed");
  if (st == TBSLA_OK) st = tbsla_matrix_set_values(A, TBSLA_F64, out, stream);
  cudaStreamSynchronize(s);
  cudaFree(sum);
  cudaFree(out);
  return st;
}
