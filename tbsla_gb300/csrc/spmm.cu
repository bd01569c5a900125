// spmm.cu -- Y = A X for k vectors of a CSR (or row-sorted COO / SCOO) handle.
//
// X and Y are row-major blocks (vector index fastest): X[j * ldx + c] is
// entry j of vector c.  The vectors go in panels of at most 32; a group of
// KT lanes takes a row, each lane VW consecutive vectors (16-byte loads of a
// gathered X row when the panel and ldx allow it, else one vector per lane),
// and sums each of its vectors over the row in stored order, one FMA per
// entry -- the
// one-thread-per-row product's arithmetic, so for rows of at most 32 entries
// each column of Y equals tbsla_spmv_ex of that vector bit for bit
// (TBSLA_TUNE_SHORT_ROWS = 0); longer rows, which the one-vector kernels
// split among lanes, agree to rounding.  The
// lanes of a group read one row's index and value together (one load each,
// broadcast) and the KT values of a gathered X row are contiguous, so one
// gather serves the whole panel.  The matrix is streamed once per panel.
// Rows the kernels never visit (past A->rows) are set to 0, as the one-vector
// product leaves them.
#include "product.cuh"

namespace tbsla {
namespace {

// VW consecutive vectors per lane (16-byte loads of X when VW > 1)
template <typename T, int VW> struct VecOf;
template <> struct VecOf<double, 1> { using type = double; };
template <> struct VecOf<float, 1> { using type = float; };
template <> struct VecOf<double, 2> { using type = double2; };
template <> struct VecOf<float, 4> { using type = float4; };
__device__ __forceinline__ void unpack(double v, double (&o)[1]) { o[0] = v; }
__device__ __forceinline__ void unpack(float v, float (&o)[1]) { o[0] = v; }
__device__ __forceinline__ void unpack(double2 v, double (&o)[2]) { o[0] = v.x; o[1] = v.y; }
__device__ __forceinline__ void unpack(float4 v, float (&o)[4]) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }

template <typename V, typename T, int KT, int VW>
__global__ void __launch_bounds__(256) csr_spmm_kernel(int rows, const int *__restrict__ rowptr,
                                                      const int *__restrict__ colidx, const V *__restrict__ values,
                                                      const T *__restrict__ X, int64_t ldx, int f_col,
                                                      T *__restrict__ Y, int64_t ldy, int width, int row_shift,
                                                      int n_out) {
  using Acc = typename AccOf<T>::type;
  using Vec = typename VecOf<T, VW>::type;
  const int lane = threadIdx.x & (KT - 1);
  const int c = lane * VW;  // first vector of this lane
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / KT;
  for (int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / KT; g < rows; g += ng) {
    const int r = (int)g;
    const int a = __ldg(rowptr + r), b = __ldg(rowptr + r + 1);
    if (c < width) {
      Acc acc[VW];
      #pragma unroll
      for (int q = 0; q < VW; ++q) acc[q] = 0;
      #pragma unroll 4
      for (int e = a; e < b; ++e) {
        const Acc v = to_acc(ld_stream(values + e), Acc());
        T xv[VW];
        unpack(__ldg(reinterpret_cast<const Vec *>(X + (int64_t)(__ldg(colidx + e) - f_col) * ldx + c)), xv);
        #pragma unroll
        for (int q = 0; q < VW; ++q) acc[q] = fma_acc(v, to_acc(xv[q], Acc()), acc[q]);
      }
      const int out = r + row_shift;
      if (out >= 0 && out < n_out) {
        #pragma unroll
        for (int q = 0; q < VW; ++q)
          if (c + q < width) Y[(int64_t)out * ldy + c + q] = (T)acc[q];
      }
    }
  }
}

// FP32 panels of handles with the ELL-layout copy (csr_sell_kernel's
// arrays): one thread per row, all 4 KW vectors of the panel; for each slot
// the warp's 32 rows load their indices and values as one 128-byte run each,
// and the gathered X rows of neighbouring rows' band entries are neighbouring
// rows of X.  Each vector's sum is one FMA per entry in stored order, as in
// csr_spmm_kernel: the same bits.
template <int KW>
__global__ void __launch_bounds__(256) sell_spmm_kernel(const int *__restrict__ cols, const float *__restrict__ vals,
                                                       int64_t stride, int width, int rows,
                                                       const float *__restrict__ X, int64_t ldx, int f_col,
                                                       float *__restrict__ Y, int64_t ldy, int row_shift, int n_out) {
  constexpr int U = KW <= 2 ? 4 : 2;  // slots in flight
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  float acc[4 * KW];
  #pragma unroll
  for (int q = 0; q < 4 * KW; ++q) acc[q] = 0.f;
  for (int j0 = 0; j0 < width; j0 += U) {
    int c[U];
    float v[U];
    #pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool in = j0 + u < width;
      c[u] = in ? ld_ell<false>(cols + (size_t)(j0 + u) * stride + r) : -1;
      v[u] = in ? ld_ell<false>(vals + (size_t)(j0 + u) * stride + r) : 0.f;
    }
    #pragma unroll
    for (int u = 0; u < U; ++u) {
      if (c[u] < 0) continue;  // padding (past the row's end)
      const float4 *xp = reinterpret_cast<const float4 *>(X + (int64_t)(c[u] - f_col) * ldx);
      #pragma unroll
      for (int q = 0; q < KW; ++q) {
        const float4 x4 = __ldg(xp + q);
        acc[4 * q + 0] = fmaf(v[u], x4.x, acc[4 * q + 0]);
        acc[4 * q + 1] = fmaf(v[u], x4.y, acc[4 * q + 1]);
        acc[4 * q + 2] = fmaf(v[u], x4.z, acc[4 * q + 2]);
        acc[4 * q + 3] = fmaf(v[u], x4.w, acc[4 * q + 3]);
      }
    }
  }
  const int out = r + row_shift;
  if (out >= 0 && out < n_out) {
    float4 *yp = reinterpret_cast<float4 *>(Y + (int64_t)out * ldy);
    #pragma unroll
    for (int q = 0; q < KW; ++q) yp[q] = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
  }
}

template <typename V, typename T>
tbsla_status_t spmm_panel(const tbsla_matrix *A, const int *rowptr, const V *vals, const T *X, int64_t ldx, T *Y,
                          int64_t ldy, int width, int row_shift, cudaStream_t s) {
  const int rows = A->rows;
  if (rows <= 0) return TBSLA_OK;
  if constexpr (std::is_same<V, float>::value && std::is_same<T, float>::value) {
    // the ELL-layout copy (default short-row mode, or 3), when the panel is
    // whole float4 runs on both sides and at most 12 wide (cqmat 2^22, ms
    // copy / CSR arrays: k = 4 0.146 / 0.339, 8 0.235 / 0.377, 12 0.325 /
    // 0.445, 16 0.598 / 0.458, 32 1.912 / 0.669: a thread's 4 k
    // accumulators and gathers crowd out the loads in flight above 12)
    if (A->sell_width && A->sell_vals[1] && vals == A->values[1] && (A->short_mode == -1 || A->short_mode == 3) &&
        width % 4 == 0 && width <= 12 && ldx % 4 == 0 && ldy % 4 == 0 &&
        (reinterpret_cast<uintptr_t>(X) & 15) == 0 && (reinterpret_cast<uintptr_t>(Y) & 15) == 0) {
      const float *sv = static_cast<const float *>(A->sell_vals[1]);
      const int grid = (rows + 255) / 256;
#define TB_SELL_SPMM(KW_)                                                                                          \
  sell_spmm_kernel<KW_><<<grid, 256, 0, s>>>(A->sell_cols, sv, A->sell_stride, A->sell_width, rows, X, ldx, A->f_col, \
                                             Y, ldy, row_shift, A->n_row)
      switch (width / 4) {
      case 1: TB_SELL_SPMM(1); break;
      case 2: TB_SELL_SPMM(2); break;
      default: TB_SELL_SPMM(3); break;
      }
#undef TB_SELL_SPMM
      TB_CUDA(cudaGetLastError());
      return TBSLA_OK;
    }
  }
  // 16-byte loads of X rows when the panel is whole 16-byte chunks, aligned
  constexpr int VW16 = 16 / (int)sizeof(T);
  const bool vec = width % VW16 == 0 && (ldx * (int64_t)sizeof(T)) % 16 == 0 &&
                   (reinterpret_cast<uintptr_t>(X) & 15) == 0;
  const int lanes = vec ? width / VW16 : width;
  const int kt = lanes <= 1 ? 1 : lanes <= 2 ? 2 : lanes <= 4 ? 4 : lanes <= 8 ? 8 : lanes <= 16 ? 16 : 32;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)rows * kt + 255) / 256, 152 * 64));
#define TB_SPMM(KT_, VW_)                                                                                          \
  csr_spmm_kernel<V, T, KT_, VW_><<<grid, 256, 0, s>>>(rows, rowptr, A->idx1, vals, X, ldx, A->f_col, Y, ldy, width, \
                                                      row_shift, A->n_row)
  if (vec) {
    switch (kt) {
    case 1: TB_SPMM(1, VW16); break;
    case 2: TB_SPMM(2, VW16); break;
    case 4: TB_SPMM(4, VW16); break;
    case 8: TB_SPMM(8, VW16); break;
    default: TB_SPMM(16, VW16); break;
    }
  } else {
    switch (kt) {
    case 1: TB_SPMM(1, 1); break;
    case 2: TB_SPMM(2, 1); break;
    case 4: TB_SPMM(4, 1); break;
    case 8: TB_SPMM(8, 1); break;
    case 16: TB_SPMM(16, 1); break;
    default: TB_SPMM(32, 1); break;
    }
  }
#undef TB_SPMM
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

template <typename V, typename T>
tbsla_status_t spmm_typed(const tbsla_matrix *A, const int *rowptr, const V *vals, int k, const T *X, int64_t ldx,
                          T *Y, int64_t ldy, int row_shift, cudaStream_t s) {
  for (int c0 = 0; c0 < k; c0 += 32)
    TB_TRY(spmm_panel<V, T>(A, rowptr, vals, X + c0, ldx, Y + c0, ldy, std::min(32, k - c0), row_shift, s));
  return TBSLA_OK;
}

}  // namespace
}  // namespace tbsla

using namespace tbsla;

extern "C" tbsla_status_t tbsla_spmm(const tbsla_matrix_t *A, tbsla_dtype_t store, int k, const void *d_X,
                                     int64_t ldx, void *d_Y, int64_t ldy, void *stream) {
  TB_CHECK(A, "matrix is NULL");
  const bool coo = A->format == TBSLA_FMT_COO || A->format == TBSLA_FMT_SCOO;
  TB_CHECK(A->format == TBSLA_FMT_CSR || (coo && A->coo_rowptr),
           "tbsla_spmm needs a CSR or COO / SCOO handle (DENSE: tbsla_dense_spmm)");
  TB_CHECK(k >= 0, "k = %d", k);
  TB_CHECK(k == 0 || (d_X && d_Y), "NULL block");
  TB_CHECK(ldx >= k && ldy >= k, "leading dimensions (%lld, %lld) below k = %d", (long long)ldx, (long long)ldy, k);
  TB_CHECK(store == TBSLA_F64 || store == TBSLA_F32 || store == TBSLA_BF16, "bad store");
  const void *vals = A->values[store_index(store)];
  TB_CHECK(vals || A->stored == 0, "value store %d not present", (int)store);
  TB_CUDA(cudaSetDevice(A->device));
  cudaStream_t s = (cudaStream_t)stream;
  if (k == 0 || A->n_row == 0) return TBSLA_OK;
  const size_t el = store == TBSLA_F64 ? 8 : 4;
  // rows no kernel writes are 0: rows past A->rows, or all of them when the
  // matrix stores nothing
  const int written = A->stored > 0 ? std::min(A->rows, A->n_row) : 0;
  if (written < A->n_row)
    TB_CUDA(cudaMemset2DAsync(static_cast<char *>(d_Y) + (size_t)written * ldy * el, (size_t)ldy * el, 0,
                              (size_t)k * el, (size_t)(A->n_row - written), s));
  if (written == 0) return TBSLA_OK;
  const int *rowptr = coo ? A->coo_rowptr : A->idx0;
  if (store == TBSLA_F64)
    return spmm_typed<double, double>(A, rowptr, static_cast<const double *>(vals), k,
                                      static_cast<const double *>(d_X), ldx, static_cast<double *>(d_Y), ldy, 0, s);
  if (store == TBSLA_F32)
    return spmm_typed<float, float>(A, rowptr, static_cast<const float *>(vals), k, static_cast<const float *>(d_X),
                                    ldx, static_cast<float *>(d_Y), ldy, 0, s);
  return spmm_typed<__nv_bfloat16, float>(A, rowptr, static_cast<const __nv_bfloat16 *>(vals), k,
                                          static_cast<const float *>(d_X), ldx, static_cast<float *>(d_Y), ldy, 0, s);
}
