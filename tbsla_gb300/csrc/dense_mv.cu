// dense_mv.cu -- the multi-vector DENSE product Y = A X (k right-hand
// sides).  Unlike the one-vector GEMV (dense_kernel, bandwidth bound), k
// vectors make it a plain GEMM, so it is handed to cuBLAS: DGEMM for the
// FP64 store, SGEMM for F32, and for the BF16 store a BF16 x BF16 -> FP32
// GEMM on the tensor cores (X rounded to BF16 on the device first).  A is the
// handle's row-major ln_row x ln_col block, i.e. column-major A^T, hence the
// transposed operand.
#include <cublas_v2.h>

#include <map>
#include <mutex>

#include "common.cuh"

namespace {

std::mutex g_mu;
std::map<int, cublasHandle_t> g_handles;

tbsla_status_t handle_for(int device, cublasHandle_t *h) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_handles.find(device);
  if (it != g_handles.end()) {
    *h = it->second;
    return TBSLA_OK;
  }
  cublasHandle_t c = nullptr;
  if (cublasCreate(&c) != CUBLAS_STATUS_SUCCESS) return tbsla::fail(TBSLA_ERR_CUDA, "cublasCreate failed");
  g_handles[device] = c;
  *h = c;
  return TBSLA_OK;
}

__global__ void to_bf16_kernel(const float *__restrict__ x, int rows, int k, int64_t ldx, __nv_bfloat16 *out) {
  const int64_t total = (int64_t)rows * k;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / rows, r = t % rows;
    out[t] = __float2bfloat16_rn(x[c * ldx + r]);
  }
}

}  // namespace

using namespace tbsla;

extern "C" tbsla_status_t tbsla_dense_spmm(const tbsla_matrix_t *A, tbsla_dtype_t store, int k, const void *d_X,
                                           int64_t ldx, void *d_Y, int64_t ldy, void *stream) {
  TB_CHECK(A && A->format == TBSLA_FMT_DENSE, "tbsla_dense_spmm needs a DENSE handle");
  TB_CHECK(k >= 0 && d_X && d_Y, "bad argument");
  const int m = A->rows, n = A->cols;
  TB_CHECK(ldx >= n && ldy >= A->n_row, "leading dimensions too small (ldx %lld < %d or ldy %lld < %d)",
           (long long)ldx, n, (long long)ldy, A->n_row);
  const void *vals = A->values[store_index(store)];
  TB_CHECK(vals, "value store %d not present", (int)store);
  TB_CUDA(cudaSetDevice(A->device));
  cudaStream_t s = (cudaStream_t)stream;
  const size_t el = store == TBSLA_F64 ? 8 : 4;
  // rows past ln_row give 0 (the one-vector product's rule)
  if (A->n_row > m && k > 0)
    TB_CUDA(cudaMemset2DAsync(static_cast<char *>(d_Y) + (size_t)m * el, (size_t)ldy * el, 0,
                              (size_t)(A->n_row - m) * el, (size_t)k, s));
  if (m == 0 || k == 0) return TBSLA_OK;
  if (n == 0) {
    TB_CUDA(cudaMemset2DAsync(d_Y, (size_t)ldy * el, 0, (size_t)m * el, (size_t)k, s));
    return TBSLA_OK;
  }
  cublasHandle_t h = nullptr;
  TB_TRY(handle_for(A->device, &h));
  if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS) return fail(TBSLA_ERR_CUDA, "cublasSetStream failed");
  cublasStatus_t cs;
  if (store == TBSLA_F64) {
    const double one = 1.0, zero = 0.0;
    cs = cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, m, k, n, &one, static_cast<const double *>(vals), n,
                     static_cast<const double *>(d_X), (int)ldx, &zero, static_cast<double *>(d_Y), (int)ldy);
  } else if (store == TBSLA_F32) {
    const float one = 1.f, zero = 0.f;
    cs = cublasSgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, m, k, n, &one, static_cast<const float *>(vals), n,
                     static_cast<const float *>(d_X), (int)ldx, &zero, static_cast<float *>(d_Y), (int)ldy);
  } else {
    __nv_bfloat16 *xb = nullptr;
    TB_CUDA(cudaMallocAsync((void **)&xb, (size_t)n * k * sizeof(__nv_bfloat16), s));
    to_bf16_kernel<<<152 * 8, 256, 0, s>>>(static_cast<const float *>(d_X), n, k, ldx, xb);
    const float one = 1.f, zero = 0.f;
    cs = cublasGemmEx(h, CUBLAS_OP_T, CUBLAS_OP_N, m, k, n, &one, vals, CUDA_R_16BF, n, xb, CUDA_R_16BF, n, &zero,
                      d_Y, CUDA_R_32F, (int)ldy, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
    cudaFreeAsync(xb, s);
  }
  if (cs != CUBLAS_STATUS_SUCCESS) return fail(TBSLA_ERR_CUDA, "cuBLAS GEMM failed (status %d)", (int)cs);
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}
