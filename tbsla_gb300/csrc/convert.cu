// convert.cu -- COO / SCOO handle -> CSR handle on the device: the
// conversion of MatrixCSR(const MatrixCOO&) (src/cpp/matrix/MatrixCSR.cpp:
// 29-74) without the host.  Entries are ordered by (row, column); the COO
// handle already holds them stably row-sorted, and the radix sort used here
// is stable, so equal (row, column) pairs keep their input order -- the
// arrays equal the host conversion's bit for bit.  The sort is CUB's
// DeviceRadixSort (a preprocessing step, not the product); rowptr is a row
// histogram and a scan.  Only rowptr travels to the host, for the row bins of
// the direct kernels.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <vector>

#include "common.cuh"

namespace tbsla {

tbsla_matrix *new_matrix(int format);
void free_matrix(tbsla_matrix *A);
tbsla_status_t alloc_ints(tbsla_matrix *A, int **p, int64_t n);
tbsla_status_t store_values_device(tbsla_matrix *A, const double *d_src, int64_t n, int stores, cudaStream_t s);
tbsla_status_t csr_bins(tbsla_matrix *A, const std::vector<int> &rp);

namespace {

// key = row * span + (col - f_col), index = entry position
__global__ void keys_kernel(const int *__restrict__ row, const int *__restrict__ col, int f_col, uint64_t span,
                            int64_t n, uint64_t *__restrict__ keys, int *__restrict__ idx) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    keys[k] = (uint64_t)row[k] * span + (uint64_t)(col[k] - f_col);
    idx[k] = (int)k;
  }
}

// counts[row + 1] += 1
__global__ void rows_kernel(const int *__restrict__ row, int64_t n, int *counts) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(counts + row[k] + 1, 1);
}

// the entries in sorted order
__global__ void gather_kernel(const int *__restrict__ order, const int *__restrict__ col,
                              const double *__restrict__ val, int64_t n, int *__restrict__ out_col,
                              double *__restrict__ out_val) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int p = order[k];
    out_col[k] = col[p];
    out_val[k] = val[p];
  }
}

int bit_width(uint64_t v) {
  int b = 0;
  while (v) { ++b; v >>= 1; }
  return b;
}

}  // namespace
}  // namespace tbsla

using namespace tbsla;

extern "C" tbsla_status_t tbsla_coo_to_csr(const tbsla_matrix_t *C, int stores, tbsla_matrix_t **out) {
  TB_CHECK(C && out, "NULL argument");
  *out = nullptr;
  TB_CHECK(C->format == TBSLA_FMT_COO || C->format == TBSLA_FMT_SCOO, "tbsla_coo_to_csr needs a COO / SCOO handle");
  TB_CHECK(C->values[0], "the conversion needs the F64 value store");
  TB_CUDA(cudaSetDevice(C->device));
  const int64_t n = C->stored;
  const int rows = C->n_row;
  const uint64_t span = (uint64_t)std::max<int64_t>(C->x_extent, 1);
  const int end_bit = std::max(1, bit_width((uint64_t)std::max(rows, 1) * span));
  tbsla_matrix *A = new_matrix(TBSLA_FMT_CSR);
  if (!A) return fail(TBSLA_ERR_OOM, "host allocation failed");
  A->n_row = C->n_row;
  A->n_col = C->n_col;
  A->f_col = C->f_col;
  A->rows = rows;
  A->stored = n;
  A->x_extent = C->x_extent;
  cudaStream_t s = nullptr;
  uint64_t *keys = nullptr, *keys2 = nullptr;
  int *idx = nullptr, *idx2 = nullptr, *counts = nullptr;
  double *vtmp = nullptr;
  void *tmp = nullptr;
  std::vector<void *> scratch;
  tbsla_status_t st = TBSLA_OK;
  auto alloc = [&](void **p, size_t b) {
    if (st != TBSLA_OK) return;
    if (cudaMalloc(p, std::max<size_t>(b, 16)) != cudaSuccess) {
      cudaGetLastError();
      st = fail(TBSLA_ERR_OOM, "conversion scratch (%zu bytes)", b);
      return;
    }
    scratch.push_back(*p);
  };
  alloc((void **)&keys, (size_t)n * 8);
  alloc((void **)&keys2, (size_t)n * 8);
  alloc((void **)&idx, (size_t)n * 4);
  alloc((void **)&idx2, (size_t)n * 4);
  alloc((void **)&counts, ((size_t)rows + 1) * 4);
  alloc((void **)&vtmp, (size_t)n * 8);
  if (st == TBSLA_OK) st = alloc_ints(A, &A->idx0, (int64_t)rows + 1);
  if (st == TBSLA_OK) st = alloc_ints(A, &A->idx1, n);
  size_t sort_bytes = 0, scan_bytes = 0;
  if (st == TBSLA_OK &&
      (cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, keys, keys2, idx, idx2, n, 0, end_bit, s) != cudaSuccess ||
       cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, counts, A->idx0, rows + 1, s) != cudaSuccess))
    st = fail(TBSLA_ERR_CUDA, "sort / scan sizing failed");
  alloc(&tmp, std::max(sort_bytes, scan_bytes));
  const int g = 152 * 8;
  if (st == TBSLA_OK && n > 0) {
    keys_kernel<<<g, 256, 0, s>>>(C->idx0, C->idx1, C->f_col, span, n, keys, idx);
    if (cub::DeviceRadixSort::SortPairs(tmp, sort_bytes, keys, keys2, idx, idx2, n, 0, end_bit, s) != cudaSuccess)
      st = fail(TBSLA_ERR_CUDA, "radix sort failed");
    if (st == TBSLA_OK)
      gather_kernel<<<g, 256, 0, s>>>(idx2, C->idx1, static_cast<const double *>(C->values[0]), n, A->idx1, vtmp);
  }
  if (st == TBSLA_OK) {
    cudaMemsetAsync(counts, 0, ((size_t)rows + 1) * 4, s);
    if (n > 0) rows_kernel<<<g, 256, 0, s>>>(C->idx0, n, counts);
    if (cub::DeviceScan::InclusiveSum(tmp, scan_bytes, counts, A->idx0, rows + 1, s) != cudaSuccess)
      st = fail(TBSLA_ERR_CUDA, "scan failed");
  }
  if (st == TBSLA_OK && cudaGetLastError() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "conversion kernels failed");
  if (st == TBSLA_OK) st = store_values_device(A, vtmp, n, stores, s);
  std::vector<int> rp((size_t)rows + 1);
  if (st == TBSLA_OK &&
      cudaMemcpy(rp.data(), A->idx0, ((size_t)rows + 1) * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    st = fail(TBSLA_ERR_CUDA, "rowptr download failed");
  if (st == TBSLA_OK) st = csr_bins(A, rp);
  cudaDeviceSynchronize();
  for (void *p : scratch) cudaFree(p);
  if (st != TBSLA_OK) {
    free_matrix(A);
    return st;
  }
  *out = A;
  return TBSLA_OK;
}
