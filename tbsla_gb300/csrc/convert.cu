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
tbsla_status_t alloc_carries(tbsla_matrix *A);

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

// ------------------------------------------------------------------ ELL / DENSE
// MatrixELL(const MatrixCOO&) (src/cpp/matrix/MatrixELL.cpp:12-53) and
// MatrixDENSE(const MatrixCOO&) (src/cpp/matrix/MatrixDENSE.cpp:11-28) on the
// device, through the (row, column)-sorted CSR arrays of tbsla_coo_to_csr:
// ELL row i holds its entries in that order in slots 0..len-1, padding slots
// column 0 and value 0 (rows padded to a multiple of four: column f_col, as
// tbsla_ell_create pads them); DENSE adds the entries of a (row, column) pair
// to 0 in input order, as the reference's += loop does.  The results equal
// tbsla_ell_create / tbsla_dense_create on the host conversion's arrays.
namespace tbsla {
namespace {

// slot-major ELL arrays from sorted CSR arrays (one thread per padded row)
__global__ void ell_fill_kernel(const int *__restrict__ rp, const int *__restrict__ ci,
                                const double *__restrict__ va, int rows, int rows_pad, int max_col, int f_col,
                                int *__restrict__ cols, double *__restrict__ vals) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows_pad; i += gridDim.x * blockDim.x) {
    const int a = i < rows ? rp[i] : 0, len = i < rows ? rp[i + 1] - a : 0;
    for (int s = 0; s < max_col; ++s) {
      const size_t o = (size_t)s * rows_pad + i;
      cols[o] = s < len ? ci[a + s] : (i < rows ? 0 : f_col);
      vals[o] = s < len ? va[a + s] : 0.0;
    }
  }
}

// dense rows from sorted CSR arrays: runs of one column summed from 0 in order
__global__ void dense_fill_kernel(const int *__restrict__ rp, const int *__restrict__ ci,
                                  const double *__restrict__ va, int rows, int ld, double *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
    const int b = rp[i + 1];
    for (int k = rp[i]; k < b;) {
      const int c = ci[k];
      double acc = 0.0;
      for (; k < b && ci[k] == c; ++k) acc += va[k];
      out[(size_t)i * ld + c] = acc;
    }
  }
}

}  // namespace
}  // namespace tbsla

extern "C" tbsla_status_t tbsla_coo_to_ell(const tbsla_matrix_t *C, int stores, tbsla_matrix_t **out) {
  TB_CHECK(C && out, "NULL argument");
  *out = nullptr;
  TB_CHECK(C->format == TBSLA_FMT_COO || C->format == TBSLA_FMT_SCOO, "tbsla_coo_to_ell needs a COO / SCOO handle");
  tbsla_matrix_t *R = nullptr;
  TB_TRY(tbsla_coo_to_csr(C, TBSLA_STORE_F64, &R));
  struct Drop {
    tbsla_matrix_t *R;
    ~Drop() { free_matrix(R); }
  } drop{R};
  const int rows = R->rows;
  std::vector<int> rp((size_t)rows + 1);
  TB_CUDA(cudaMemcpy(rp.data(), R->idx0, rp.size() * sizeof(int), cudaMemcpyDeviceToHost));
  int max_col = 0;
  for (int i = 0; i < rows; ++i) max_col = std::max(max_col, rp[(size_t)i + 1] - rp[(size_t)i]);
  tbsla_matrix *E = new_matrix(TBSLA_FMT_ELL);
  if (!E) return fail(TBSLA_ERR_OOM, "host allocation failed");
  E->x_keep = 0.3f;
  E->n_row = C->n_row; E->n_col = C->n_col; E->f_col = C->f_col;
  E->rows = rows; E->max_col = max_col; E->rows_pad = (rows + 3) / 4 * 4;
  const int64_t slots = (int64_t)rows * max_col, padded = (int64_t)E->rows_pad * max_col;
  E->stored = slots;
  E->x_extent = slots > 0 ? std::max<int64_t>(C->x_extent, 1) : 0;
  double *vtmp = nullptr;
  tbsla_status_t st = alloc_ints(E, &E->idx0, padded);
  if (st == TBSLA_OK && cudaMalloc(&vtmp, (size_t)std::max<int64_t>(padded, 1) * 8) != cudaSuccess) {
    cudaGetLastError();
    st = fail(TBSLA_ERR_OOM, "conversion scratch");
  }
  if (st == TBSLA_OK && padded > 0) {
    ell_fill_kernel<<<std::max(1, std::min((E->rows_pad + 255) / 256, 152 * 16)), 256>>>(
        R->idx0, R->idx1, static_cast<const double *>(R->values[0]), rows, E->rows_pad, max_col, C->f_col, E->idx0,
        vtmp);
    if (cudaGetLastError() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "ELL fill kernel failed");
  }
  if (st == TBSLA_OK) st = store_values_device(E, vtmp, padded, stores, nullptr);
  if (st == TBSLA_OK && cudaDeviceSynchronize() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "ELL conversion failed");
  if (vtmp) cudaFree(vtmp);
  if (st != TBSLA_OK) {
    free_matrix(E);
    return st;
  }
  *out = E;
  return TBSLA_OK;
}

extern "C" tbsla_status_t tbsla_coo_to_dense(const tbsla_matrix_t *C, int stores, tbsla_matrix_t **out) {
  TB_CHECK(C && out, "NULL argument");
  *out = nullptr;
  TB_CHECK(C->format == TBSLA_FMT_COO || C->format == TBSLA_FMT_SCOO,
           "tbsla_coo_to_dense needs a COO / SCOO handle");
  // the reference indexes the dense row with the stored column itself
  TB_CHECK(C->stored == 0 || (int64_t)C->f_col + C->x_extent <= C->n_col,
           "a stored column reaches past n_col = %d", C->n_col);
  tbsla_matrix_t *R = nullptr;
  TB_TRY(tbsla_coo_to_csr(C, TBSLA_STORE_F64, &R));
  struct Drop {
    tbsla_matrix_t *R;
    ~Drop() { free_matrix(R); }
  } drop{R};
  tbsla_matrix *D = new_matrix(TBSLA_FMT_DENSE);
  if (!D) return fail(TBSLA_ERR_OOM, "host allocation failed");
  const int ln_row = C->n_row, ln_col = C->n_col;
  const int64_t n = (int64_t)ln_row * ln_col;
  D->n_row = C->n_row; D->n_col = C->n_col; D->rows = ln_row; D->cols = ln_col;
  D->stored = n;
  D->x_extent = D->rows > 0 ? ln_col : 0;
  double *vtmp = nullptr;
  tbsla_status_t st = TBSLA_OK;
  if (cudaMalloc(&vtmp, (size_t)std::max<int64_t>(n, 1) * 8) != cudaSuccess) {
    cudaGetLastError();
    st = fail(TBSLA_ERR_OOM, "dense conversion buffer (%lld doubles)", (long long)n);
  }
  if (st == TBSLA_OK && n > 0) {
    cudaMemset(vtmp, 0, (size_t)n * 8);
    if (R->stored > 0)
      dense_fill_kernel<<<std::max(1, std::min((ln_row + 255) / 256, 152 * 16)), 256>>>(
          R->idx0, R->idx1, static_cast<const double *>(R->values[0]), ln_row, ln_col, vtmp);
    if (cudaGetLastError() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "dense fill kernel failed");
  }
  if (st == TBSLA_OK) st = store_values_device(D, vtmp, n, stores, nullptr);
  if (st == TBSLA_OK && cudaDeviceSynchronize() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "dense conversion failed");
  if (vtmp) cudaFree(vtmp);
  if (st != TBSLA_OK) {
    free_matrix(D);
    return st;
  }
  *out = D;
  return TBSLA_OK;
}

extern "C" tbsla_status_t tbsla_ell_download(const tbsla_matrix_t *A, int *columns, double *values) {
  TB_CHECK(A && A->format == TBSLA_FMT_ELL, "not an ELL handle");
  const int64_t padded = (int64_t)A->rows_pad * A->max_col;
  if (padded == 0) return TBSLA_OK;
  TB_CHECK(!values || A->values[0], "the F64 value store is not present");
  std::vector<int> cm(columns ? (size_t)padded : 0);
  std::vector<double> vm(values ? (size_t)padded : 0);
  if (columns) TB_CUDA(cudaMemcpy(cm.data(), A->idx0, (size_t)padded * sizeof(int), cudaMemcpyDeviceToHost));
  if (values) TB_CUDA(cudaMemcpy(vm.data(), A->values[0], (size_t)padded * sizeof(double), cudaMemcpyDeviceToHost));
  for (int i = 0; i < A->rows; ++i)
    for (int s = 0; s < A->max_col; ++s) {
      const size_t o = (size_t)s * A->rows_pad + i, r = (size_t)i * A->max_col + s;
      if (columns) columns[r] = cm[o];
      if (values) values[r] = vm[o];
    }
  return TBSLA_OK;
}

extern "C" tbsla_status_t tbsla_dense_download(const tbsla_matrix_t *A, double *values) {
  TB_CHECK(A && A->format == TBSLA_FMT_DENSE, "not a DENSE handle");
  if (A->stored == 0 || !values) return TBSLA_OK;
  TB_CHECK(A->values[0], "the F64 value store is not present");
  TB_CUDA(cudaMemcpy(values, A->values[0], (size_t)A->stored * sizeof(double), cudaMemcpyDeviceToHost));
  return TBSLA_OK;
}

// MatrixSCOO(const MatrixCOO&) (src/cpp/matrix/MatrixSCOO.cpp:53-68) copies the
// arrays and the block geometry: on the device, a copy of the handle's arrays
// (device to device) under the SCOO tag, with its own row bins and carries.
extern "C" tbsla_status_t tbsla_coo_to_scoo(const tbsla_matrix_t *C, int stores, tbsla_matrix_t **out) {
  TB_CHECK(C && out, "NULL argument");
  *out = nullptr;
  TB_CHECK(C->format == TBSLA_FMT_COO || C->format == TBSLA_FMT_SCOO, "tbsla_coo_to_scoo needs a COO / SCOO handle");
  TB_CHECK(C->values[0], "the conversion needs the F64 value store");
  TB_CUDA(cudaSetDevice(C->device));
  tbsla_matrix *S = new_matrix(TBSLA_FMT_SCOO);
  if (!S) return fail(TBSLA_ERR_OOM, "host allocation failed");
  const int64_t n = C->stored;
  S->n_row = C->n_row; S->n_col = C->n_col; S->f_row = C->f_row; S->f_col = C->f_col;
  S->rows = C->rows; S->stored = n; S->x_extent = C->x_extent; S->num_tiles = C->num_tiles;
  S->csr_variant = C->csr_variant;
  tbsla_status_t st = alloc_ints(S, &S->idx0, n);
  if (st == TBSLA_OK) st = alloc_ints(S, &S->idx1, n);
  if (st == TBSLA_OK && n > 0 &&
      (cudaMemcpy(S->idx0, C->idx0, (size_t)n * 4, cudaMemcpyDeviceToDevice) != cudaSuccess ||
       cudaMemcpy(S->idx1, C->idx1, (size_t)n * 4, cudaMemcpyDeviceToDevice) != cudaSuccess))
    st = fail(TBSLA_ERR_CUDA, "array copy failed");
  if (st == TBSLA_OK) st = store_values_device(S, static_cast<const double *>(C->values[0]), n, stores, nullptr);
  if (st == TBSLA_OK) st = alloc_carries(S);
  if (st == TBSLA_OK && C->coo_rowptr && S->n_row > 0) {
    std::vector<int> rp((size_t)S->n_row + 1);
    st = alloc_ints(S, &S->coo_rowptr, (int64_t)S->n_row + 1);
    if (st == TBSLA_OK &&
        (cudaMemcpy(S->coo_rowptr, C->coo_rowptr, rp.size() * 4, cudaMemcpyDeviceToDevice) != cudaSuccess ||
         cudaMemcpy(rp.data(), C->coo_rowptr, rp.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess))
      st = fail(TBSLA_ERR_CUDA, "row pointer copy failed");
    if (st == TBSLA_OK) st = csr_bins(S, rp);
  }
  if (st == TBSLA_OK && cudaDeviceSynchronize() != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "SCOO copy failed");
  if (st != TBSLA_OK) {
    free_matrix(S);
    return st;
  }
  *out = S;
  return TBSLA_OK;
}
