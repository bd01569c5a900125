// device_gen.cu -- the reference's synthetic matrices built on the device
// (tbsla_generate_device).
//
// fill_cdiag (src/cpp/utils/values_generation.cpp:4-24 and the per-format
// fills: CSR MatrixCSR.cpp:234-297, ELL MatrixELL.cpp:192-260, DENSE
// MatrixDENSE.cpp:137-190) needs no random numbers: row i of the block holds
// (i, i - c) when that column lies in the block and, for c != 0, (i, i + c),
// in that order, values 1.  So a row's entry count and its row-pointer offset
// have closed forms, and one thread per row writes the arrays straight into
// the handle: the same arrays as the host fill, bit for bit.
//
// fill_cqmat_stochastic (CSR MatrixCSR.cpp:411-421, ELL MatrixELL.cpp:394-404,
// DENSE MatrixDENSE.cpp:273-286) is fill_cqmat followed by a division of each
// value by its column's sum from the global generator
// (values_generation.cpp:47-62).  The pattern and the column sums come from
// glibc rand_r draws and stay on the host; the division runs on the device
// (IEEE division, the host's quotient bit for bit).
//
// COO and SCOO, and the other generators, take the host path of
// tbsla_generate_matrix.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "host_gen.h"

namespace tbsla {

tbsla_matrix *new_matrix(int format);
void free_matrix(tbsla_matrix *A);
tbsla_status_t alloc_ints(tbsla_matrix *A, int **p, int64_t n);
tbsla_status_t store_values_device(tbsla_matrix *A, const double *d_src, int64_t n, int stores, cudaStream_t s);
tbsla_status_t csr_bins(tbsla_matrix *A, const std::vector<int> &rp);
tbsla_status_t rederive_stores(tbsla_matrix *A, cudaStream_t s);

namespace {

// the block of the matrix a fill covers (range::lnv / range::pflv,
// src/cpp/utils/range.cpp:7-26)
struct Window {
  int64_t fr, lr, fc, lc;
};

int64_t lnv(int64_t size, int pos, int npos) { return size / npos + (pos < size % npos ? 1 : 0); }
int64_t pflv(int64_t size, int pos, int npos) {
  const int64_t mod = size % npos;
  return lnv(size, pos, npos) * pos + (pos >= mod ? mod : 0);
}

// rows r of [fr, i) with the column r + d inside [fc, fc + lc)
__host__ __device__ inline int64_t rows_with(int64_t fr, int64_t i, int64_t fc, int64_t lc, int64_t d) {
  const int64_t a = std::max(fr, fc - d), b = std::min(i, fc + lc - d);
  return b > a ? b - a : 0;
}

__global__ void cdiag_csr_kernel(Window w, int64_t c, int *__restrict__ rowptr, int *__restrict__ colidx,
                                 double *__restrict__ values) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= w.lr; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = w.fr + k;
    // entries of the rows before i: the lower diagonal, then the upper one
    const int64_t start = rows_with(w.fr, i, w.fc, w.lc, -c) + (c != 0 ? rows_with(w.fr, i, w.fc, w.lc, c) : 0);
    rowptr[k] = (int)start;
    if (k == w.lr) break;
    int64_t o = start;
    if (i - c >= w.fc && i - c < w.fc + w.lc) {
      colidx[o] = (int)(i - c);
      values[o++] = 1.0;
    }
    if (c != 0 && i + c >= w.fc && i + c < w.fc + w.lc) {
      colidx[o] = (int)(i + c);
      values[o] = 1.0;
    }
  }
}

// slot-major ELL (rows padded to rows_pad with column f_col, value 0); the
// reference's row i: the lower slot (column i - c or 0 with value 0 when
// outside the block), then for c != 0 the upper slot likewise
__global__ void cdiag_ell_kernel(Window w, int64_t c, int max_col, int rows_pad, int f_col, int *__restrict__ cols,
                                 double *__restrict__ vals) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < rows_pad; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = w.fr + k;
    for (int s = 0; s < max_col; ++s) {
      const int64_t col = s == 0 ? i - c : i + c;
      const bool in = k < w.lr && col >= w.fc && col < w.fc + w.lc;
      cols[(size_t)s * rows_pad + k] = k < w.lr ? (in ? (int)col : 0) : f_col;
      vals[(size_t)s * rows_pad + k] = in ? 1.0 : 0.0;
    }
  }
}

// the dense block (zeroed before): ones at (i, i - c) and (i, i + c)
__global__ void cdiag_dense_kernel(Window w, int64_t c, double *__restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < w.lr; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = w.fr + k;
    if (i - c >= w.fc && i - c < w.fc + w.lc) out[k * w.lc + (i - c - w.fc)] = 1.0;
    if (c != 0 && i + c >= w.fc && i + c < w.fc + w.lc) out[k * w.lc + (i + c - w.fc)] = 1.0;
  }
}

// values[k] /= sum[col[k]] (CSR: every entry; ELL: nonzero slots)
__global__ void divide_by_column_kernel(double *__restrict__ values, const int *__restrict__ cols, int64_t n,
                                        const double *__restrict__ sum, int skip_zero) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double v = values[k];
    if (skip_zero && v == 0) continue;
    values[k] = v / sum[cols[k]];
  }
}

// the dense block: column j divided by sum[fc + j] (a zero sum counts as 1)
__global__ void divide_dense_kernel(double *__restrict__ values, int64_t lr, int64_t lc, int64_t fc,
                                    const double *__restrict__ sum) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < lr * lc; k += (int64_t)gridDim.x * blockDim.x) {
    const double s = sum[fc + k % lc];
    values[k] = values[k] / (s == 0 ? 1.0 : s);
  }
}

int grid_of(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

tbsla_status_t cdiag_on_device(int format, const Window &w, int n_row, int n_col, int c, int stores,
                               tbsla_matrix **out) {
  const cudaStream_t s = nullptr;
  tbsla_matrix *A = new_matrix(format);
  if (!A) return fail(TBSLA_ERR_OOM, "host allocation failed");
  struct Guard {
    tbsla_matrix *A;
    double *tmp = nullptr;
    ~Guard() {
      if (tmp) cudaFree(tmp);
      if (A) free_matrix(A);
    }
  } g{A};
  A->n_row = n_row;
  A->n_col = n_col;
  // entries: the lower and upper diagonals' rows inside the block
  const int64_t n_lo = rows_with(w.fr, w.fr + w.lr, w.fc, w.lc, -c);
  const int64_t n_hi = c != 0 ? rows_with(w.fr, w.fr + w.lr, w.fc, w.lc, c) : 0;
  const int64_t nnz = n_lo + n_hi;
  // the largest column an entry reaches, relative to the block
  int64_t cmax = -1;
  if (n_lo) cmax = std::max(cmax, std::min(w.fr + w.lr, w.fc + w.lc + c) - 1 - c - w.fc);
  if (n_hi) cmax = std::max(cmax, std::min(w.fr + w.lr, w.fc + w.lc - c) - 1 + c - w.fc);
  if (format == TBSLA_FMT_CSR) {
    // as tbsla_csr_create(n_row, n_col, fc, lr, ...): no rows without an entry array
    const int rows = nnz ? (int)w.lr : 0;
    A->f_col = (int)w.fc;
    A->rows = rows;
    A->stored = nnz;
    A->x_extent = cmax + 1;
    TB_TRY(alloc_ints(A, &A->idx0, (int64_t)rows + 1));
    TB_TRY(alloc_ints(A, &A->idx1, nnz));
    TB_CUDA(cudaMalloc(&g.tmp, (size_t)std::max<int64_t>(nnz, 1) * 8));
    if (rows) {
      cdiag_csr_kernel<<<grid_of(w.lr + 1), 256, 0, s>>>(w, c, A->idx0, A->idx1, g.tmp);
    } else {
      TB_CUDA(cudaMemsetAsync(A->idx0, 0, sizeof(int), s));
    }
    TB_CUDA(cudaGetLastError());
    TB_TRY(store_values_device(A, g.tmp, nnz, stores, s));
    std::vector<int> rp((size_t)rows + 1);
    TB_CUDA(cudaMemcpy(rp.data(), A->idx0, rp.size() * sizeof(int), cudaMemcpyDeviceToHost));
    TB_TRY(csr_bins(A, rp));
  } else if (format == TBSLA_FMT_ELL) {
    // MatrixELL::fill_cdiag: max_col 1 (c = 0) or 2; no slots when nothing is stored
    const int max_col = c == 0 ? 1 : 2;
    const int rows = nnz ? (int)w.lr : 0;
    A->x_keep = 0.3f;
    A->f_col = (int)w.fc;
    A->rows = rows;
    A->max_col = max_col;
    A->rows_pad = (rows + 3) / 4 * 4;
    const int64_t padded = (int64_t)A->rows_pad * A->max_col;
    A->stored = (int64_t)rows * A->max_col;
    // padding slots (column 0) read x[0] after the reference's clamp
    A->x_extent = A->stored ? std::max<int64_t>(cmax, 0) + 1 : 0;
    TB_TRY(alloc_ints(A, &A->idx0, padded));
    TB_CUDA(cudaMalloc(&g.tmp, (size_t)std::max<int64_t>(padded, 1) * 8));
    if (padded) cdiag_ell_kernel<<<grid_of(A->rows_pad), 256, 0, s>>>(w, c, A->max_col, A->rows_pad, A->f_col,
                                                                         A->idx0, g.tmp);
    TB_CUDA(cudaGetLastError());
    TB_TRY(store_values_device(A, g.tmp, padded, stores, s));
  } else {
    // MatrixDENSE::fill_cdiag: the ln_row x ln_col block, or nothing when no
    // entry is stored
    const int64_t n = nnz ? w.lr * w.lc : 0;
    A->rows = nnz ? (int)w.lr : 0;
    A->cols = (int)w.lc;
    A->stored = n;
    A->x_extent = A->rows > 0 ? w.lc : 0;
    TB_CUDA(cudaMalloc(&g.tmp, (size_t)std::max<int64_t>(n, 1) * 8));
    if (n) {
      TB_CUDA(cudaMemsetAsync(g.tmp, 0, (size_t)n * 8, s));
      cdiag_dense_kernel<<<grid_of(w.lr), 256, 0, s>>>(w, c, g.tmp);
    }
    TB_CUDA(cudaGetLastError());
    TB_TRY(store_values_device(A, g.tmp, n, stores, s));
  }
  TB_CUDA(cudaDeviceSynchronize());
  *out = A;
  g.A = nullptr;
  return TBSLA_OK;
}

// fill_cqmat's arrays uploaded as a handle with the F64 store, the values
// then divided by the column sums on the device, the other stores derived
tbsla_status_t cqmat_stochastic_on_device(int format, int n_row, int n_col, int c, double q, unsigned seed_mult,
                                          int pr, int pc, int NR, int NC, int stores, tbsla_matrix **out) {
  GenArrays o;
  TB_TRY(generate_arrays(format, 0, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC, o));
  const int *gm = o.geom;
  tbsla_matrix_t *A = nullptr;
  const int up = TBSLA_STORE_F64;
  if (format == TBSLA_FMT_CSR) {
    static const int zero = 0;
    const int rows = o.idx0.empty() ? 0 : (int)o.idx0.size() - 1;
    TB_TRY(tbsla_csr_create(gm[0], gm[1], gm[5], rows, o.idx0.empty() ? &zero : o.idx0.data(), o.idx1.data(),
                            o.values.data(), up | stores, &A));
  } else if (format == TBSLA_FMT_ELL) {
    const int mc = gm[10];
    const int rows = mc ? (int)std::min<int64_t>(gm[2], (int64_t)o.values.size() / mc) : 0;
    TB_TRY(tbsla_ell_create(gm[0], gm[1], gm[5], rows, mc, o.idx0.data(), o.values.data(), up | stores, &A));
  } else {
    TB_TRY(tbsla_dense_create(gm[0], gm[1], o.values.empty() ? 0 : gm[2], gm[3], o.values.data(), up | stores,
                              &A));
  }
  struct Guard {
    tbsla_matrix_t *A;
    double *sum = nullptr;
    ~Guard() {
      if (sum) cudaFree(sum);
      if (A) tbsla_matrix_destroy(A);
    }
  } g{A};
  // the column sums of the global generator (rand_r draws: on the host)
  const std::vector<double> sum = cqmat_column_sums(n_row, n_col, c, q, seed_mult);
  TB_CUDA(cudaMalloc(&g.sum, std::max<size_t>(sum.size(), 1) * sizeof(double)));
  if (!sum.empty()) TB_CUDA(cudaMemcpy(g.sum, sum.data(), sum.size() * sizeof(double), cudaMemcpyHostToDevice));
  double *v = static_cast<double *>(A->values[0]);
  if (format == TBSLA_FMT_CSR && A->stored) {
    divide_by_column_kernel<<<grid_of(A->stored), 256>>>(v, A->idx1, A->stored, g.sum, 0);
  } else if (format == TBSLA_FMT_ELL && A->max_col) {
    // every slot of the slot-major arrays, padding rows included (value 0)
    const int64_t padded = (int64_t)A->rows_pad * A->max_col;
    divide_by_column_kernel<<<grid_of(padded), 256>>>(v, A->idx0, padded, g.sum, 1);
  } else if (format == TBSLA_FMT_DENSE && A->stored) {
    divide_dense_kernel<<<grid_of(A->stored), 256>>>(v, A->rows, A->cols, gm[5], g.sum);
  }
  TB_CUDA(cudaGetLastError());
  TB_TRY(rederive_stores(A, nullptr));
  if (!(stores & TBSLA_STORE_F64)) {
    // only the reduced stores were asked for: drop the F64 one
    cudaFree(A->values[0]);
    A->values[0] = nullptr;
    if (A->sell_vals[0]) cudaFree(A->sell_vals[0]);
    A->sell_vals[0] = nullptr;
    A->stores &= ~TBSLA_STORE_F64;
  }
  TB_CUDA(cudaDeviceSynchronize());
  *out = A;
  g.A = nullptr;
  return TBSLA_OK;
}

}  // namespace
}  // namespace tbsla

using namespace tbsla;

extern "C" tbsla_status_t tbsla_generate_device(int format, int gen, int n_row, int n_col, int c, double q,
                                                unsigned int seed_mult, int pr, int pc, int NR, int NC, int stores,
                                                tbsla_matrix_t **out) {
  TB_CHECK(out, "out is NULL");
  *out = nullptr;
  TB_CHECK(n_row >= 0 && n_col >= 0 && NR >= 1 && NC >= 1 && pr >= 0 && pc >= 0 && pr < NR && pc < NC,
           "bad geometry");
  TB_CHECK(stores & (TBSLA_STORE_F64 | TBSLA_STORE_F32 | TBSLA_STORE_BF16), "no value store requested");
  const bool device_format = format == TBSLA_FMT_CSR || format == TBSLA_FMT_ELL || format == TBSLA_FMT_DENSE;
  if (device_format && gen == 1) {
    const Window w{pflv(n_row, pr, NR), lnv(n_row, pr, NR), pflv(n_col, pc, NC), lnv(n_col, pc, NC)};
    return cdiag_on_device(format, w, n_row, n_col, c, stores, out);
  }
  if (device_format && gen == 2) {
    TB_CHECK(c >= 0, "c must be >= 0");
    return cqmat_stochastic_on_device(format, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC, stores, out);
  }
  TB_CHECK(pr == 0 && pc == 0 && NR == 1 && NC == 1, "this format / generator is built on the host for the whole "
                                                     "matrix only (block 0,0 of 1x1)");
  return tbsla_generate_matrix(format, gen, n_row, n_col, c, q, seed_mult, stores, out);
}
