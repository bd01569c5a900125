// pr_relabel.cu -- PageRank on a relabelled copy of the graph.
//
// A PageRank sweep gathers the iterate at the column of every stored entry.
// On power-law graphs (R-MAT) most gathers land on a small set of hot
// vertices, but in the generator's labels these are spread over the whole
// index range: every hot value shares its 32-byte sector with cold ones, so
// the hot set needs several times its size in L2 and most gathers go to
// DRAM.  Relabelling the vertices in decreasing out-degree (stored entries
// per column) packs the hot values together.  The relabelling is symmetric
// (rows and columns), so a sweep on the copy is the sweep on the original
// with permuted vectors; teleport, dangling mass, residual and maximum are
// permutation invariant, and the result is gathered back to the original
// labels.  Each row's entries are sorted by their new column, so the lanes
// of a long row's group gather neighbouring values of the hot set in one
// load instruction (R-MAT 2^24: 1.54 -> 1.40 ms per FP64 sweep against the
// rows in their original order); sums differ from the original labels'
// only by rounding.
//
// Order: out-degree class (floor(log2(out-degree + 1)), descending) first,
// which keeps the hot values together; inside a class, in-degree (the row
// length) descending, so that neighbouring rows have similar lengths and
// the thread-per-row kernel's warps run similar trip counts.
//
// The copy is built once per handle on the host (download, counting sort by
// degree, row copy) and uploaded as an ordinary CSR handle with the same
// value stores.
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace tbsla {

tbsla_status_t csr_unsplit_tiny(tbsla_matrix *A);

namespace {

constexpr int kBandSamples = 4096;
constexpr int kBandWidth = 1024;

// entries within kBandWidth of the diagonal, and all entries, on
// kBandSamples rows spread evenly (one warp per sampled row)
__global__ void band_sample_kernel(const int *__restrict__ rowptr, const int *__restrict__ colidx, int n,
                                   int f_col, unsigned long long *cnt) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= kBandSamples) return;
  const int r = (int)(((long long)w * n) / kBandSamples);
  const int a = rowptr[r], b = rowptr[r + 1];
  unsigned long long near = 0, all = 0;
  for (int k = a + lane; k < b; k += 32) {
    ++all;
    if (abs(colidx[k] - f_col - r) <= kBandWidth) ++near;
  }
  for (int o = 16; o > 0; o >>= 1) {
    near += __shfl_down_sync(0xffffffffu, near, o);
    all += __shfl_down_sync(0xffffffffu, all, o);
  }
  if (lane == 0) {
    atomicAdd(cnt, near);
    atomicAdd(cnt + 1, all);
  }
}

// deg[c - f_col] += 1 for every stored entry
__global__ void column_count_kernel(const int *__restrict__ colidx, int64_t nnz, int f_col, int *deg) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(deg + (colidx[k] - f_col), 1);  // columns are in [f_col, f_col + n) (candidate())
}

// out[v] = x[newid[v]]
__global__ void relabel_gather_kernel(const double *__restrict__ x, const int *__restrict__ newid, int n,
                                      double *__restrict__ out) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) out[v] = x[newid[v]];
}

int cls_max(int maxdeg) { return 31 - __builtin_clz((unsigned)maxdeg + 1u); }

bool candidate(const tbsla_matrix *A) {
  return A->format == TBSLA_FMT_CSR && A->csr_variant == 0 && A->n_row == A->n_col && A->rows == A->n_row &&
         A->stored > 0 && A->values[0] != nullptr && A->x_extent <= A->n_col;
}

// banded matrices (cqmat, cdiag) already gather locally
tbsla_status_t banded(const tbsla_matrix *A, bool *is_banded) {
  unsigned long long *d = nullptr, h[2] = {0, 0};
  TB_CUDA(cudaMalloc(&d, 2 * sizeof(unsigned long long)));
  cudaMemset(d, 0, 2 * sizeof(unsigned long long));
  band_sample_kernel<<<kBandSamples * 32 / 256, 256>>>(A->idx0, A->idx1, A->n_row, A->f_col, d);
  const cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  TB_CUDA(e);
  *is_banded = h[1] == 0 || 2 * h[0] >= h[1];
  return TBSLA_OK;
}

tbsla_status_t build(tbsla_matrix *A, bool check_skew, bool *built) {
  *built = false;
  const int n = A->n_row;
  const int64_t nnz = A->stored;
  // out-degrees on the device
  int *d_deg = nullptr;
  TB_CUDA(cudaMalloc(&d_deg, (size_t)n * sizeof(int)));
  cudaMemset(d_deg, 0, (size_t)n * sizeof(int));
  column_count_kernel<<<152 * 8, 256>>>(A->idx1, nnz, A->f_col, d_deg);
  std::vector<int> deg((size_t)n);
  const cudaError_t e = cudaMemcpy(deg.data(), d_deg, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d_deg);
  TB_CUDA(e);
  const int maxdeg = *std::max_element(deg.begin(), deg.end());
  if (check_skew) {
    // entries in the columns of the n/10 vertices of highest out-degree
    std::vector<int64_t> hist((size_t)maxdeg + 1, 0);
    for (int v = 0; v < n; ++v) ++hist[(size_t)deg[(size_t)v]];
    int64_t taken = 0, top = 0;
    for (int d = maxdeg; d >= 0 && taken < n / 10; --d) {
      const int64_t t = std::min<int64_t>(hist[(size_t)d], n / 10 - taken);
      taken += t;
      top += t * d;
    }
    if (2 * top < nnz) return TBSLA_OK;  // no hot set worth packing
  }
  std::vector<int> rp((size_t)n + 1), ci((size_t)nnz);
  std::vector<double> va((size_t)nnz);
  TB_TRY(tbsla_csr_download(A, rp.data(), ci.data(), va.data()));
  // two stable counting sorts: by in-degree (descending), then by out-degree
  // class (descending)
  int maxin = 0;
  for (int v = 0; v < n; ++v) maxin = std::max(maxin, rp[(size_t)v + 1] - rp[(size_t)v]);
  std::vector<int> by_in((size_t)n), order((size_t)n);
  {
    std::vector<int64_t> start((size_t)maxin + 2, 0);
    for (int v = 0; v < n; ++v) ++start[(size_t)(maxin - (rp[(size_t)v + 1] - rp[(size_t)v])) + 1];
    for (size_t k = 1; k < start.size(); ++k) start[k] += start[k - 1];
    for (int v = 0; v < n; ++v) by_in[(size_t)start[(size_t)(maxin - (rp[(size_t)v + 1] - rp[(size_t)v]))]++] = v;
  }
  {
    auto cls = [&](int v) { return 31 - __builtin_clz((unsigned)deg[(size_t)v] + 1u); };  // floor(log2(d + 1))
    const int top_cls = cls_max(maxdeg);
    std::vector<int64_t> start((size_t)top_cls + 2, 0);
    for (int v = 0; v < n; ++v) ++start[(size_t)(top_cls - cls(v)) + 1];
    for (size_t k = 1; k < start.size(); ++k) start[k] += start[k - 1];
    for (int i = 0; i < n; ++i) {
      const int v = by_in[(size_t)i];
      order[(size_t)start[(size_t)(top_cls - cls(v))]++] = v;
    }
  }
  std::vector<int> newid((size_t)n);
  for (int i = 0; i < n; ++i) newid[(size_t)order[(size_t)i]] = i;
  // the copy: row i is old row order[i] with columns relabelled
  std::vector<int> nrp((size_t)n + 1);
  nrp[0] = 0;
  for (int i = 0; i < n; ++i) {
    const int old = order[(size_t)i];
    nrp[(size_t)i + 1] = nrp[(size_t)i] + (rp[(size_t)old + 1] - rp[(size_t)old]);
  }
  std::vector<int> nci((size_t)nnz);
  std::vector<double> nva((size_t)nnz);
  const int f_col = A->f_col;
#pragma omp parallel
  {
    std::vector<int> idx;
    std::vector<int> tc;
    std::vector<double> tv;
#pragma omp for schedule(dynamic, 4096)
    for (int i = 0; i < n; ++i) {
      const int old = order[(size_t)i];
      const int o0 = nrp[(size_t)i], len = nrp[(size_t)i + 1] - o0;
      int *c = nci.data() + o0;
      double *v = nva.data() + o0;
      for (int k = 0; k < len; ++k) {
        c[k] = newid[(size_t)(ci[(size_t)rp[(size_t)old] + k] - f_col)];
        v[k] = va[(size_t)rp[(size_t)old] + k];
      }
      // entries in increasing new column (stable: repeated columns keep their order)
      if (len <= 64) {
        for (int k = 1; k < len; ++k) {
          const int ck = c[k];
          const double vk = v[k];
          int j = k - 1;
          for (; j >= 0 && c[j] > ck; --j) {
            c[j + 1] = c[j];
            v[j + 1] = v[j];
          }
          c[j + 1] = ck;
          v[j + 1] = vk;
        }
      } else {
        idx.resize((size_t)len);
        for (int k = 0; k < len; ++k) idx[(size_t)k] = k;
        std::stable_sort(idx.begin(), idx.end(), [c](int p, int q) { return c[p] < c[q]; });
        tc.assign(c, c + len);
        tv.assign(v, v + len);
        for (int k = 0; k < len; ++k) {
          c[k] = tc[(size_t)idx[(size_t)k]];
          v[k] = tv[(size_t)idx[(size_t)k]];
        }
      }
    }
  }
  rp.clear(); rp.shrink_to_fit();
  ci.clear(); ci.shrink_to_fit();
  va.clear(); va.shrink_to_fit();
  tbsla_matrix_t *B = nullptr;
  TB_TRY(tbsla_csr_create(n, n, 0, n, nrp.data(), nci.data(), nva.data(), A->stores, &B));
  // rows are grouped by length here: one thread per short row over the
  // whole list (the tiny-row tiles measured slower on this order)
  const tbsla_status_t su = csr_unsplit_tiny(B);
  if (su != TBSLA_OK) {
    tbsla_matrix_destroy(B);
    return su;
  }
  B->x_keep = A->x_keep;
  B->x_keep_range = A->x_keep_range;
  B->short_mode = A->short_mode;
  int *d_newid = nullptr;
  if (cudaMalloc(&d_newid, (size_t)n * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    tbsla_matrix_destroy(B);
    return fail(TBSLA_ERR_OOM, "relabel map (%d ints)", n);
  }
  const cudaError_t e2 = cudaMemcpy(d_newid, newid.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice);
  if (e2 != cudaSuccess) {
    cudaFree(d_newid);
    tbsla_matrix_destroy(B);
    TB_CUDA(e2);
  }
  A->pr_relabel = B;
  A->pr_newid = d_newid;
  A->pr_newid_host = std::move(newid);
  *built = true;
  return TBSLA_OK;
}

}  // namespace

// The relabelled copy to run PageRank on, or NULL for A itself.
tbsla_status_t pr_relabelled(tbsla_matrix *A, tbsla_matrix **B) {
  *B = nullptr;
  if (A->pr_relabel_mode == 0 || !candidate(A)) return TBSLA_OK;
  if (A->pr_relabel_state == 1) {
    *B = A->pr_relabel;
    return TBSLA_OK;
  }
  if (A->pr_relabel_state == 2 && A->pr_relabel_mode == -1) return TBSLA_OK;
  const bool forced = A->pr_relabel_mode == 1;
  if (!forced) {
    bool is_banded = true;
    if (A->n_row < (1 << 20)) {
      A->pr_relabel_state = 2;
      return TBSLA_OK;
    }
    TB_TRY(banded(A, &is_banded));
    if (is_banded) {
      A->pr_relabel_state = 2;
      return TBSLA_OK;
    }
  }
  bool built = false;
  TB_TRY(build(A, !forced, &built));
  A->pr_relabel_state = built ? 1 : 2;
  *B = built ? A->pr_relabel : nullptr;
  return TBSLA_OK;
}

// out[v] = x[newid[v]] for the n vertices of A, ordered on s
tbsla_status_t pr_relabel_gather(const tbsla_matrix *A, const double *x, double *out, cudaStream_t s) {
  relabel_gather_kernel<<<152 * 4, 256, 0, s>>>(x, A->pr_newid, A->n_row, out);
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

}  // namespace tbsla
