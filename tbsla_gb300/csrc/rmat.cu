// rmat.cu -- R-MAT PageRank matrices (the synthetic graph of the PageRank
// benchmark): edges drawn on the device, assembled into CSR on the host.
//
// R-MAT (Chakrabarti, Zhan, Faloutsos 2004): each of the m edges picks one
// quadrant per bit level, (a, b, c, d) = (top-left, top-right, bottom-left,
// bottom-right), giving a source bit and a destination bit per level (level
// 0 is the most significant).  Uniform numbers are counter based, so every
// edge is reproducible on its own: edge e uses the 64-bit words
// mix64(mix64(seed) + 32*e + w), w = 0, 1, ..., taking the high then the low
// 32 bits of each word as two levels' draws scaled by 2^-32 (mix64 is the
// splitmix64 finaliser of Steele, Lea and Flood 2014).  The same arithmetic
// in plain C lives in the oracle, and the tests compare the two edge lists.
//
// The PageRank matrix is column stochastic: A[v][u] = 1/outdeg(u) for every
// distinct edge u -> v (repeated draws of an edge are merged, self loops
// kept); columns of nodes without out-edges are empty (dangling nodes).
#include <algorithm>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "common.cuh"

namespace tbsla {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// key = (dst << scale) | src
__global__ void rmat_edges_kernel(int scale, int64_t m, double ta, double tb, double tc, uint64_t key,
                                  uint64_t *out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
    uint32_t s = 0, d = 0;
    uint64_t h = 0;
    for (int l = 0; l < scale; ++l) {
      if ((l & 1) == 0) h = mix64(key + 32ull * (uint64_t)e + (uint64_t)(l >> 1));
      const uint32_t bits = (l & 1) ? (uint32_t)h : (uint32_t)(h >> 32);
      const double u = (double)bits * (1.0 / 4294967296.0);
      uint32_t rb, cb;
      if (u < ta) { rb = 0; cb = 0; }
      else if (u < tb) { rb = 0; cb = 1; }
      else if (u < tc) { rb = 1; cb = 0; }
      else { rb = 1; cb = 1; }
      s = (s << 1) | rb;
      d = (d << 1) | cb;
    }
    out[e] = ((uint64_t)d << scale) | s;
  }
}

// LSD radix sort of keys below 2^bits, 16-bit digits, OpenMP over chunks
// (stable per pass).
static void radix_sort(std::vector<uint64_t> &k, int bits) {
  const int64_t n = (int64_t)k.size();
  std::vector<uint64_t> tmp((size_t)n);
  int nt = 1;
#pragma omp parallel
  {
#pragma omp single
    {
#ifdef _OPENMP
      nt = omp_get_num_threads();
#endif
    }
  }
  const int R = 1 << 16;
  std::vector<int64_t> cnt((size_t)nt * R);
  uint64_t *src = k.data(), *dst = tmp.data();
  for (int shift = 0; shift < bits; shift += 16) {
    std::fill(cnt.begin(), cnt.end(), 0);
#pragma omp parallel num_threads(nt)
    {
      int t = 0;
#ifdef _OPENMP
      t = omp_get_thread_num();
#endif
      const int64_t a = n * t / nt, b = n * (t + 1) / nt;
      int64_t *c = cnt.data() + (size_t)t * R;
      for (int64_t i = a; i < b; ++i) ++c[(src[i] >> shift) & (R - 1)];
#pragma omp barrier
#pragma omp single
      {
        int64_t run = 0;
        for (int d = 0; d < R; ++d)
          for (int u = 0; u < nt; ++u) {
            int64_t &x = cnt[(size_t)u * R + d];
            const int64_t v = x;
            x = run;
            run += v;
          }
      }
      for (int64_t i = a; i < b; ++i) dst[c[(src[i] >> shift) & (R - 1)]++] = src[i];
    }
    std::swap(src, dst);
  }
  if (src != k.data()) std::memcpy(k.data(), src, (size_t)n * sizeof(uint64_t));
}

}  // namespace tbsla

using namespace tbsla;

extern "C" tbsla_status_t tbsla_rmat_pagerank_matrix(int scale, int64_t m, double a, double b, double c,
                                                     uint64_t seed, int stores, tbsla_matrix_t **out) {
  TB_CHECK(out, "out is NULL");
  *out = nullptr;
  TB_CHECK(scale >= 1 && scale <= 30, "scale %d out of range [1, 30]", scale);
  TB_CHECK(m >= 0 && m <= ((int64_t)1 << 31) - 1, "edge count out of range");
  TB_CHECK(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0, "bad R-MAT probabilities");
  const int n = 1 << scale;
  std::vector<uint64_t> keys((size_t)m);
  if (m > 0) {
    uint64_t *d = nullptr;
    TB_CUDA(cudaMalloc(&d, (size_t)m * sizeof(uint64_t)));
    rmat_edges_kernel<<<152 * 8, 256>>>(scale, m, a, a + b, a + b + c, mix64(seed), d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(keys.data(), d, (size_t)m * sizeof(uint64_t), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "R-MAT edge generation", __FILE__, __LINE__);
  }
  radix_sort(keys, 2 * scale);
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  const int64_t nnz = (int64_t)keys.size();
  TB_CHECK(nnz <= INT32_MAX, "too many distinct edges");
  const uint64_t mask = ((uint64_t)1 << scale) - 1;
  std::vector<int> rowptr((size_t)n + 1, 0), colidx((size_t)nnz), outdeg((size_t)n, 0);
  for (int64_t k = 0; k < nnz; ++k) {
    const int dst = (int)(keys[(size_t)k] >> scale), src = (int)(keys[(size_t)k] & mask);
    ++rowptr[(size_t)dst + 1];
    colidx[(size_t)k] = src;
    ++outdeg[(size_t)src];
  }
  for (int i = 0; i < n; ++i) rowptr[(size_t)i + 1] += rowptr[(size_t)i];
  std::vector<double> values((size_t)nnz);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < nnz; ++k) values[(size_t)k] = 1.0 / (double)outdeg[(size_t)colidx[(size_t)k]];
  return tbsla_csr_create(n, n, 0, n, rowptr.data(), colidx.data(), values.data(), stores, out);
}

extern "C" tbsla_status_t tbsla_csr_download(const tbsla_matrix_t *A, int *rowptr, int *colidx, double *values) {
  TB_CHECK(A && A->format == TBSLA_FMT_CSR, "not a CSR handle");
  if (rowptr) TB_CUDA(cudaMemcpy(rowptr, A->idx0, ((size_t)A->rows + 1) * sizeof(int), cudaMemcpyDeviceToHost));
  if (colidx && A->stored) TB_CUDA(cudaMemcpy(colidx, A->idx1, (size_t)A->stored * sizeof(int), cudaMemcpyDeviceToHost));
  if (values && A->stored) {
    TB_CHECK(A->values[0], "the F64 value store is not present");
    TB_CUDA(cudaMemcpy(values, A->values[0], (size_t)A->stored * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return TBSLA_OK;
}
