// ppr_batch.cu -- many personalized PageRank vectors of one graph solved
// together (TBSLA_PR_TELEPORT form, one teleport set per vector).
//
// The k iterates are kept in tiles of KT columns (KT = 2, 4, 8, 16 or 32), each
// tile row-major: tile t, row i holds X[i*KT + c] for its KT vectors, so the
// gather of a column index brings all KT values in one contiguous segment.
// A group of KT lanes sums a row, lane c for vector c: no cross-lane
// reduction, every lane does useful multiply-adds.  Rows longer than
// kPprChunk entries are cut into chunks (partials + a fixup kernel) so that
// hub rows of power-law graphs spread over many groups.
//
// Per vector c with seed set P_c (v_c = 1/|P_c| on P_c):
//   x_c <- beta A x_c + (beta d.x_c + 1 - beta) v_c,
// stopped on its own when ||x_c - x_c,prev||_1 < tol (or max_iter sweeps);
// a stopped vector is frozen (its lanes copy the old value), and a tile
// whose vectors have all stopped skips its kernels.  Every check_every
// sweeps the host writes out the vectors that stopped and, when the ones
// still running fit in fewer tiles, repacks them (iterates, seeds, control
// state) so that no tile sweeps for one slow vector while its other lanes
// idle.  A column's arithmetic and its reduction order do not depend on its
// tile or lane, so repacking leaves every result bit for bit as it was.
// All sums have a fixed order: results do not depend on scheduling.
//
// Large skewed graphs run on the degree-relabelled copy (pr_relabel.cu);
// seeds are mapped in and the results gathered back to the original labels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "product.cuh"

namespace tbsla {

tbsla_status_t pr_relabelled(tbsla_matrix *A, tbsla_matrix **B);

namespace {

constexpr int kPprChunk = 512;

struct ColCtl {
  double add;    // beta * d.x + cst of the current iterate
  double resid;  // last L1 change
  double tol;    // the column's stopping threshold
  int iter, done;
};
struct TileCtl {
  int done, iter;  // iter: sweeps run on the tile (parity of the buffer holding it)
  int pad[2];
};

// Lane-column sums of a block for (resid, dmass) into partials[(part*KT+c)*2]
template <int KT>
__device__ __forceinline__ void block_columns(double r, double d, double *partials, int part) {
  __shared__ double sh[8][32][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  #pragma unroll
  for (int o = 16; o >= KT; o >>= 1) {
    r += __shfl_down_sync(0xffffffffu, r, o);
    d += __shfl_down_sync(0xffffffffu, d, o);
  }
  if (lane < KT) {
    sh[warp][lane][0] = r;
    sh[warp][lane][1] = d;
  }
  __syncthreads();
  if (threadIdx.x < KT) {
    double a = 0, b = 0;
    const int nw = blockDim.x >> 5;
    for (int w = 0; w < nw; ++w) {
      a += sh[w][threadIdx.x][0];
      b += sh[w][threadIdx.x][1];
    }
    partials[((size_t)part * KT + threadIdx.x) * 2 + 0] = a;
    partials[((size_t)part * KT + threadIdx.x) * 2 + 1] = b;
  }
}

// y for one finished row (all KT lanes of the group)
template <typename T, int KT>
__device__ __forceinline__ void ppr_emit(int row, int c, T acc, const T *xo, T *xn, const unsigned *seeds,
                                         const unsigned char *dmask, const ColCtl *col, const double *inv_size,
                                         double beta, const T *rhs, double &r_acc, double &d_acc) {
  const ColCtl cc = col[c];
  const T old = xo[(size_t)row * KT + c];
  T y;
  if (cc.done) {
    y = old;
  } else {
    double t = ((seeds[row] >> c) & 1u) ? cc.add * inv_size[c] : 0.0;
    if (rhs) t += (double)rhs[(size_t)row * KT + c];
    y = (T)((double)beta * (double)acc + t);
    r_acc += fabs((double)y - (double)old);
  }
  if (dmask[row]) d_acc += (double)y;
  xn[(size_t)row * KT + c] = y;
}

// items: (row, begin, end, chunk slot or -1)
template <typename T, int KT>
__global__ void __launch_bounds__(256) ppr_spmm_kernel(const int4 *__restrict__ items, int n_items,
                                                      const int *__restrict__ colidx, const T *__restrict__ values,
                                                      const T *__restrict__ xo, T *__restrict__ xn,
                                                      const unsigned *__restrict__ seeds,
                                                      const unsigned char *__restrict__ dmask,
                                                      const ColCtl *__restrict__ col,
                                                      const double *__restrict__ inv_size, double beta,
                                                      const T *__restrict__ rhs, T *__restrict__ chunk_partials,
                                                      double *partials, const TileCtl *tile) {
  if (*(volatile const int *)&tile->done) return;
  const int c = threadIdx.x & (KT - 1);
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / KT;
  double r_acc = 0, d_acc = 0;
  for (int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / KT; g < n_items; g += ng) {
    const int4 it = items[g];
    T acc = 0;
    int e = it.y;
    for (; e + 4 <= it.z; e += 4) {
      const int c0 = __ldg(colidx + e), c1 = __ldg(colidx + e + 1), c2 = __ldg(colidx + e + 2),
                c3 = __ldg(colidx + e + 3);
      const T v0 = __ldg(values + e), v1 = __ldg(values + e + 1), v2 = __ldg(values + e + 2),
              v3 = __ldg(values + e + 3);
      const T x0 = __ldg(xo + (size_t)c0 * KT + c), x1 = __ldg(xo + (size_t)c1 * KT + c),
              x2 = __ldg(xo + (size_t)c2 * KT + c), x3 = __ldg(xo + (size_t)c3 * KT + c);
      acc = fma(v0, x0, acc);
      acc = fma(v1, x1, acc);
      acc = fma(v2, x2, acc);
      acc = fma(v3, x3, acc);
    }
    for (; e < it.z; ++e) acc = fma(__ldg(values + e), __ldg(xo + (size_t)__ldg(colidx + e) * KT + c), acc);
    if (it.w >= 0) chunk_partials[(size_t)it.w * KT + c] = acc;
    else ppr_emit<T, KT>(it.x, c, acc, xo, xn, seeds, dmask, col, inv_size, beta, rhs, r_acc, d_acc);
  }
  block_columns<KT>(r_acc, d_acc, partials, blockIdx.x);
}

// rows cut into chunks: crow[h] = (row, first slot), crow[n].y = total slots
template <typename T, int KT>
__global__ void __launch_bounds__(256) ppr_fixup_kernel(const int2 *__restrict__ crow, int n_crow,
                                                       const T *__restrict__ chunk_partials,
                                                       const T *__restrict__ xo, T *__restrict__ xn,
                                                       const unsigned *__restrict__ seeds,
                                                       const unsigned char *__restrict__ dmask,
                                                       const ColCtl *__restrict__ col,
                                                       const double *__restrict__ inv_size, double beta,
                                                       const T *__restrict__ rhs, double *partials, int part_base,
                                                       const TileCtl *tile) {
  if (*(volatile const int *)&tile->done) return;
  const int c = threadIdx.x & (KT - 1);
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / KT;
  double r_acc = 0, d_acc = 0;
  for (int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / KT; g < n_crow; g += ng) {
    const int2 h = crow[g];
    T acc = 0;
    for (int s = h.y; s < crow[g + 1].y; ++s) acc += chunk_partials[(size_t)s * KT + c];
    ppr_emit<T, KT>(h.x, c, acc, xo, xn, seeds, dmask, col, inv_size, beta, rhs, r_acc, d_acc);
  }
  block_columns<KT>(r_acc, d_acc, partials, part_base + blockIdx.x);
}

// per column: sum the parts in order, advance the column, then the tile
template <int KT>
__global__ void ppr_finalize_kernel(const double *__restrict__ partials, int nparts, ColCtl *col, TileCtl *tile,
                                    double beta, double cst, int max_iter, int k_in_tile, int first) {
  __shared__ int active;
  if (threadIdx.x == 0) active = 0;
  __syncthreads();
  if (*(volatile int *)&tile->done) return;
  const int c = threadIdx.x;
  if (c < KT) {
    double r = 0, d = 0;
    for (int p = 0; p < nparts; ++p) {
      r += partials[((size_t)p * KT + c) * 2 + 0];
      d += partials[((size_t)p * KT + c) * 2 + 1];
    }
    ColCtl &cc = col[c];
    if (first) {
      cc.add = beta * d + cst;  // initial vector: only the dangling mass is new
    } else if (!cc.done) {
      cc.iter += 1;
      cc.resid = r;
      cc.add = beta * d + cst;
      cc.done = r < cc.tol || cc.iter >= max_iter;
    } else {
      cc.add = beta * d + cst;
    }
    if (c < k_in_tile && !cc.done) atomicOr(&active, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!first) tile->iter += 1;
    tile->done = active == 0;
  }
}

// x0 = v (seeds), dangling mass of x0 per column
template <typename T, int KT>
__global__ void __launch_bounds__(256) ppr_init_kernel(int n, const unsigned *__restrict__ seeds,
                                                      const unsigned char *__restrict__ dmask,
                                                      const double *__restrict__ inv_size, T *__restrict__ x,
                                                      double *partials) {
  const int c = threadIdx.x & (KT - 1);
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / KT;
  double d_acc = 0;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / KT; i < n; i += ng) {
    const T v = ((seeds[i] >> c) & 1u) ? (T)inv_size[c] : T(0);
    x[(size_t)i * KT + c] = v;
    if (dmask[i]) d_acc += (double)v;
  }
  block_columns<KT>(0.0, d_acc, partials, blockIdx.x);
}

// x (one tile) from FP64 vectors in the original labels: vector vec[c] of
// src (src + vec[c] * n) at tile row newid[u] (u when not relabelled);
// columns with vec[c] < 0 get 0.  With partials: the dangling mass per column.
template <typename T, int KT>
__global__ void __launch_bounds__(256) ppr_load_kernel(int n, const double *__restrict__ src,
                                                      const int *__restrict__ vec, const int *__restrict__ newid,
                                                      const unsigned char *__restrict__ dmask, T *__restrict__ x,
                                                      double *partials) {
  const int c = threadIdx.x & (KT - 1);
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / KT;
  const int v = vec[c];
  double d_acc = 0;
  for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / KT; u < n; u += ng) {
    const int i = newid ? newid[u] : (int)u;
    const T val = v >= 0 ? (T)src[(size_t)v * n + u] : T(0);
    x[(size_t)i * KT + c] = val;
    if (partials && dmask[i]) d_acc += (double)val;
  }
  if (partials) block_columns<KT>(0.0, d_acc, partials, blockIdx.x);
}

// dmask[j] = 1 when column j holds no nonzero value
template <typename T>
__global__ void ppr_dangling_kernel(const int *__restrict__ colidx, const T *__restrict__ values, int64_t nnz,
                                    unsigned char *dmask) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
    if (values[k] != T(0)) dmask[colidx[k]] = 0;
}

// out[v_j * n + u] = column c_j of a tile at row map(u), as FP64, for the
// cnt (column, vector) pairs of a list
struct PprPicks {
  int cnt;
  int col[32], vec[32];
};
template <typename T, int KT>
__global__ void ppr_pick_kernel(const T *__restrict__ x, int n, const int *__restrict__ newid, PprPicks pk,
                                double *__restrict__ out) {
  const int64_t total = (int64_t)n * pk.cnt;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t / n), u = (int)(t % n);
    const int i = newid ? newid[u] : u;
    out[(size_t)pk.vec[j] * n + u] = (double)x[(size_t)i * KT + pk.col[j]];
  }
}

// repacked layout: slot s of the new tiles takes old slot map[s] (-1: zero)
template <typename T, int KT>
__global__ void ppr_move_kernel(const T *__restrict__ src, T *__restrict__ dst, int n, const int *__restrict__ map,
                                int new_tiles) {
  const int64_t total = (int64_t)new_tiles * n * KT;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(q % KT);
    const int64_t ti = q / KT;
    const int i = (int)(ti % n), t = (int)(ti / n);
    const int from = map[t * KT + c];
    dst[q] = from < 0 ? T(0) : src[((size_t)(from / KT) * n + i) * KT + (from % KT)];
  }
}

// Options of one batched solve: by default x0 = v_c and the teleport form
// x = beta A x + (beta d.x + 1 - beta) v_c.  A defect-correction solve passes
// x0 = rhs = r_c and cst = 0: e = beta A e + beta (d.e) v_c + r_c.
struct RunOpts {
  const double *x0 = nullptr;   // start: vector c at x0 + src(c) * n (original labels), FP64
  const double *rhs = nullptr;  // added to every sweep: rhs + src(c) * n
  const int *src = nullptr;     // host: column of x0 / rhs for vector c (NULL: c)
  double cst = -1.0;            // the constant of the teleport term (< 0: 1 - beta)
  const double *tol = nullptr;  // host: stopping threshold per vector (NULL: p->tol)
};

template <typename T, int KT>
tbsla_status_t run_tiles(const tbsla_matrix *M, const int *newid_dev, const std::vector<int> *newid_host,
                         const tbsla_pagerank_params_t *p, int k, const int *nodes, const int *offsets,
                         double *d_out, int *iters_out, double *resid_out, cudaStream_t s,
                         const RunOpts &opt = RunOpts()) {
  const int n = M->n_row;
  const int64_t nnz = M->stored;
  const T *values = static_cast<const T *>(M->values[std::is_same<T, double>::value ? 0 : 1]);
  TB_CHECK(values, "the matrix lacks the %s value store", std::is_same<T, double>::value ? "F64" : "F32");
  const int tiles = (k + KT - 1) / KT;
  // work items: rows, and chunks of rows longer than kPprChunk
  std::vector<int> rp((size_t)n + 1);
  TB_CUDA(cudaMemcpy(rp.data(), M->idx0, ((size_t)n + 1) * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int4> items;
  std::vector<int2> crow;
  int slots = 0;
  items.reserve((size_t)n);
  for (int r = 0; r < n; ++r) {
    const int a = rp[(size_t)r], b = rp[(size_t)r + 1];
    if (b - a <= kPprChunk) {
      items.push_back(make_int4(r, a, b, -1));
      continue;
    }
    crow.push_back(make_int2(r, slots));
    for (int e = a; e < b; e += kPprChunk) items.push_back(make_int4(r, e, std::min(e + kPprChunk, b), slots++));
  }
  const int n_crow = (int)crow.size();
  crow.push_back(make_int2(-1, slots));
  // seeds: bit c of seeds[t*n + i] = row i is a seed of vector t*KT + c
  std::vector<unsigned> seeds((size_t)tiles * n, 0u);
  std::vector<double> inv((size_t)tiles * KT, 0.0);
  std::vector<std::vector<int>> seed_sets((size_t)k);  // per vector, in the matrix's labels
  for (int c = 0; c < k; ++c) {
    const int b = offsets[c], e = offsets[c + 1];
    TB_CHECK(e > b, "vector %d has an empty seed set", c);
    std::vector<int> &dist = seed_sets[(size_t)c];
    for (int q = b; q < e; ++q) {
      int v = nodes[q];
      TB_CHECK(v >= 0 && v < n, "seed %d of vector %d outside [0, %d)", v, c, n);
      if (newid_host) v = (*newid_host)[(size_t)v];
      dist.push_back(v);
    }
    std::sort(dist.begin(), dist.end());
    dist.erase(std::unique(dist.begin(), dist.end()), dist.end());
    for (int v : dist) seeds[(size_t)(c / KT) * n + v] |= 1u << (c % KT);
    inv[(size_t)c] = 1.0 / (double)dist.size();
  }
  const int grid_mm = kStrideBlocks;
  const int grid_fx = std::max(1, std::min((n_crow * KT + 255) / 256, 152 * 4));
  const int grid_in = 152 * 4;
  const int nparts = std::max(grid_mm + grid_fx, grid_in);
  // device buffers
  const size_t xbytes = (size_t)n * KT * sizeof(T);
  T *x[2] = {nullptr, nullptr};
  T *chunk = nullptr;
  int4 *d_items = nullptr;
  int2 *d_crow = nullptr;
  unsigned *d_seeds = nullptr;
  unsigned char *dmask = nullptr;
  double *d_inv = nullptr, *partials = nullptr;
  ColCtl *d_col = nullptr;
  TileCtl *d_tile = nullptr;
  T *rhs_t[2] = {nullptr, nullptr};  // the right-hand side in the tiles' layout (ping-pong for repacking)
  int *d_vec = nullptr;              // per slot: the column of x0 / rhs it holds, or -1
  std::vector<void *> owned;
  tbsla_status_t st = TBSLA_OK;
  auto alloc = [&](void **ptr, size_t bytes) {
    if (st != TBSLA_OK) return;
    if (cudaMalloc(ptr, std::max<size_t>(bytes, 16)) != cudaSuccess) {
      cudaGetLastError();
      st = fail(TBSLA_ERR_OOM, "batched PageRank buffers (%zu bytes)", bytes);
      return;
    }
    owned.push_back(*ptr);
  };
  alloc((void **)&x[0], (size_t)tiles * xbytes);
  alloc((void **)&x[1], (size_t)tiles * xbytes);
  alloc((void **)&chunk, (size_t)std::max(slots, 1) * KT * sizeof(T));
  alloc((void **)&d_items, items.size() * sizeof(int4));
  alloc((void **)&d_crow, crow.size() * sizeof(int2));
  alloc((void **)&d_seeds, seeds.size() * sizeof(unsigned));
  alloc((void **)&dmask, (size_t)n);
  alloc((void **)&d_inv, inv.size() * sizeof(double));
  alloc((void **)&partials, (size_t)tiles * nparts * KT * 2 * sizeof(double));
  alloc((void **)&d_col, (size_t)tiles * KT * sizeof(ColCtl));
  alloc((void **)&d_tile, (size_t)tiles * sizeof(TileCtl));
  alloc((void **)&d_vec, (size_t)tiles * KT * sizeof(int));
  if (opt.rhs) {
    alloc((void **)&rhs_t[0], (size_t)tiles * xbytes);
    alloc((void **)&rhs_t[1], (size_t)tiles * xbytes);
  }
  auto cleanup = [&]() {
    cudaStreamSynchronize(s);
    for (void *q : owned) cudaFree(q);
  };
  if (st != TBSLA_OK) { cleanup(); return st; }
  const double cst = opt.cst < 0 ? 1.0 - p->beta : opt.cst;
  auto src_col = [&](int v) { return v < 0 ? -1 : opt.src ? opt.src[v] : v; };
  std::vector<ColCtl> hcol((size_t)tiles * KT);
  std::vector<int> hvec((size_t)tiles * KT, -1);
  for (int c = 0; c < tiles * KT; ++c) {
    // padding columns start stopped
    hcol[(size_t)c] = ColCtl{0.0, 0.0, c < k && opt.tol ? opt.tol[c] : p->tol, 0, c >= k ? 1 : 0};
    hvec[(size_t)c] = src_col(c < k ? c : -1);
  }
  std::vector<TileCtl> htile((size_t)tiles, TileCtl{0, 0, {0, 0}});
  if (p->max_iter == 0)
    for (auto &tc : htile) tc.done = 1;
  cudaError_t e = cudaSuccess;
  auto up = [&](void *d, const void *h, size_t b) {
    if (e == cudaSuccess && b) e = cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, s);
  };
  up(d_items, items.data(), items.size() * sizeof(int4));
  up(d_crow, crow.data(), crow.size() * sizeof(int2));
  up(d_seeds, seeds.data(), seeds.size() * sizeof(unsigned));
  up(d_inv, inv.data(), inv.size() * sizeof(double));
  up(d_col, hcol.data(), hcol.size() * sizeof(ColCtl));
  up(d_tile, htile.data(), htile.size() * sizeof(TileCtl));
  up(d_vec, hvec.data(), hvec.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(dmask, 1, (size_t)n, s);
  if (e != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank upload: %s", cudaGetErrorString(e)); }
  ppr_dangling_kernel<T><<<152 * 8, 256, 0, s>>>(M->idx1, values, nnz, dmask);
  const double beta = p->beta;
  for (int t = 0; t < tiles; ++t) {
    double *pt = partials + (size_t)t * nparts * KT * 2;
    if (opt.x0)
      ppr_load_kernel<T, KT><<<grid_in, 256, 0, s>>>(n, opt.x0, d_vec + (size_t)t * KT, newid_dev, dmask,
                                                     x[0] + (size_t)t * n * KT, pt);
    else
      ppr_init_kernel<T, KT><<<grid_in, 256, 0, s>>>(n, d_seeds + (size_t)t * n, dmask, d_inv + (size_t)t * KT,
                                                     x[0] + (size_t)t * n * KT, pt);
    if (opt.rhs)
      ppr_load_kernel<T, KT><<<grid_in, 256, 0, s>>>(n, opt.rhs, d_vec + (size_t)t * KT, newid_dev, dmask,
                                                     rhs_t[0] + (size_t)t * n * KT, nullptr);
    ppr_finalize_kernel<KT><<<1, 32, 0, s>>>(pt, grid_in, d_col + (size_t)t * KT, d_tile + t, beta, cst,
                                             p->max_iter, std::min(KT, k - t * KT), 1);
  }
  int rbase = 0;  // rhs_t[rbase] holds the current layout's right-hand side
  if (cudaGetLastError() != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank init"); }
  // Sweeps in rounds of K on every tile of the current layout (stopped tiles
  // return at once).  After each round the vectors that stopped are written
  // out and dropped; when the live vectors fit in fewer tiles they are
  // repacked (compaction), so a tile never keeps sweeping for one slow
  // vector while its other lanes idle.  All tiles of a layout sweep in step:
  // the layout's iterates start in x[base] and sweep j reads x[(base+j)&1].
  const int K = p->check_every > 0 ? p->check_every : 4;  // 4: R-MAT 2^22, 256 vectors, 3-9 % faster than 8
  int cur_tiles = tiles, base = 0;
  std::vector<int> slot_vec((size_t)tiles * KT, -1);  // vector in each slot, -1 for none
  for (int c = 0; c < k; ++c) slot_vec[(size_t)c] = c;
  std::vector<TileCtl> htc((size_t)tiles);
  std::vector<ColCtl> hcc((size_t)tiles * KT);
  int *d_map = nullptr;
  alloc((void **)&d_map, (size_t)tiles * KT * sizeof(int));
  if (st != TBSLA_OK) { cleanup(); return st; }
  std::vector<char> tile_live((size_t)tiles, 1);
  int phase = 0;
  while (true) {
    for (int k2 = 0; k2 < K; ++k2, ++phase) {
      for (int t = 0; t < cur_tiles; ++t) {
        if (!tile_live[(size_t)t]) continue;  // stopped in an earlier round
        const T *xo = x[(base + phase) & 1] + (size_t)t * n * KT;
        T *xn = x[(base + phase + 1) & 1] + (size_t)t * n * KT;
        double *pt = partials + (size_t)t * nparts * KT * 2;
        const unsigned *sd = d_seeds + (size_t)t * n;
        const ColCtl *cl = d_col + (size_t)t * KT;
        const double *iv = d_inv + (size_t)t * KT;
        const T *rh = opt.rhs ? rhs_t[rbase] + (size_t)t * n * KT : nullptr;
        ppr_spmm_kernel<T, KT><<<grid_mm, 256, 0, s>>>(d_items, (int)items.size(), M->idx1, values, xo, xn, sd,
                                                       dmask, cl, iv, beta, rh, chunk, pt, d_tile + t);
        if (n_crow)
          ppr_fixup_kernel<T, KT><<<grid_fx, 256, 0, s>>>(d_crow, n_crow, chunk, xo, xn, sd, dmask, cl, iv, beta,
                                                          rh, pt, grid_mm, d_tile + t);
        ppr_finalize_kernel<KT><<<1, 32, 0, s>>>(pt, n_crow ? grid_mm + grid_fx : grid_mm, d_col + (size_t)t * KT,
                                                 d_tile + t, beta, cst, p->max_iter, KT, 0);
      }
    }
    if (cudaMemcpyAsync(htc.data(), d_tile, (size_t)cur_tiles * sizeof(TileCtl), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(hcc.data(), d_col, (size_t)cur_tiles * KT * sizeof(ColCtl), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      cleanup();
      return fail(TBSLA_ERR_CUDA, "batched PageRank sweeps failed");
    }
    // write out and drop the vectors that stopped (a stopped vector is
    // frozen: its tile's last iterate, x[(base + tile iter) & 1], holds it;
    // a stopped tile's vectors have all stopped, or max_iter is 0)
    int live = 0, busy = 0;
    for (int t = 0; t < cur_tiles; ++t) {
      PprPicks pk;
      pk.cnt = 0;
      for (int c = 0; c < KT; ++c) {
        const int v = slot_vec[(size_t)t * KT + c];
        if (v < 0) continue;
        const ColCtl &cc = hcc[(size_t)t * KT + c];
        if (cc.done || htc[(size_t)t].done) {
          pk.col[pk.cnt] = c;
          pk.vec[pk.cnt++] = v;
          if (iters_out) iters_out[v] = cc.iter;
          if (resid_out) resid_out[v] = cc.resid;
          slot_vec[(size_t)t * KT + c] = -1;
        } else {
          ++live;
        }
      }
      if (pk.cnt) {
        const T *xf = x[(base + htc[(size_t)t].iter) & 1] + (size_t)t * n * KT;
        ppr_pick_kernel<T, KT><<<152 * 8, 256, 0, s>>>(xf, n, newid_dev, pk, d_out);
      }
      tile_live[(size_t)t] = !htc[(size_t)t].done;
      busy += !htc[(size_t)t].done;
    }
    if (cudaGetLastError() != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank results"); }
    if (live == 0) break;
    const int need = (live + KT - 1) / KT;
    if (need < busy) {
      // repack the live vectors into `need` tiles: their iterates (all in
      // x[(base+phase)&1], every live tile having run all `phase` sweeps)
      // move to the other buffer, which becomes the new layout's start
      std::vector<int> map((size_t)need * KT, -1), nvec((size_t)need * KT, -1);
      std::vector<unsigned> nseeds((size_t)need * n, 0u);
      std::vector<double> ninv((size_t)need * KT, 0.0);
      std::vector<ColCtl> ncol((size_t)need * KT);
      int q = 0;
      for (int t = 0; t < cur_tiles; ++t)
        for (int c = 0; c < KT; ++c) {
          const int v = slot_vec[(size_t)t * KT + c];
          if (v < 0) continue;
          map[(size_t)q] = t * KT + c;
          nvec[(size_t)q] = v;
          ncol[(size_t)q] = hcc[(size_t)t * KT + c];
          ninv[(size_t)q] = inv[(size_t)t * KT + c];
          for (int u : seed_sets[(size_t)v]) nseeds[(size_t)(q / KT) * n + u] |= 1u << (q % KT);
          ++q;
        }
      for (size_t r = (size_t)q; r < ncol.size(); ++r) ncol[r] = ColCtl{0.0, 0.0, 0.0, 0, 1};
      std::vector<TileCtl> ntile((size_t)need, TileCtl{0, 0, {0, 0}});
      up(d_map, map.data(), map.size() * sizeof(int));
      up(d_seeds, nseeds.data(), nseeds.size() * sizeof(unsigned));
      up(d_inv, ninv.data(), ninv.size() * sizeof(double));
      up(d_col, ncol.data(), ncol.size() * sizeof(ColCtl));
      up(d_tile, ntile.data(), ntile.size() * sizeof(TileCtl));
      if (e != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank repack: %s", cudaGetErrorString(e)); }
      const int src = (base + phase) & 1;
      ppr_move_kernel<T, KT><<<152 * 8, 256, 0, s>>>(x[src], x[src ^ 1], n, d_map, need);
      if (opt.rhs) {
        ppr_move_kernel<T, KT><<<152 * 8, 256, 0, s>>>(rhs_t[rbase], rhs_t[rbase ^ 1], n, d_map, need);
        rbase ^= 1;
      }
      if (cudaGetLastError() != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank repack"); }
      base = src ^ 1;
      phase = 0;
      cur_tiles = need;
      slot_vec = nvec;
      inv = ninv;
      std::fill(tile_live.begin(), tile_live.end(), 1);
    }
  }
  if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    cleanup();
    return fail(TBSLA_ERR_CUDA, "batched PageRank results");
  }
  cleanup();
  return TBSLA_OK;
}

__global__ void ppr_sub_kernel(double *__restrict__ g, const double *__restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    g[i] -= x[i];
}
__global__ void ppr_add_kernel(double *__restrict__ x, const double *__restrict__ e, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += e[i];
}

// FP32 sweeps with FP64 defect correction (tbsla_ppr_batched_refined):
// x = the FP32 solve; then rounds of r = G(x) - x by one FP64 sweep of every
// vector, stopping when every ||r_c||_1 < tol (the result is G(x)), else the
// FP32 correction solve e = beta A e + beta (d.e) v_c + r_c from e = r_c to
// ||e_j+1 - e_j||_1 < eta ||r_c||_1, and x += e.  Iterations: FP32 and FP64
// sweeps together.
constexpr double kRefineEta = 1e-3;     // inner tolerance relative to ||r_c||_1
constexpr double kF32SolveFloor = 1e-6; // the FP32 solve's stopping threshold at least this
constexpr int kRefineRounds = 8;

template <int KT>
tbsla_status_t run_refined(const tbsla_matrix *M, const int *nd, const std::vector<int> *nh,
                           const tbsla_pagerank_params_t *p, int k, const int *nodes, const int *offsets,
                           double *d_out, int *iters_out, double *resid_out, cudaStream_t s) {
  const int64_t n = M->n_row, total = n * k;
  std::vector<int> itot((size_t)k), it((size_t)k);
  std::vector<double> res((size_t)k, 0.0), tolc((size_t)k);
  tbsla_pagerank_params_t q = *p;
  q.tol = std::max(p->tol, kF32SolveFloor);
  TB_TRY((run_tiles<float, KT>(M, nd, nh, &q, k, nodes, offsets, d_out, itot.data(), nullptr, s)));
  double *g = nullptr, *e = nullptr;
  TB_CUDA(cudaMallocAsync((void **)&g, (size_t)total * sizeof(double), s));
  if (cudaMallocAsync((void **)&e, (size_t)total * sizeof(double), s) != cudaSuccess) {
    cudaGetLastError();
    cudaFreeAsync(g, s);
    return fail(TBSLA_ERR_OOM, "refinement buffers (2 x %lld doubles)", (long long)total);
  }
  struct Free {
    cudaStream_t s;
    double *a, *b;
    ~Free() {
      cudaFreeAsync(a, s);
      cudaFreeAsync(b, s);
      cudaStreamSynchronize(s);
    }
  } release{s, g, e};
  const int grid = 152 * 8;
  for (int round = 0;; ++round) {
    // r = G(x) - x: one FP64 sweep from x (the sweep's L1 change is ||r_c||_1)
    tbsla_pagerank_params_t q64 = *p;
    q64.max_iter = 1;
    RunOpts o64;
    o64.x0 = d_out;
    TB_TRY((run_tiles<double, KT>(M, nd, nh, &q64, k, nodes, offsets, g, nullptr, res.data(), s, o64)));
    bool all = true;
    for (int c = 0; c < k; ++c) {
      itot[(size_t)c] += 1;
      all = all && res[(size_t)c] < p->tol;
    }
    if (all || round == kRefineRounds) {
      TB_CUDA(cudaMemcpyAsync(d_out, g, (size_t)total * sizeof(double), cudaMemcpyDeviceToDevice, s));
      break;
    }
    ppr_sub_kernel<<<grid, 256, 0, s>>>(g, d_out, total);
    TB_CUDA(cudaGetLastError());
    // the correction, only as far as each vector still needs it
    for (int c = 0; c < k; ++c)
      tolc[(size_t)c] = res[(size_t)c] < p->tol ? HUGE_VAL : kRefineEta * res[(size_t)c];
    RunOpts oc;
    oc.x0 = g;
    oc.rhs = g;
    oc.cst = 0.0;
    oc.tol = tolc.data();
    TB_TRY((run_tiles<float, KT>(M, nd, nh, p, k, nodes, offsets, e, it.data(), nullptr, s, oc)));
    for (int c = 0; c < k; ++c) itot[(size_t)c] += it[(size_t)c];
    ppr_add_kernel<<<grid, 256, 0, s>>>(d_out, e, total);
    TB_CUDA(cudaGetLastError());
  }
  TB_CUDA(cudaStreamSynchronize(s));
  for (int c = 0; c < k; ++c) {
    if (iters_out) iters_out[c] = itot[(size_t)c];
    if (resid_out) resid_out[c] = res[(size_t)c];
  }
  return TBSLA_OK;
}

template <typename T>
tbsla_status_t run_kt(int kt, const tbsla_matrix *M, const int *nd, const std::vector<int> *nh,
                      const tbsla_pagerank_params_t *p, int k, const int *nodes, const int *offsets, double *out,
                      int *it, double *rs, cudaStream_t s) {
  switch (kt) {
  case 2: return run_tiles<T, 2>(M, nd, nh, p, k, nodes, offsets, out, it, rs, s);
  case 4: return run_tiles<T, 4>(M, nd, nh, p, k, nodes, offsets, out, it, rs, s);
  case 8: return run_tiles<T, 8>(M, nd, nh, p, k, nodes, offsets, out, it, rs, s);
  case 16: return run_tiles<T, 16>(M, nd, nh, p, k, nodes, offsets, out, it, rs, s);
  default: return run_tiles<T, 32>(M, nd, nh, p, k, nodes, offsets, out, it, rs, s);
  }
}

}  // namespace
}  // namespace tbsla

using namespace tbsla;

static tbsla_status_t ppr_batched(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p, int k,
                                  const int *nodes, const int *offsets, int tile, double *d_out, int *iterations,
                                  double *residuals, void *stream, bool refined) {
  TB_CHECK(A && p && nodes && offsets && d_out, "NULL argument");
  TB_CHECK(k > 0, "k = %d", k);
  TB_CHECK(A->format == TBSLA_FMT_CSR, "batched PageRank needs a CSR handle");
  TB_CHECK(A->n_row == A->n_col && A->rows == A->n_row && A->f_col == 0, "batched PageRank needs a square graph");
  TB_CHECK(p->precision == TBSLA_F64 || p->precision == TBSLA_F32, "precision must be TBSLA_F64 or TBSLA_F32");
  TB_CHECK(tile == 0 || tile == 2 || tile == 4 || tile == 8 || tile == 16 || tile == 32,
           "tile %d not 0, 2, 4, 8, 16 or 32", tile);
  TB_CUDA(cudaSetDevice(A->device));
  tbsla_matrix *M = const_cast<tbsla_matrix *>(A);
  tbsla_matrix *B = nullptr;
  TB_TRY(pr_relabelled(M, &B));
  const int *nd = B ? M->pr_newid : nullptr;
  const std::vector<int> *nh = B ? &M->pr_newid_host : nullptr;
  const tbsla_matrix *R = B ? B : M;
  const int tuned = M->ppr_tile[p->precision == TBSLA_F64 ? 0 : 1];
  // default: the widest tile the vectors fill (wide tiles stream the matrix
  // fewer times per vector: R-MAT 2^22, 256 vectors, FP64 ms per vector 15.8 /
  // 10.5 / 9.7 / 9.3 / 8.5 for tiles 2 / 4 / 8 / 16 / 32)
  const int kt = tile ? tile : tuned ? tuned : (k >= 32 ? 32 : k >= 16 ? 16 : k >= 8 ? 8 : k >= 4 ? 4 : 2);
  cudaStream_t s = (cudaStream_t)stream;
  if (refined) {
    TB_CHECK(p->precision == TBSLA_F32, "the refined batched solve takes TBSLA_F32");
    TB_CHECK(R->values[0] && R->values[1], "the refined batched solve needs the F64 and F32 value stores");
    switch (kt) {
    case 2: return run_refined<2>(R, nd, nh, p, k, nodes, offsets, d_out, iterations, residuals, s);
    case 4: return run_refined<4>(R, nd, nh, p, k, nodes, offsets, d_out, iterations, residuals, s);
    case 8: return run_refined<8>(R, nd, nh, p, k, nodes, offsets, d_out, iterations, residuals, s);
    case 16: return run_refined<16>(R, nd, nh, p, k, nodes, offsets, d_out, iterations, residuals, s);
    default: return run_refined<32>(R, nd, nh, p, k, nodes, offsets, d_out, iterations, residuals, s);
    }
  }
  if (p->precision == TBSLA_F64) return run_kt<double>(kt, R, nd, nh, p, k, nodes, offsets, d_out, iterations, residuals, s);
  return run_kt<float>(kt, R, nd, nh, p, k, nodes, offsets, d_out, iterations, residuals, s);
}

extern "C" tbsla_status_t tbsla_ppr_batched(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p, int k,
                                            const int *nodes, const int *offsets, int tile, double *d_out,
                                            int *iterations, double *residuals, void *stream) {
  return ppr_batched(A, p, k, nodes, offsets, tile, d_out, iterations, residuals, stream, false);
}

extern "C" tbsla_status_t tbsla_ppr_batched_refined(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p,
                                                    int k, const int *nodes, const int *offsets, int tile,
                                                    double *d_out, int *iterations, double *residuals,
                                                    void *stream) {
  return ppr_batched(A, p, k, nodes, offsets, tile, d_out, iterations, residuals, stream, true);
}
