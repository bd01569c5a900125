// ppr_batch.cu -- many personalized PageRank vectors of one graph solved
// together (TBSLA_PR_TELEPORT form, one teleport set per vector).
//
// The k iterates are kept in tiles of KT columns (KT = 2, 4, 8, 16 or 32), each
// tile row-major: tile t, row i holds X[i*KT + c] for its KT vectors, so the
// gather of a column index brings all KT values in one contiguous segment.
// A group of G lanes sums a row, each lane VW consecutive vectors (16 bytes
// of the tile row): no cross-lane reduction, every lane does useful
// multiply-adds, and a warp sweeps 32 / G rows at once.  Rows longer than
// kPprChunk entries are cut into chunks (partials + a fixup kernel) so that
// hub rows of power-law graphs spread over many groups.  The FP64 sweeps are
// bound by the FP64 pipe (2 operations per clock per SM): a 32-vector sweep
// of R-MAT 2^20 (5.2e8 FMAs and the epilogue's FP64 work) keeps it 90 % busy
// while DRAM runs at 10 %.
//
// Anderson acceleration (p->accel = 1), per vector as in the one-vector
// solve: the sweep writes its output g and residual r = g - x into rings of
// three slots and sums r's dots with the two previous residuals; the
// finalize solves each vector's 3x3 normal equations (aa_coefficients) and
// the next input is the combination of the last three outputs.
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

#include "anderson.cuh"
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
  int ran;         // the last sweep ran on the tile (it was not stopped before)
  int pad;
};
// Anderson state of a column (accelerated solves): the next-sweep terms of
// the last three outputs and their residuals' Gram matrix, newest first; the
// weights of the next input in those outputs; residuals stored so far (0-3)
struct ColAa {
  double add[3];
  double gram[3][3];
  double coef[3];
  int hist, m;
};

// Lanes of the sweep kernels: each lane carries VW consecutive vectors (16
// bytes of a tile row, or the whole row when it is narrower), so a row takes
// G = KT / VW lanes and a warp sweeps 32 / G rows at once.
template <typename T, int KT>
struct PprLanes {
  static constexpr int VW = KT * (int)sizeof(T) >= 16 ? 16 / (int)sizeof(T) : KT;
  static constexpr int G = KT / VW;
};
template <typename T, int VW> struct PprVec;
template <> struct PprVec<double, 2> { using type = double2; };
template <> struct PprVec<float, 2> { using type = float2; };
template <> struct PprVec<float, 4> { using type = float4; };

template <typename T, int VW>
__device__ __forceinline__ void ppr_ld(const T *p, T (&v)[VW]) {
  using V = typename PprVec<T, VW>::type;
  const V q = __ldg(reinterpret_cast<const V *>(p));
  const T *s = reinterpret_cast<const T *>(&q);
  #pragma unroll
  for (int i = 0; i < VW; ++i) v[i] = s[i];
}
template <typename T, int VW>
__device__ __forceinline__ void ppr_st(T *p, const T (&v)[VW]) {
  using V = typename PprVec<T, VW>::type;
  V q;
  T *d = reinterpret_cast<T *>(&q);
  #pragma unroll
  for (int i = 0; i < VW; ++i) d[i] = v[i];
  *reinterpret_cast<V *>(p) = q;
}

// Per-column sums of a block into partials[(part*KT + c)*NV + v], for the NV
// values (resid, dangling mass, and with acceleration the residual dots
// r.r, r.r_prev, r.r_prev2) that each lane holds for its VW columns (lane l
// of a row group: columns l*VW .. l*VW+VW-1).  The warp's row groups are
// summed by shuffles, then the warps in order.
template <int KT, int VW, int NV>
__device__ __forceinline__ void block_columns(double (&v)[NV][VW], double *partials, int part) {
  constexpr int G = KT / VW;
  __shared__ double sh[8][32][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  #pragma unroll
  for (int o = 16; o >= G; o >>= 1) {
    #pragma unroll
    for (int j = 0; j < NV; ++j)
      #pragma unroll
      for (int q = 0; q < VW; ++q) v[j][q] += __shfl_down_sync(0xffffffffu, v[j][q], o);
  }
  if (lane < G) {
    #pragma unroll
    for (int j = 0; j < NV; ++j)
      #pragma unroll
      for (int q = 0; q < VW; ++q) sh[warp][lane * VW + q][j] = v[j][q];
  }
  __syncthreads();
  if (threadIdx.x < KT) {
    double a[NV];
    #pragma unroll
    for (int j = 0; j < NV; ++j) a[j] = 0;
    const int nw = blockDim.x >> 5;
    for (int w = 0; w < nw; ++w)
      #pragma unroll
      for (int j = 0; j < NV; ++j) a[j] += sh[w][threadIdx.x][j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) partials[((size_t)part * KT + threadIdx.x) * NV + j] = a[j];
  }
}

// the residual ring of an accelerated sweep: r0 receives r = y - x, r1 / r2
// hold the previous two sweeps' residuals
template <typename T>
struct PprRing {
  T *r0;
  const T *r1, *r2;
};

// A sweep's per-column constants for one lane's VW columns
template <int VW>
struct PprCols {
  double tele[VW];  // teleport term added at seed rows
  float tele_f[VW];  // the same rounded to FP32 (FP32 tiles)
  bool stopped[VW];
  int hist[VW];  // accelerated: residuals stored before this sweep
};
template <int VW, bool AA>
__device__ __forceinline__ void ppr_cols(PprCols<VW> &pc, int c, const ColCtl *col, const double *inv_size,
                                         const ColAa *aa) {
  #pragma unroll
  for (int q = 0; q < VW; ++q) {
    const ColCtl cc = col[c + q];
    pc.stopped[q] = cc.done != 0;
    pc.tele[q] = cc.add * inv_size[c + q];
    pc.tele_f[q] = (float)pc.tele[q];
    pc.hist[q] = AA ? aa[c + q].hist : 0;
  }
}

// The loads of a row's epilogue
template <typename T, int VW, bool AA>
struct PprRowIn {
  T old[VW], rh[VW], r1[VW], r2[VW];
  unsigned sd;
  bool dm;
};
template <typename T, int VW, bool AA>
__device__ __forceinline__ void ppr_row_in(PprRowIn<T, VW, AA> &in, int row, int KT, int c, const PprCols<VW> &pc,
                                           const T *xo, const unsigned *seeds, const unsigned char *dmask,
                                           const T *rhs, const PprRing<T> &ring) {
  const size_t at = (size_t)row * KT + c;
  ppr_ld<T, VW>(xo + at, in.old);
  if (rhs) ppr_ld<T, VW>(rhs + at, in.rh);
  in.sd = __ldg(seeds + row) >> c;
  in.dm = __ldg(dmask + row) != 0;
  if constexpr (AA) {
    int h = 0;
    #pragma unroll
    for (int q = 0; q < VW; ++q) h = max(h, pc.hist[q]);
    if (h >= 1) ppr_ld<T, VW>(ring.r1 + at, in.r1);
    if (h >= 2) ppr_ld<T, VW>(ring.r2 + at, in.r2);
  }
}

// New values of one finished row for a lane's VW columns:
//   y = beta acc + [seed row] tele + rhs (a stopped column keeps its value),
// their L1 change (res) and dangling mass (dm, FP64: it sets the next
// sweep's teleport term, so the fixed point); accelerated: r = y - x into
// the ring and its dots with the previous residuals, summed per thread in
// shared memory (dots[(j*VW + q)*256 + thread]: registers are the sweep's
// limit).  FP32 tiles compute y, the L1 change and the dots in FP32 (the
// per-thread sums cover a few hundred rows; the block and grid sums are
// FP64): the FP64 pipe, two operations per clock per SM, is kept for the
// dangling mass.
template <typename T, int VW, bool AA>
__device__ __forceinline__ void ppr_emit(int row, int KT, int c, const T (&acc)[VW], const PprCols<VW> &pc,
                                         const PprRowIn<T, VW, AA> &in, T *xn, double beta, bool has_rhs,
                                         const PprRing<T> &ring, T (&res)[VW], double (&dm)[VW], T *dots) {
  const size_t at = (size_t)row * KT + c;
  T y[VW];
  #pragma unroll
  for (int q = 0; q < VW; ++q) {
    if (pc.stopped[q]) {
      y[q] = in.old[q];
    } else {
      if constexpr (std::is_same<T, float>::value) {
        float t = ((in.sd >> q) & 1u) ? pc.tele_f[q] : 0.f;
        if (has_rhs) t += in.rh[q];
        y[q] = fmaf((float)beta, acc[q], t);
        res[q] += fabsf(y[q] - in.old[q]);
      } else {
        double t = ((in.sd >> q) & 1u) ? pc.tele[q] : 0.0;
        if (has_rhs) t += (double)in.rh[q];
        y[q] = (T)((double)beta * (double)acc[q] + t);
        res[q] += fabs((double)y[q] - (double)in.old[q]);
      }
    }
    if (in.dm) dm[q] += (double)y[q];
  }
  ppr_st<T, VW>(xn + at, y);
  if constexpr (AA) {
    T r[VW];
    #pragma unroll
    for (int q = 0; q < VW; ++q) r[q] = y[q] - in.old[q];
    ppr_st<T, VW>(ring.r0 + at, r);
    #pragma unroll
    for (int q = 0; q < VW; ++q) {
      T *dq = dots + (size_t)q * 256 + threadIdx.x;
      dq[0] += r[q] * r[q];
      if (pc.hist[q] >= 1) dq[VW * 256] += r[q] * in.r1[q];
      if (pc.hist[q] >= 2) dq[2 * VW * 256] += r[q] * in.r2[q];
    }
  }
}

// the per-thread sums of a sweep kernel in the layout of block_columns
template <typename T, int VW, int NV, bool AA>
__device__ __forceinline__ void ppr_gather_parts(const T (&res)[VW], const double (&dm)[VW], const T *dots,
                                                 double (&part)[NV][VW]) {
  #pragma unroll
  for (int q = 0; q < VW; ++q) {
    part[0][q] = (double)res[q];
    part[1][q] = dm[q];
  }
  if constexpr (AA)
    #pragma unroll
    for (int j = 0; j < 3; ++j)
      #pragma unroll
      for (int q = 0; q < VW; ++q) part[2 + j][q] = (double)dots[(j * VW + q) * 256 + threadIdx.x];
}

// Resident blocks per SM the sweep kernel is compiled for (its register
// budget, 64 registers): the sweeps are bound by the latency of their
// gathers, and resident warps keep them in flight (R-MAT 2^22, 256 vectors,
// FP64: 1 block per SM (144 registers) 1.77x the time of 4; 5 no faster)
template <typename T, bool AA>
constexpr int ppr_min_blocks() {
  return 4;
}

// items: (row, begin, end, chunk slot or -1).  A row group of G lanes takes
// an item, lane l its vectors l*VW .. l*VW+VW-1 (one 16-byte gather of the
// tile row per entry); each vector's sum is one FMA per entry in stored order.
template <typename T, int KT, bool AA>
__global__ void __launch_bounds__(256, ppr_min_blocks<T, AA>()) ppr_spmm_kernel(const int4 *__restrict__ items, int n_items,
                                                      const int *__restrict__ colidx, const T *__restrict__ values,
                                                      const T *__restrict__ xo, T *__restrict__ xn,
                                                      const unsigned *__restrict__ seeds,
                                                      const unsigned char *__restrict__ dmask,
                                                      const ColCtl *__restrict__ col, const ColAa *__restrict__ aa,
                                                      const double *__restrict__ inv_size, double beta,
                                                      const T *__restrict__ rhs, PprRing<T> ring,
                                                      T *__restrict__ chunk_partials, double *partials,
                                                      const TileCtl *tile) {
  if (*(volatile const int *)&tile->done) return;
  constexpr int VW = PprLanes<T, KT>::VW, G = PprLanes<T, KT>::G, NV = AA ? 5 : 2;
  const int c = (threadIdx.x & (G - 1)) * VW;  // first vector of this lane
  PprCols<VW> pc;
  ppr_cols<VW, AA>(pc, c, col, inv_size, aa);
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
  T res[VW];
  double dm[VW];
  #pragma unroll
  for (int q = 0; q < VW; ++q) {
    res[q] = 0;
    dm[q] = 0;
  }
  __shared__ T dots[AA ? 3 * VW * 256 : 1];
  if (AA)
    for (int j = 0; j < 3 * VW; ++j) dots[j * 256 + threadIdx.x] = 0;
  for (int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; g < n_items; g += ng) {
    const int4 it = items[g];
    T acc[VW];
    #pragma unroll
    for (int q = 0; q < VW; ++q) acc[q] = 0;
    // four entries per step, the last step predicated: a short row's
    // gathers are all issued before its first multiply-add (R-MAT rows are
    // mostly short, and one entry at a time chains index -> gather -> FMA)
    for (int e = it.y; e < it.z; e += 4) {
      const int rem = it.z - e;
      int cj[4];
      T vj[4], xj[4][VW];
      #pragma unroll
      for (int u = 0; u < 4; ++u) {
        cj[u] = u < rem ? __ldg(colidx + e + u) : 0;
        vj[u] = u < rem ? __ldg(values + e + u) : T(0);
      }
      #pragma unroll
      for (int u = 0; u < 4; ++u)
        if (u < rem) ppr_ld<T, VW>(xo + (size_t)cj[u] * KT + c, xj[u]);
      #pragma unroll
      for (int u = 0; u < 4; ++u)
        if (u < rem)
          #pragma unroll
          for (int q = 0; q < VW; ++q) acc[q] = fma(vj[u], xj[u][q], acc[q]);
    }
    if (it.w >= 0) {
      ppr_st<T, VW>(chunk_partials + (size_t)it.w * KT + c, acc);
    } else {
      PprRowIn<T, VW, AA> in;
      ppr_row_in<T, VW, AA>(in, it.x, KT, c, pc, xo, seeds, dmask, rhs, ring);
      ppr_emit<T, VW, AA>(it.x, KT, c, acc, pc, in, xn, beta, rhs != nullptr, ring, res, dm, dots);
    }
  }
  double part[NV][VW];
  ppr_gather_parts<T, VW, NV, AA>(res, dm, dots, part);
  block_columns<KT, VW, NV>(part, partials, blockIdx.x);
}

// rows cut into chunks: crow[h] = (row, first slot), crow[n].y = total slots;
// the chunks' sums are added in order
template <typename T, int KT, bool AA>
__global__ void __launch_bounds__(256) ppr_fixup_kernel(const int2 *__restrict__ crow, int n_crow,
                                                       const T *__restrict__ chunk_partials,
                                                       const T *__restrict__ xo, T *__restrict__ xn,
                                                       const unsigned *__restrict__ seeds,
                                                       const unsigned char *__restrict__ dmask,
                                                       const ColCtl *__restrict__ col, const ColAa *__restrict__ aa,
                                                       const double *__restrict__ inv_size, double beta,
                                                       const T *__restrict__ rhs, PprRing<T> ring, double *partials,
                                                       int part_base, const TileCtl *tile) {
  if (*(volatile const int *)&tile->done) return;
  constexpr int VW = PprLanes<T, KT>::VW, G = PprLanes<T, KT>::G, NV = AA ? 5 : 2;
  const int c = (threadIdx.x & (G - 1)) * VW;
  PprCols<VW> pc;
  ppr_cols<VW, AA>(pc, c, col, inv_size, aa);
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
  T res[VW];
  double dm[VW];
  #pragma unroll
  for (int q = 0; q < VW; ++q) {
    res[q] = 0;
    dm[q] = 0;
  }
  __shared__ T dots[AA ? 3 * VW * 256 : 1];
  if (AA)
    for (int j = 0; j < 3 * VW; ++j) dots[j * 256 + threadIdx.x] = 0;
  for (int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; g < n_crow; g += ng) {
    const int2 h = crow[g];
    T acc[VW];
    #pragma unroll
    for (int q = 0; q < VW; ++q) acc[q] = 0;
    for (int s = h.y; s < crow[g + 1].y; ++s) {
      T p[VW];
      ppr_ld<T, VW>(chunk_partials + (size_t)s * KT + c, p);
      #pragma unroll
      for (int q = 0; q < VW; ++q) acc[q] += p[q];
    }
    PprRowIn<T, VW, AA> in;
    ppr_row_in<T, VW, AA>(in, h.x, KT, c, pc, xo, seeds, dmask, rhs, ring);
    ppr_emit<T, VW, AA>(h.x, KT, c, acc, pc, in, xn, beta, rhs != nullptr, ring, res, dm, dots);
  }
  double part[NV][VW];
  ppr_gather_parts<T, VW, NV, AA>(res, dm, dots, part);
  block_columns<KT, VW, NV>(part, partials, part_base + blockIdx.x);
}

// per column: sum the parts in order, advance the column, then the tile.
// Accelerated: the new output's term and residual dots enter the column's
// history and the weights of the next input are solved (aa_coefficients); a
// column that stops takes its last output as it is.
// 1024 threads: warp w sums the parts w, w + 32, ... in order, its lanes
// reading each part's KT * NV values together; then the warps' sums are added
// in order, and one thread per column advances it.
template <int KT, bool AA>
__global__ void __launch_bounds__(1024) ppr_finalize_kernel(const double *__restrict__ partials, int nparts,
                                                           ColCtl *col, ColAa *aa, TileCtl *tile, double beta,
                                                           double cst, int max_iter, int k_in_tile, int first) {
  constexpr int NV = AA ? 5 : 2, W = KT * NV, PER = (W + 31) / 32;
  __shared__ double sh[32][W];
  __shared__ int active;
  if (threadIdx.x == 0) active = 0;
  __syncthreads();
  if (*(volatile int *)&tile->done) {
    if (threadIdx.x == 0) tile->ran = 0;
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double a[PER];
  #pragma unroll
  for (int i = 0; i < PER; ++i) a[i] = 0;
  #pragma unroll 4
  for (int p = warp; p < nparts; p += 32)
    #pragma unroll
    for (int i = 0; i < PER; ++i)
      if (lane + 32 * i < W) a[i] += partials[(size_t)p * W + lane + 32 * i];
  #pragma unroll
  for (int i = 0; i < PER; ++i)
    if (lane + 32 * i < W) sh[warp][lane + 32 * i] = a[i];
  __syncthreads();
  if (threadIdx.x < W) {
    double t = 0;
    for (int w = 0; w < 32; ++w) t += sh[w][threadIdx.x];
    sh[0][threadIdx.x] = t;  // read only by this thread above
  }
  __syncthreads();
  const int c = threadIdx.x;
  double v[NV];
  if (c < KT)
    #pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = sh[0][c * NV + j];
  if (c < KT) {
    const double r = v[0], d = v[1];
    ColCtl &cc = col[c];
    if (first) {
      cc.add = beta * d + cst;  // initial vector: only the dangling mass is new
    } else if (!cc.done) {
      cc.iter += 1;
      cc.resid = r;
      cc.add = beta * d + cst;
      cc.done = r < cc.tol || cc.iter >= max_iter;
      if constexpr (AA) {
        ColAa &st = aa[c];
        st.add[2] = st.add[1];
        st.add[1] = st.add[0];
        st.add[0] = beta * d + cst;
        aa_gram_push(st.gram, v[2], v[3], v[4]);
        st.hist = min(st.hist + 1, 3);
        if (cc.done) {
          st.coef[0] = 1.0;
          st.coef[1] = st.coef[2] = 0.0;
          st.m = 0;
        } else {
          st.m = aa_coefficients(st.gram, st.hist - 1, st.coef);
          double add = st.coef[0] * st.add[0];
          if (st.m >= 1) add += st.coef[1] * st.add[1];
          if (st.m >= 2) add += st.coef[2] * st.add[2];
          cc.add = add;
        }
      }
    } else {
      cc.add = beta * d + cst;
    }
    if (c < k_in_tile && !cc.done) atomicOr(&active, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!first) tile->iter += 1;
    tile->done = active == 0;
    tile->ran = 1;
  }
}

// accelerated: x = c0 g0 + c1 g1 + c2 g2 per column (g0 the newest output;
// only the terms in use are read), after every sweep that ran on the tile
// (also the one that stopped its last vector: x then takes its outputs)
template <typename T, int KT>
__global__ void __launch_bounds__(256) ppr_combine_kernel(int n, const T *__restrict__ g0,
                                                         const T *__restrict__ g1, const T *__restrict__ g2,
                                                         T *__restrict__ x, const ColAa *__restrict__ aa,
                                                         const TileCtl *tile) {
  if (!*(volatile const int *)&tile->ran) return;
  constexpr int VW = PprLanes<T, KT>::VW, G = PprLanes<T, KT>::G;
  const int c = (threadIdx.x & (G - 1)) * VW;
  T c0[VW], c1[VW], c2[VW];
  int m[VW], mm = 0;
  #pragma unroll
  for (int q = 0; q < VW; ++q) {
    const ColAa &st = aa[c + q];
    c0[q] = (T)st.coef[0];
    c1[q] = (T)st.coef[1];
    c2[q] = (T)st.coef[2];
    m[q] = st.m;
    mm = max(mm, m[q]);
  }
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; i < n; i += ng) {
    const size_t at = (size_t)i * KT + c;
    T a[VW], b[VW], e[VW], v[VW];
    ppr_ld<T, VW>(g0 + at, a);
    if (mm >= 1) ppr_ld<T, VW>(g1 + at, b);
    if (mm >= 2) ppr_ld<T, VW>(g2 + at, e);
    #pragma unroll
    for (int q = 0; q < VW; ++q) {
      v[q] = c0[q] * a[q];
      if (m[q] >= 1) v[q] = fma(c1[q], b[q], v[q]);
      if (m[q] >= 2) v[q] = fma(c2[q], e[q], v[q]);
    }
    ppr_st<T, VW>(x + at, v);
  }
}

// x0 = v (seeds), dangling mass of x0 per column (partials of NV values per
// column, the others 0)
template <typename T, int KT, int NV>
__global__ void __launch_bounds__(256) ppr_init_kernel(int n, const unsigned *__restrict__ seeds,
                                                      const unsigned char *__restrict__ dmask,
                                                      const double *__restrict__ inv_size, T *__restrict__ x,
                                                      double *partials) {
  const int c = threadIdx.x & (KT - 1);
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / KT;
  double part[NV][1] = {};
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / KT; i < n; i += ng) {
    const T v = ((seeds[i] >> c) & 1u) ? (T)inv_size[c] : T(0);
    x[(size_t)i * KT + c] = v;
    if (dmask[i]) part[1][0] += (double)v;
  }
  block_columns<KT, 1, NV>(part, partials, blockIdx.x);
}

// x (one tile) from FP64 vectors in the original labels: vector vec[c] of
// src (src + vec[c] * n) at tile row newid[u] (u when not relabelled);
// columns with vec[c] < 0 get 0.  With partials: the dangling mass per column.
template <typename T, int KT, int NV>
__global__ void __launch_bounds__(256) ppr_load_kernel(int n, const double *__restrict__ src,
                                                      const int *__restrict__ vec, const int *__restrict__ newid,
                                                      const unsigned char *__restrict__ dmask, T *__restrict__ x,
                                                      double *partials) {
  const int c = threadIdx.x & (KT - 1);
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / KT;
  const int v = vec[c];
  double part[NV][1] = {};
  for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / KT; u < n; u += ng) {
    const int i = newid ? newid[u] : (int)u;
    const T val = v >= 0 ? (T)src[(size_t)v * n + u] : T(0);
    x[(size_t)i * KT + c] = val;
    if (partials && dmask[i]) part[1][0] += (double)val;
  }
  if (partials) block_columns<KT, 1, NV>(part, partials, blockIdx.x);
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

// seeds[(slot / KT) * n + node] |= bit (slot % KT) for the (slot, node) pairs
// of the seed sets (the array zeroed before)
template <int KT>
__global__ void ppr_seed_bits_kernel(unsigned *seeds, int n, const int2 *__restrict__ pairs, int npairs) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npairs; i += gridDim.x * blockDim.x) {
    const int2 q = pairs[i];
    atomicOr(seeds + (size_t)(q.x / KT) * n + q.y, 1u << (q.x % KT));
  }
}

// The work list of a handle's batched sweeps: rows, and rows longer than
// kPprChunk entries cut into chunks; built once (it depends on the row
// structure only) and kept on the handle.
struct PprPlan {
  int4 *items = nullptr;  // (row, begin, end, chunk slot or -1)
  int2 *crow = nullptr;   // chunked rows: (row, first slot); crow[n_crow].y = slots
  int n_items = 0, n_crow = 0, slots = 0;
};
void ppr_plan_free(void *q) {
  PprPlan *P = static_cast<PprPlan *>(q);
  if (P->items) cudaFree(P->items);
  if (P->crow) cudaFree(P->crow);
  delete P;
}
tbsla_status_t ppr_plan(const tbsla_matrix *Mc, const PprPlan **out) {
  tbsla_matrix *M = const_cast<tbsla_matrix *>(Mc);
  if (M->ppr_plan) {
    *out = static_cast<const PprPlan *>(M->ppr_plan);
    return TBSLA_OK;
  }
  const int n = M->n_row;
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
  PprPlan *P = new PprPlan;
  P->n_items = (int)items.size();
  P->n_crow = (int)crow.size();
  P->slots = slots;
  crow.push_back(make_int2(-1, slots));
  if (cudaMalloc((void **)&P->items, std::max<size_t>(items.size(), 1) * sizeof(int4)) != cudaSuccess ||
      cudaMalloc((void **)&P->crow, crow.size() * sizeof(int2)) != cudaSuccess) {
    cudaGetLastError();
    ppr_plan_free(P);
    return fail(TBSLA_ERR_OOM, "batched PageRank work list");
  }
  if ((!items.empty() &&
       cudaMemcpy(P->items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess) ||
      cudaMemcpy(P->crow, crow.data(), crow.size() * sizeof(int2), cudaMemcpyHostToDevice) != cudaSuccess) {
    ppr_plan_free(P);
    return fail(TBSLA_ERR_CUDA, "batched PageRank work list upload");
  }
  M->ppr_plan = P;
  M->ppr_plan_free = ppr_plan_free;
  *out = P;
  return TBSLA_OK;
}

// Accelerated repacking, in place: destination tile t of buf takes, per
// column c, old slot map[c] (-1: zero).  The live vectors keep their order,
// so every source of tile t lies in tile t or later; with the destination
// tiles done in increasing order (one launch each) and the lanes of a warp
// reading all their rows' sources before any of them writes (a row's sources
// and destinations are in the same row, one warp's), nothing is overwritten
// before it is read.
template <typename T, int KT>
__global__ void __launch_bounds__(256) ppr_compact_kernel(T *buf, int n, const int *__restrict__ map, int t) {
  constexpr int VW = PprLanes<T, KT>::VW, G = PprLanes<T, KT>::G;
  const int c = (threadIdx.x & (G - 1)) * VW;
  int from[VW];
  #pragma unroll
  for (int q = 0; q < VW; ++q) from[q] = map[c + q];
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
  // warp-uniform loop: the warp's first row, then its lanes' rows
  for (int64_t i0 = ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / G; i0 < n; i0 += ng) {
    const int64_t i = i0 + (threadIdx.x & 31) / G;
    T v[VW];
    if (i < n) {
      #pragma unroll
      for (int q = 0; q < VW; ++q)
        v[q] = from[q] < 0 ? T(0) : buf[((size_t)(from[q] / KT) * n + i) * KT + (from[q] % KT)];
    }
    __syncwarp();
    if (i < n) ppr_st<T, VW>(buf + ((size_t)t * n + i) * KT + c, v);
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

// One batched solve in tiles of KT vectors; AA: Anderson-accelerated
// (p->accel).  Plain sweeps ping-pong between two iterate buffers per tile;
// accelerated ones read the iterate x, write the output g and residual r to
// slot j % 3 of their rings (j counting the solve's sweeps), and the
// combination of the last three outputs becomes the next x.
template <typename T, int KT, bool AA>
tbsla_status_t run_tiles_impl(const tbsla_matrix *M, const int *newid_dev, const std::vector<int> *newid_host,
                              const tbsla_pagerank_params_t *p, int k, const int *nodes, const int *offsets,
                              double *d_out, int *iters_out, double *resid_out, cudaStream_t s, const RunOpts &opt) {
  constexpr int NV = AA ? 5 : 2;
  constexpr int G = PprLanes<T, KT>::G;
  const int n = M->n_row;
  const int64_t nnz = M->stored;
  const T *values = static_cast<const T *>(M->values[std::is_same<T, double>::value ? 0 : 1]);
  TB_CHECK(values, "the matrix lacks the %s value store", std::is_same<T, double>::value ? "F64" : "F32");
  const int tiles = (k + KT - 1) / KT;
  const PprPlan *plan = nullptr;
  TB_TRY(ppr_plan(M, &plan));
  const int n_crow = plan->n_crow, slots = plan->slots;
  // seeds: bit c of seeds[t*n + i] = row i is a seed of vector t*KT + c, set
  // on the device from the (slot, node) pairs
  std::vector<int2> pairs;
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
    for (int v : dist) pairs.push_back(make_int2(c, v));
    inv[(size_t)c] = 1.0 / (double)dist.size();
  }
  // the sweep grid: two waves of the blocks that fit on the GPU at once (a
  // grid-stride loop; one wave leaves SMs idle in its tail, more waves give
  // the finalize more per-block partials to add: R-MAT 2^20, 64 vectors,
  // 16 waves 1.47 ms per sweep + 0.75 ms finalize, 1 wave 1.58 + 0.05)
  int sms = 0, per_sm = 0;
  TB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, M->device));
  TB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ppr_spmm_kernel<T, KT, AA>, 256, 0));
  const int grid_mm = std::max(1, 2 * sms * std::max(per_sm, 1));
  const int grid_fx = std::max(1, std::min((n_crow * G + 255) / 256, sms * 4));
  const int grid_in = 152 * 4;
  const int grid_vec = 152 * 8;  // streaming passes over a tile (combine, compaction)
  const int nparts = std::max(grid_mm + grid_fx, grid_in);
  // device buffers
  const size_t xbytes = (size_t)n * KT * sizeof(T);
  T *x[2] = {nullptr, nullptr};
  T *g_ring[3] = {nullptr, nullptr, nullptr}, *r_ring[3] = {nullptr, nullptr, nullptr};
  T *chunk = nullptr;
  unsigned *d_seeds = nullptr;
  int2 *d_pairs = nullptr;
  unsigned char *dmask = nullptr;
  double *d_inv = nullptr, *partials = nullptr;
  ColCtl *d_col = nullptr;
  ColAa *d_aa = nullptr;
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
  if (AA) {
    for (int j = 0; j < 3; ++j) {
      alloc((void **)&g_ring[j], (size_t)tiles * xbytes);
      alloc((void **)&r_ring[j], (size_t)tiles * xbytes);
    }
  } else {
    alloc((void **)&x[1], (size_t)tiles * xbytes);
  }
  alloc((void **)&chunk, (size_t)std::max(slots, 1) * KT * sizeof(T));
  alloc((void **)&d_seeds, (size_t)tiles * n * sizeof(unsigned));
  alloc((void **)&d_pairs, pairs.size() * sizeof(int2));
  alloc((void **)&dmask, (size_t)n);
  alloc((void **)&d_inv, inv.size() * sizeof(double));
  alloc((void **)&partials, (size_t)tiles * nparts * KT * NV * sizeof(double));
  alloc((void **)&d_col, (size_t)tiles * KT * sizeof(ColCtl));
  alloc((void **)&d_aa, (size_t)tiles * KT * sizeof(ColAa));
  alloc((void **)&d_tile, (size_t)tiles * sizeof(TileCtl));
  alloc((void **)&d_vec, (size_t)tiles * KT * sizeof(int));
  if (opt.rhs) {
    alloc((void **)&rhs_t[0], (size_t)tiles * xbytes);
    if (!AA) alloc((void **)&rhs_t[1], (size_t)tiles * xbytes);
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
  // no history; the plain step
  ColAa aa0;
  std::memset(&aa0, 0, sizeof(aa0));
  aa0.coef[0] = 1.0;
  std::vector<ColAa> haa((size_t)tiles * KT, aa0);
  std::vector<TileCtl> htile((size_t)tiles, TileCtl{0, 0, 0, 0});
  if (p->max_iter == 0)
    for (auto &tc : htile) tc.done = 1;
  cudaError_t e = cudaSuccess;
  auto up = [&](void *d, const void *h, size_t b) {
    if (e == cudaSuccess && b) e = cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, s);
  };
  up(d_pairs, pairs.data(), pairs.size() * sizeof(int2));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_seeds, 0, (size_t)tiles * n * sizeof(unsigned), s);
  if (e == cudaSuccess)
    ppr_seed_bits_kernel<KT><<<152, 256, 0, s>>>(d_seeds, n, d_pairs, (int)pairs.size());
  up(d_inv, inv.data(), inv.size() * sizeof(double));
  up(d_col, hcol.data(), hcol.size() * sizeof(ColCtl));
  up(d_aa, haa.data(), haa.size() * sizeof(ColAa));
  up(d_tile, htile.data(), htile.size() * sizeof(TileCtl));
  up(d_vec, hvec.data(), hvec.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(dmask, 1, (size_t)n, s);
  if (e != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank upload: %s", cudaGetErrorString(e)); }
  ppr_dangling_kernel<T><<<152 * 8, 256, 0, s>>>(M->idx1, values, nnz, dmask);
  const double beta = p->beta;
  for (int t = 0; t < tiles; ++t) {
    double *pt = partials + (size_t)t * nparts * KT * NV;
    if (opt.x0)
      ppr_load_kernel<T, KT, NV><<<grid_in, 256, 0, s>>>(n, opt.x0, d_vec + (size_t)t * KT, newid_dev, dmask,
                                                         x[0] + (size_t)t * n * KT, pt);
    else
      ppr_init_kernel<T, KT, NV><<<grid_in, 256, 0, s>>>(n, d_seeds + (size_t)t * n, dmask,
                                                         d_inv + (size_t)t * KT, x[0] + (size_t)t * n * KT, pt);
    if (opt.rhs)
      ppr_load_kernel<T, KT, NV><<<grid_in, 256, 0, s>>>(n, opt.rhs, d_vec + (size_t)t * KT, newid_dev, dmask,
                                                         rhs_t[0] + (size_t)t * n * KT, nullptr);
    ppr_finalize_kernel<KT, AA><<<1, 1024, 0, s>>>(pt, grid_in, d_col + (size_t)t * KT, d_aa + (size_t)t * KT,
                                                 d_tile + t, beta, cst, p->max_iter, std::min(KT, k - t * KT), 1);
  }
  int rbase = 0;  // rhs_t[rbase] holds the current layout's right-hand side
  if (cudaGetLastError() != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank init"); }
  // Sweeps in sets of K on every tile of the current layout (stopped tiles
  // return at once).  After each set the vectors that stopped are written
  // out and dropped; when the live vectors fit in fewer tiles they are
  // repacked (compaction), so a tile never keeps sweeping for one slow
  // vector while its other lanes idle.  All tiles of a layout sweep in step:
  // plain, the layout's iterates start in x[base] and sweep j reads
  // x[(base+j)&1]; accelerated, sweep number gk of the solve writes ring slot
  // gk % 3.
  const int K = p->check_every > 0 ? p->check_every : 4;  // 4: R-MAT 2^22, 256 vectors, 3-9 % faster than 8
  int cur_tiles = tiles, base = 0;
  int64_t gk = 0;
  std::vector<int> slot_vec((size_t)tiles * KT, -1);  // vector in each slot, -1 for none
  for (int c = 0; c < k; ++c) slot_vec[(size_t)c] = c;
  std::vector<TileCtl> htc((size_t)tiles);
  std::vector<ColCtl> hcc((size_t)tiles * KT);
  std::vector<ColAa> hca((size_t)tiles * KT);
  int *d_map = nullptr;
  alloc((void **)&d_map, (size_t)tiles * KT * sizeof(int));
  if (st != TBSLA_OK) { cleanup(); return st; }
  std::vector<char> tile_live((size_t)tiles, 1);
  int phase = 0;
  const size_t tstride = (size_t)n * KT;
  while (true) {
    for (int k2 = 0; k2 < K; ++k2, ++phase, ++gk) {
      const int w = (int)(gk % 3), w1 = (int)((gk + 2) % 3), w2 = (int)((gk + 1) % 3);
      for (int t = 0; t < cur_tiles; ++t) {
        if (!tile_live[(size_t)t]) continue;  // stopped before this set of K sweeps
        const size_t off = (size_t)t * tstride;
        const T *xo = AA ? x[0] + off : x[(base + phase) & 1] + off;
        T *xn = AA ? g_ring[w] + off : x[(base + phase + 1) & 1] + off;
        PprRing<T> ring{AA ? r_ring[w] + off : nullptr, AA ? r_ring[w1] + off : nullptr,
                        AA ? r_ring[w2] + off : nullptr};
        double *pt = partials + (size_t)t * nparts * KT * NV;
        const unsigned *sd = d_seeds + (size_t)t * n;
        const ColCtl *cl = d_col + (size_t)t * KT;
        const ColAa *ca = d_aa + (size_t)t * KT;
        const double *iv = d_inv + (size_t)t * KT;
        const T *rh = opt.rhs ? rhs_t[rbase] + off : nullptr;
        ppr_spmm_kernel<T, KT, AA><<<grid_mm, 256, 0, s>>>(plan->items, plan->n_items, M->idx1, values, xo, xn,
                                                           sd, dmask, cl, ca, iv, beta, rh, ring, chunk, pt,
                                                           d_tile + t);
        if (n_crow)
          ppr_fixup_kernel<T, KT, AA><<<grid_fx, 256, 0, s>>>(plan->crow, n_crow, chunk, xo, xn, sd, dmask, cl, ca,
                                                              iv, beta, rh, ring, pt, grid_mm, d_tile + t);
        ppr_finalize_kernel<KT, AA><<<1, 1024, 0, s>>>(pt, n_crow ? grid_mm + grid_fx : grid_mm,
                                                     d_col + (size_t)t * KT, d_aa + (size_t)t * KT, d_tile + t,
                                                     beta, cst, p->max_iter, KT, 0);
        if (AA)
          ppr_combine_kernel<T, KT><<<grid_vec, 256, 0, s>>>(n, g_ring[w] + off, g_ring[w1] + off,
                                                            g_ring[w2] + off, x[0] + off, d_aa + (size_t)t * KT,
                                                            d_tile + t);
      }
    }
    if (cudaMemcpyAsync(htc.data(), d_tile, (size_t)cur_tiles * sizeof(TileCtl), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(hcc.data(), d_col, (size_t)cur_tiles * KT * sizeof(ColCtl), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        (AA && cudaMemcpyAsync(hca.data(), d_aa, (size_t)cur_tiles * KT * sizeof(ColAa), cudaMemcpyDeviceToHost,
                               s) != cudaSuccess) ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      cleanup();
      return fail(TBSLA_ERR_CUDA, "batched PageRank sweeps failed");
    }
    // write out and drop the vectors that stopped (a stopped vector is
    // frozen: plain, its tile's last iterate, x[(base + tile iter) & 1],
    // holds it; accelerated, x; a stopped tile's vectors have all stopped,
    // or max_iter is 0)
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
        const T *xf = (AA ? x[0] : x[(base + htc[(size_t)t].iter) & 1]) + (size_t)t * tstride;
        ppr_pick_kernel<T, KT><<<152 * 8, 256, 0, s>>>(xf, n, newid_dev, pk, d_out);
      }
      tile_live[(size_t)t] = !htc[(size_t)t].done;
      busy += !htc[(size_t)t].done;
    }
    if (cudaGetLastError() != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank results"); }
    if (live == 0) break;
    const int need = (live + KT - 1) / KT;
    if (need < busy) {
      // repack the live vectors into `need` tiles (every live tile has run all
      // `phase` sweeps of the layout): plain, their iterates (in
      // x[(base+phase)&1]) move to the other buffer, which becomes the new
      // layout's start; accelerated, the iterates, the rings and the
      // right-hand side are compacted in place
      std::vector<int> map((size_t)need * KT, -1), nvec((size_t)need * KT, -1);
      std::vector<int2> npairs;
      std::vector<double> ninv((size_t)need * KT, 0.0);
      std::vector<ColCtl> ncol((size_t)need * KT);
      std::vector<ColAa> naa((size_t)need * KT, aa0);
      int q = 0;
      for (int t = 0; t < cur_tiles; ++t)
        for (int c = 0; c < KT; ++c) {
          const int v = slot_vec[(size_t)t * KT + c];
          if (v < 0) continue;
          map[(size_t)q] = t * KT + c;
          nvec[(size_t)q] = v;
          ncol[(size_t)q] = hcc[(size_t)t * KT + c];
          if (AA) naa[(size_t)q] = hca[(size_t)t * KT + c];
          ninv[(size_t)q] = inv[(size_t)t * KT + c];
          for (int u : seed_sets[(size_t)v]) npairs.push_back(make_int2(q, u));
          ++q;
        }
      for (size_t r = (size_t)q; r < ncol.size(); ++r) ncol[r] = ColCtl{0.0, 0.0, 0.0, 0, 1};
      std::vector<TileCtl> ntile((size_t)need, TileCtl{0, 0, 0, 0});
      up(d_map, map.data(), map.size() * sizeof(int));
      up(d_pairs, npairs.data(), npairs.size() * sizeof(int2));  // no more pairs than at the start
      if (e == cudaSuccess) e = cudaMemsetAsync(d_seeds, 0, (size_t)need * n * sizeof(unsigned), s);
      if (e == cudaSuccess)
        ppr_seed_bits_kernel<KT><<<152, 256, 0, s>>>(d_seeds, n, d_pairs, (int)npairs.size());
      up(d_inv, ninv.data(), ninv.size() * sizeof(double));
      up(d_col, ncol.data(), ncol.size() * sizeof(ColCtl));
      if (AA) up(d_aa, naa.data(), naa.size() * sizeof(ColAa));
      up(d_tile, ntile.data(), ntile.size() * sizeof(TileCtl));
      if (e != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank repack: %s", cudaGetErrorString(e)); }
      if (AA) {
        T *bufs[8] = {x[0], g_ring[0], g_ring[1], g_ring[2], r_ring[0], r_ring[1], r_ring[2], rhs_t[0]};
        for (int t = 0; t < need; ++t)
          for (T *b : bufs)
            if (b) ppr_compact_kernel<T, KT><<<grid_vec, 256, 0, s>>>(b, n, d_map + (size_t)t * KT, t);
      } else {
        const int src = (base + phase) & 1;
        ppr_move_kernel<T, KT><<<152 * 8, 256, 0, s>>>(x[src], x[src ^ 1], n, d_map, need);
        if (opt.rhs) {
          ppr_move_kernel<T, KT><<<152 * 8, 256, 0, s>>>(rhs_t[rbase], rhs_t[rbase ^ 1], n, d_map, need);
          rbase ^= 1;
        }
        base = src ^ 1;
      }
      if (cudaGetLastError() != cudaSuccess) { cleanup(); return fail(TBSLA_ERR_CUDA, "batched PageRank repack"); }
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

template <typename T, int KT>
tbsla_status_t run_tiles(const tbsla_matrix *M, const int *newid_dev, const std::vector<int> *newid_host,
                         const tbsla_pagerank_params_t *p, int k, const int *nodes, const int *offsets,
                         double *d_out, int *iters_out, double *resid_out, cudaStream_t s,
                         const RunOpts &opt = RunOpts()) {
  if (p->accel)
    return run_tiles_impl<T, KT, true>(M, newid_dev, newid_host, p, k, nodes, offsets, d_out, iters_out,
                                       resid_out, s, opt);
  return run_tiles_impl<T, KT, false>(M, newid_dev, newid_host, p, k, nodes, offsets, d_out, iters_out, resid_out,
                                      s, opt);
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
constexpr double kRefineEta = 1e-3;       // inner tolerance relative to ||r_c||_1
constexpr double kRefineEtaAccel = 1e-4;  // the same for accelerated correction solves
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
    q64.accel = 0;
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
      tolc[(size_t)c] = res[(size_t)c] < p->tol ? HUGE_VAL : (p->accel ? kRefineEtaAccel : kRefineEta) * res[(size_t)c];
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
