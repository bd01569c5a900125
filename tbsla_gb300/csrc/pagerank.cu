// pagerank.cu -- PageRank on GB300: fused sweeps, deterministic reductions,
// CUDA-graph captured iteration, FP64 and mixed precision.
//
// A sweep is one SpMV whose epilogue writes the new iterate and accumulates
// per-thread partial sums (residual, dangling mass, total mass, or the
// maximum), reduced per block into a partials array; pr_finalize_kernel
// (one block) reduces the partials in a fixed order and updates the control
// block (iteration count, stopping flag, the teleport term of the next
// sweep).  No atomics on values: every result is independent of scheduling.
// Sweeps run from a CUDA graph of check_every sweeps with ping-pong iterate
// buffers; kernels of sweeps after convergence return immediately (they test
// the control block's flag), and the host reads the flag once per graph.
//
// Modes
//   TBSLA_PR_REFERENCE  Matrix::page_rank (src/cpp/matrix/Matrix.cpp:13-61):
//     b = beta*A b_prev + (1-beta)/n * sum(b_prev); b /= max(b);
//     err = sum |b - b_prev|; finally b /= sum(b).  With a node list this is
//     Matrix::personalized_page_rank (Matrix.cpp:63-114).
//   TBSLA_PR_DANGLING   x = beta*A x + (beta*dangling(x) + (1-beta)*sum(x))/n,
//     stop when ||x - x_prev||_1 < tol.
//   accelerated (DANGLING, FP64, accel = 1): Anderson acceleration of the
//     same fixed-point map over the last two differences (pr_aa_*), same
//     stopping rule on ||G(x) - x||_1, the result is G(x) of the last sweep.
//   mixed precision (DANGLING, precision F32/BF16): FP64 defect correction.
//     r = G(x) - x by an FP64 sweep (its L1 norm is the stopping quantity),
//     then e_{j+1} = G~ e_j + r by sweeps on the reduced-precision value store
//     with FP32 vectors until ||e_{j+1} - e_j||_1 < inner_tol, x += e (FP64).
#include <cmath>
#include <cstring>
#include <vector>

#include "anderson.cuh"
#include "product.cuh"

namespace tbsla {

tbsla_status_t spmv_dispatch(const tbsla_matrix *A, tbsla_dtype_t store, tbsla_dtype_t xt, const void *x,
                             tbsla_dtype_t yt, void *y, int vect_incr, cudaStream_t s);

// ------------------------------------------------------------ control
struct PrCtl {
  double beta, tol, inv_n, tele_scale;  // tele_scale: (1-beta)/n or (1-beta)/|P|
  double add;       // term of the next FP64 sweep (reference: tele; dangling: (b d + (1-b) s)/n)
  double add_in;    // term of the next inner sweep
  double maxv;      // reference mode: max of the unnormalised iterate
  double resid, d, s;
  double inner_resid, inner_tol;
  int iter, done, converged, max_iter;
  int inner_iter, inner_done, inner_max, pad;
  // Anderson acceleration: for the last three sweep outputs (slot k % 3),
  // the sweep term each would give as the next input (linear in it), their
  // residuals' Gram matrix with the newest first (gram[i][j] = r_{k-i} .
  // r_{k-j}), and the coefficients of the next input in the newest-first
  // outputs.  aa: the FP64 solves; iaa: the inner (correction) solves of the
  // mixed-precision solve.
  struct Aa {
    double add[3];
    double gram[3][3];
    double coef[3];
    int m, pad;
  } aa, iaa;
};

enum { kSweepRef = 0, kSweepDang = 1, kSweepInner = 2, kSweepTele = 3 };

// Block reduction of three per-thread values into partials[blk*3 + k]
// (sums, or a maximum for k = 0 when take_max): values go to shared memory,
// one warp adds them in a fixed order.
__device__ __forceinline__ void block_reduce3(double a, double b, double c, bool take_max, double *partials,
                                              int blk) {
  __shared__ double sh[3][256];
  const int t = threadIdx.x, nt = blockDim.x;
  sh[0][t] = a; sh[1][t] = b; sh[2][t] = c;
  __syncthreads();
  if (t < 32) {
    double v[3];
    for (int k = 0; k < 3; ++k) {
      double acc = sh[k][t];
      for (int u = t + 32; u < nt; u += 32) acc = (k == 0 && take_max) ? fmax(acc, sh[k][u]) : acc + sh[k][u];
      #pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_down_sync(0xffffffffu, acc, o);
        acc = (k == 0 && take_max) ? fmax(acc, w) : acc + w;
      }
      v[k] = acc;
    }
    if (t == 0) {
      partials[blk * 3 + 0] = v[0];
      partials[blk * 3 + 1] = v[1];
      partials[blk * 3 + 2] = v[2];
    }
  }
}

// The sweep epilogue: y[row] = beta*v + add (+ r[row]) and the partial sums.
template <typename YT, typename AccT> struct PrEpi {
  using Acc = AccT;
  static constexpr bool kReduces = true;  // per-block partials: capped grids
  // per-thread sums in the accumulator type: FP64 sweeps sum in FP64, the
  // FP32 inner sweeps of the mixed solve in FP32 (no FP64 operation per row)
  struct State {
    AccT a = 0, b = 0, c = 0;
  };
  YT *y;
  const YT *xold;               // previous iterate (residual)
  const YT *rvec;               // inner sweeps: + r
  const unsigned char *dmask;   // dangling columns (sums b)
  const unsigned char *tmask;   // reference mode with nodes: teleport only there
  const double *tvec;           // teleport mode: the teleport vector
  const double *add;            // device scalar
  const double *betap;          // device scalar (the damping of this run)
  const int *done;              // device flag: sweep inactive when set
  double *partials;
  int n, mode, part_base;
  __device__ __forceinline__ bool active() const { return *(volatile const int *)done == 0; }
  __host__ __device__ void set_part_base(int k) { part_base = k; }
  __device__ __forceinline__ void emit(int row, Acc v, State &st) const {
    if (row < 0 || row >= n) return;
    const double beta = *betap;
    if constexpr (std::is_same<AccT, float>::value) {
      // inner sweep (kSweepInner): e' = beta*G~e + add + r in FP32
      const float f = __fmaf_rn((float)beta, (float)v, (float)*add) + (float)rvec[row];
      st.a += fabsf(f - (float)xold[row]);
      if (dmask && dmask[row]) st.b += f;
      st.c += f;
      __stcs(y + row, (YT)f);
    } else {
      const double t = mode == kSweepTele ? *add * tvec[row]
                       : (mode == kSweepRef && tmask) ? (tmask[row] ? *add : 0.0) : *add;
      const double val = __fma_rn(beta, (double)v, t);
      if (mode == kSweepRef) {
        st.a = fmax(st.a, val);
      } else {
        st.a += fabs(val - (double)xold[row]);
        if (dmask && dmask[row]) st.b += val;
        st.c += val;
      }
      __stcs(y + row, (YT)val);
    }
  }
  __device__ __forceinline__ void block_done(State &st, int blk) const {
    block_reduce3((double)st.a, (double)st.b, (double)st.c, mode == kSweepRef, partials, part_base + blk);
  }
  __device__ __forceinline__ void fixup_done(State &st, int blk) const { block_done(st, blk); }
};

// Adjoint sweep epilogue, run on the transposed copy (row j = column j of
// A): lambda'[j] = beta * (A^T lambda)[j] + w[j] + (dangling[j] ? c1 : 0)
// with c1 = beta * (v . lambda); partials |lambda' - lambda| and v . lambda'.
struct AdjEpi {
  using Acc = double;
  static constexpr bool kReduces = true;
  struct State {
    double a = 0, b = 0, c = 0;
  };
  double *y;
  const double *yold;
  const double *w;
  const unsigned char *dmask;
  const double *v;      // teleport vector, NULL: uniform 1/n
  const double *c1;     // device scalar
  const double *betap;
  const int *done;
  double *partials;
  double inv_n;
  int n, part_base;
  __device__ __forceinline__ bool active() const { return *(volatile const int *)done == 0; }
  __host__ __device__ void set_part_base(int k) { part_base = k; }
  __device__ __forceinline__ void emit(int row, double acc, State &st) const {
    if (row < 0 || row >= n) return;
    const double val = __fma_rn(*betap, acc, w[row] + (dmask[row] ? *c1 : 0.0));
    st.a += fabs(val - yold[row]);
    st.b += (v ? v[row] : inv_n) * val;
    __stcs(y + row, val);
  }
  __device__ __forceinline__ void block_done(State &st, int blk) const {
    block_reduce3(st.a, st.b, st.c, false, partials, part_base + blk);
  }
  __device__ __forceinline__ void fixup_done(State &st, int blk) const { block_done(st, blk); }
};

// partial (0, v . x (or sum(x)/n), 0)
__global__ void __launch_bounds__(256) pr_dot_kernel(const double *__restrict__ x, const double *__restrict__ v,
                                                     int n, double inv_n, double *partials) {
  double d = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    d += (v ? v[i] : inv_n) * x[i];
  block_reduce3(0.0, d, 0.0, false, partials, blockIdx.x);
}

// out = (*s) * x
__global__ void pr_scale_to_kernel(const double *__restrict__ x, int n, const double *s, double *__restrict__ out) {
  const double f = *s;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = f * x[i];
}

// y = beta*(A x) + add (+r) over rows [0, n) from a plain product in `prod`:
// the path for formats whose kernels do not visit every row
template <typename YT>
__global__ void __launch_bounds__(256) pr_affine_kernel(const YT *__restrict__ prod, PrEpi<YT, typename AccOf<YT>::type> epi) {
  if (!epi.active()) return;
  typename PrEpi<YT, typename AccOf<YT>::type>::State st;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < epi.n; i += gridDim.x * blockDim.x)
    epi.emit(i, (typename AccOf<YT>::type)prod[i], st);
  epi.block_done(st, blockIdx.x);
}

// reference mode: b /= max; partial sums of |b - b_prev| and of b
__global__ void __launch_bounds__(256) pr_normalize_kernel(double *__restrict__ b, const double *__restrict__ bprev,
                                                           int n, const PrCtl *ctl, double *partials) {
  if (*(volatile const int *)&ctl->done) return;
  const double m = ctl->maxv;
  double err = 0, s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = b[i] / m;
    b[i] = v;
    err += fabs(v - bprev[i]);
    s += v;
  }
  block_reduce3(err, 0.0, s, false, partials, blockIdx.x);
}

// reduces partials [0, nparts) and advances the control block
__global__ void __launch_bounds__(256) pr_finalize_kernel(const double *__restrict__ partials, int nparts,
                                                          PrCtl *ctl, int stage) {
  const bool inner = stage == 3 || stage == 16 || stage == 17;
  if ((stage <= 3 || stage == 8 || stage == 10 || stage >= 12) &&
      (inner ? *(volatile int *)&ctl->inner_done : *(volatile int *)&ctl->done))
    return;
  __shared__ double sh[3][256];
  const int t = threadIdx.x;
  const bool take_max = stage == 0;
  double a = take_max ? -INFINITY : 0.0, b = 0, c = 0;
  for (int k = t; k < nparts; k += blockDim.x) {
    a = take_max ? fmax(a, partials[3 * k]) : a + partials[3 * k];
    b += partials[3 * k + 1];
    c += partials[3 * k + 2];
  }
  sh[0][t] = a; sh[1][t] = b; sh[2][t] = c;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      sh[0][t] = take_max ? fmax(sh[0][t], sh[0][t + w]) : sh[0][t] + sh[0][t + w];
      sh[1][t] += sh[1][t + w];
      sh[2][t] += sh[2][t + w];
    }
    __syncthreads();
  }
  if (t != 0) return;
  a = sh[0][0]; b = sh[1][0]; c = sh[2][0];
  if (stage == 7) { ctl->s = c; return; }
  switch (stage) {
  case 0:  // reference sweep: maximum of the unnormalised iterate
    ctl->maxv = a;
    break;
  case 1:  // reference normalisation: err = a, sum = c
    ctl->resid = a;
    ctl->s = c;
    ctl->iter += 1;
    ctl->add = ctl->tele_scale * c;
    ctl->converged = a < ctl->tol;
    ctl->done = ctl->converged || ctl->iter >= ctl->max_iter;
    break;
  case 2:  // dangling sweep: resid = a, dangling mass = b, sum = c
    ctl->resid = a;
    ctl->d = b;
    ctl->s = c;
    ctl->iter += 1;
    ctl->add = (ctl->beta * b + (1.0 - ctl->beta) * c) * ctl->inv_n;
    ctl->converged = a < ctl->tol;
    ctl->done = ctl->converged || ctl->iter >= ctl->max_iter;
    break;
  case 3:  // inner sweep
    ctl->inner_resid = a;
    ctl->inner_iter += 1;
    ctl->add_in = (ctl->beta * b + (1.0 - ctl->beta) * c) * ctl->inv_n;
    ctl->inner_done = a < ctl->inner_tol || ctl->inner_iter >= ctl->inner_max;
    break;
  case 4:  // initial vector: dangling mass b, sum c (FP64 sweeps)
    ctl->add = (ctl->beta * b + (1.0 - ctl->beta) * c) * ctl->inv_n;
    ctl->s = c;
    break;
  case 5:  // initial inner vector e0 = r
    ctl->add_in = (ctl->beta * b + (1.0 - ctl->beta) * c) * ctl->inv_n;
    break;
  case 6:  // reference start: tele of b0 = sum(b0) * tele_scale
    ctl->add = ctl->tele_scale * c;
    break;
  case 7:  // plain sum of a vector (final normalisation)
    ctl->s = c;
    break;
  case 8:  // teleport sweep: resid = a, dangling mass = b, sum = c
    ctl->resid = a;
    ctl->d = b;
    ctl->s = c;
    ctl->iter += 1;
    ctl->add = ctl->beta * b + (1.0 - ctl->beta);
    ctl->converged = a < ctl->tol;
    ctl->done = ctl->converged || ctl->iter >= ctl->max_iter;
    break;
  case 9:  // initial teleport-mode vector: dangling mass b
    ctl->add = ctl->beta * b + (1.0 - ctl->beta);
    ctl->s = c;
    break;
  case 10:  // adjoint sweep: resid = a, b = v . lambda
    ctl->resid = a;
    ctl->iter += 1;
    ctl->add = ctl->beta * b;
    ctl->converged = a < ctl->tol;
    ctl->done = ctl->converged || ctl->iter >= ctl->max_iter;
    break;
  case 11:  // initial adjoint vector: b = v . lambda0
    ctl->add = ctl->beta * b;
    break;
  case 12:    // accelerated dangling sweep k (as stage 2)
  case 14:    // accelerated teleport sweep k (as stage 8)
  case 15: {  // accelerated adjoint sweep k (as stage 10)
    // the term of the next sweep if g_k were its input, kept per slot; the
    // Anderson step combines them like the outputs
    const int slot = ctl->iter % 3;
    ctl->resid = a;
    ctl->aa.add[slot] = stage == 12 ? (ctl->beta * b + (1.0 - ctl->beta) * c) * ctl->inv_n
                        : stage == 14 ? ctl->beta * b + (1.0 - ctl->beta)
                                      : ctl->beta * b;
    ctl->d = b;
    ctl->s = c;
    ctl->iter += 1;
    ctl->converged = a < ctl->tol;
    ctl->done = ctl->converged || ctl->iter >= ctl->max_iter;
    break;
  }
  case 13:    // residual dots of sweep k: r_k . r_k, r_k . r_{k-1}, r_k . r_{k-2}
  case 16: {  // the same for inner sweep k
    // shift the newest-first Gram matrix by one and add the new row
    aa_gram_push(stage == 13 ? ctl->aa.gram : ctl->iaa.gram, a, b, c);
    break;
  }
  case 17: {  // accelerated inner sweep k (as stage 3), its next-sweep term kept per slot
    const int slot = ctl->inner_iter % 3;
    ctl->inner_resid = a;
    ctl->iaa.add[slot] = (ctl->beta * b + (1.0 - ctl->beta) * c) * ctl->inv_n;
    ctl->inner_iter += 1;
    ctl->inner_done = a < ctl->inner_tol || ctl->inner_iter >= ctl->inner_max;
    break;
  }
  }
}

// The Anderson step after sweep k (one thread): the coefficients of the next
// input in the last three outputs (aa_coefficients).  They sum to 1, and the
// next sweep's term is affine in its input, so it is the same combination of
// the outputs' terms.
__global__ void pr_aa_solve_kernel(PrCtl *ctl, int inner) {
  if (*(volatile int *)(inner ? &ctl->inner_done : &ctl->done)) return;
  PrCtl::Aa &st = inner ? ctl->iaa : ctl->aa;
  const int k = (inner ? ctl->inner_iter : ctl->iter) - 1;  // the sweep just finished
  st.m = aa_coefficients(st.gram, k < 2 ? k : 2, st.coef);
  const double c0 = st.coef[0], c1 = st.coef[1], c2 = st.coef[2];
  const int s0 = k % 3, s1 = (k + 2) % 3, s2 = (k + 1) % 3;  // slots of g_k, g_{k-1}, g_{k-2}
  double add = c0 * st.add[s0];
  if (st.m >= 1) add += c1 * st.add[s1];
  if (st.m >= 2) add += c2 * st.add[s2];
  (inner ? ctl->add_in : ctl->add) = add;
}

// r_k = g_k - x_k into its slot, and the partial dots of r_k with r_k,
// r_{k-1}, r_{k-2} (the missing ones are 0)
template <typename T>
__global__ void __launch_bounds__(256) pr_aa_dots_kernel(const T *__restrict__ g, const T *__restrict__ x,
                                                         T *__restrict__ r0, const T *__restrict__ r1,
                                                         const T *__restrict__ r2, int n, const PrCtl *ctl, int inner,
                                                         double *partials) {
  if (*(volatile const int *)(inner ? &ctl->inner_done : &ctl->done)) return;
  const int k = (inner ? ctl->inner_iter : ctl->iter) - 1;
  double p0 = 0, p1 = 0, p2 = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const T r = g[i] - x[i];
    r0[i] = r;
    p0 += (double)r * (double)r;
    if (k >= 1) p1 += (double)r * (double)r1[i];
    if (k >= 2) p2 += (double)r * (double)r2[i];
  }
  block_reduce3(p0, p1, p2, false, partials, blockIdx.x);
}

// x_{k+1} = c0 g_k + c1 g_{k-1} + c2 g_{k-2} (only the terms in use are read)
template <typename T>
__global__ void __launch_bounds__(256) pr_aa_combine_kernel(const T *__restrict__ g0, const T *__restrict__ g1,
                                                            const T *__restrict__ g2, T *__restrict__ x, int n,
                                                            const PrCtl *ctl, int inner) {
  if (*(volatile const int *)(inner ? &ctl->inner_done : &ctl->done)) return;
  const PrCtl::Aa &st = inner ? ctl->iaa : ctl->aa;
  const T c0 = (T)st.coef[0], c1 = (T)st.coef[1], c2 = (T)st.coef[2];
  const int m = st.m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    T v = c0 * g0[i];
    if (m >= 1) v = fma(c1, g1[i], v);
    if (m >= 2) v = fma(c2, g2[i], v);
    x[i] = v;
  }
}

// partial (0, dangling mass, sum) of a vector
template <typename T>
__global__ void __launch_bounds__(256) pr_mass_kernel(const T *__restrict__ v, int n, const unsigned char *dmask,
                                                      double *partials) {
  double d = 0, s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double x = v[i];
    if (dmask && dmask[i]) d += x;
    s += x;
  }
  block_reduce3(0.0, d, s, false, partials, blockIdx.x);
}

__global__ void pr_fill_kernel(double *x, int n, double v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = v;
}

// r = x1 - x0 in FP32, e0 = r
__global__ void pr_residual_kernel(const double *__restrict__ x1, const double *__restrict__ x0, float *r,
                                   float *e, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float d = (float)(x1[i] - x0[i]);
    r[i] = d;
    e[i] = d;
  }
}

// x += e
__global__ void pr_correct_kernel(double *__restrict__ x, const float *__restrict__ e, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += (double)e[i];
}

__global__ void pr_scale_kernel(double *x, int n, const double *sum) {
  const double s = *sum;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = x[i] / s;
}

// columns with a nonzero stored value are not dangling
template <typename V>
__global__ void pr_dangling_kernel(const int *__restrict__ cols, const V *__restrict__ vals, int64_t n,
                                   int f_col, int n_col, unsigned char *dmask) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int c = cols[k] - f_col;
    if (vals[k] != V(0) && c >= 0 && c < n_col) dmask[c] = 0;
  }
}
__global__ void pr_dangling_dense_kernel(const double *__restrict__ a, int rows, int cols, unsigned char *dmask) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < cols; j += gridDim.x * blockDim.x) {
    bool any = false;
    for (int i = 0; i < rows && !any; ++i) any = a[(size_t)i * cols + j] != 0.0;
    if (any) dmask[j] = 0;
  }
}

// ------------------------------------------------------------ workspace
constexpr int kAffineBlocks = 152 * 4;

struct PrWork {
  int n = 0;
  double *x[2] = {nullptr, nullptr};  // FP64 iterates
  double *prod = nullptr;             // plain product (generic path)
  float *e[2] = {nullptr, nullptr};   // inner iterates
  float *prod32 = nullptr;
  float *r = nullptr;
  unsigned char *dmask = nullptr, *tmask = nullptr;
  double *tvec = nullptr;             // teleport mode: copy of the teleport vector
  double *lam[2] = {nullptr, nullptr};  // adjoint iterates
  double *ag[3] = {nullptr, nullptr, nullptr};  // accelerated solve: sweep outputs (slot k % 3)
  double *ar[3] = {nullptr, nullptr, nullptr};  // and their residuals
  float *eg[3] = {nullptr, nullptr, nullptr};   // accelerated inner solve: outputs (slot k % 3)
  float *er[3] = {nullptr, nullptr, nullptr};   // and their residuals
  double *adj_partials = nullptr;
  int adj_nparts = 0;
  double *partials = nullptr;
  int nparts = 0;
  PrCtl *ctl = nullptr;
  PrCtl *ctl_host = nullptr;          // pinned
  cudaStream_t stream = nullptr;
  double *result = nullptr;           // buffer holding the last result
  // captured graphs: key = (kind, sweeps)
  struct G { int kind, sweeps, precision; cudaGraphExec_t exec; };
  std::vector<G> graphs;
  ~PrWork() {
    for (auto &g : graphs) cudaGraphExecDestroy(g.exec);
    void *ps[] = {x[0], x[1], prod, e[0], e[1], prod32, r, dmask, tmask, tvec, lam[0], lam[1], adj_partials,
                  partials, ctl, ag[0], ag[1], ag[2], ar[0], ar[1], ar[2], eg[0], eg[1], eg[2], er[0], er[1],
                  er[2]};
    for (void *p : ps) if (p) cudaFree(p);
    if (ctl_host) cudaFreeHost(ctl_host);
    if (stream) cudaStreamDestroy(stream);
  }
};

static tbsla_status_t pr_alloc(void **p, size_t bytes) {
  const cudaError_t e = cudaMalloc(p, bytes + 64);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(TBSLA_ERR_OOM, "cudaMalloc(%zu) for PageRank failed: %s", bytes, cudaGetErrorString(e));
  }
  return TBSLA_OK;
}

// blocks of one sweep's partials
static int sweep_parts(const tbsla_matrix *A, bool fused) {
  if (!fused) return kAffineBlocks;
  int p = 0;
  p += short_parts_reducing(A);
  for (int c = 0; c < kGroupClasses; ++c) {
    const int count = A->item_class_start[c + 1] - A->item_class_start[c];
    if (count > 0) p += group_grid(count, kGroupLanes[c], true);
  }
  if (A->n_chunk_rows > 0) p += fixup_grid(A->n_chunk_rows);
  return std::max(p, 1);
}

// the fused path: CSR direct kernels visit every row exactly once
static bool fused_ok(const tbsla_matrix *A) {
  return A->format == TBSLA_FMT_CSR && A->csr_variant == 0 && A->rows == A->n_row && A->stored > 0;
}

static tbsla_status_t pr_setup(tbsla_matrix *A, PrWork **out) {
  PrWork *W = static_cast<PrWork *>(A->pr_work);
  if (W) { *out = W; return TBSLA_OK; }
  W = new PrWork();
  const int n = A->n_col;
  W->n = n;
  tbsla_status_t st = TBSLA_OK;
  auto alloc = [&](void **p, size_t b) { if (st == TBSLA_OK) st = pr_alloc(p, b); };
  alloc((void **)&W->x[0], (size_t)n * 8);
  alloc((void **)&W->x[1], (size_t)n * 8);
  alloc((void **)&W->prod, (size_t)n * 8);
  alloc((void **)&W->dmask, (size_t)n);
  alloc((void **)&W->tmask, (size_t)n);
  W->nparts = std::max(sweep_parts(A, fused_ok(A)), kAffineBlocks);
  alloc((void **)&W->partials, (size_t)W->nparts * 3 * 8);
  alloc((void **)&W->ctl, sizeof(PrCtl));
  if (st == TBSLA_OK && cudaMallocHost((void **)&W->ctl_host, sizeof(PrCtl)) != cudaSuccess)
    st = fail(TBSLA_ERR_OOM, "pinned control block");
  if (st == TBSLA_OK && cudaStreamCreateWithFlags(&W->stream, cudaStreamNonBlocking) != cudaSuccess)
    st = fail(TBSLA_ERR_CUDA, "stream creation failed");
  if (st == TBSLA_OK) {
    // dangling columns: those without a nonzero stored value
    cudaMemsetAsync(W->dmask, 1, (size_t)n, W->stream);
    const int g = 152 * 8;
    switch (A->format) {
    case TBSLA_FMT_CSR:
    case TBSLA_FMT_COO:
    case TBSLA_FMT_SCOO: {
      const int *cols = A->idx1;
      if (A->values[0]) pr_dangling_kernel<double><<<g, 256, 0, W->stream>>>(cols, (const double *)A->values[0], A->stored, A->f_col, n, W->dmask);
      else if (A->values[1]) pr_dangling_kernel<float><<<g, 256, 0, W->stream>>>(cols, (const float *)A->values[1], A->stored, A->f_col, n, W->dmask);
      break;
    }
    case TBSLA_FMT_ELL:
      if (A->values[0])
        pr_dangling_kernel<double><<<g, 256, 0, W->stream>>>(A->idx0, (const double *)A->values[0],
                                                             (int64_t)A->rows_pad * A->max_col, A->f_col, n, W->dmask);
      break;
    case TBSLA_FMT_DENSE:
      if (A->values[0]) pr_dangling_dense_kernel<<<g, 256, 0, W->stream>>>((const double *)A->values[0], A->rows, A->cols, W->dmask);
      break;
    }
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(W->stream) != cudaSuccess)
      st = fail(TBSLA_ERR_CUDA, "PageRank setup kernels failed");
  }
  if (st != TBSLA_OK) { delete W; return st; }
  A->pr_work = W;
  A->pr_work_free = [](void *p) { delete static_cast<PrWork *>(p); };
  *out = W;
  return TBSLA_OK;
}

static tbsla_status_t pr_inner_buffers(PrWork *W) {
  if (W->e[0]) return TBSLA_OK;
  const size_t b = (size_t)W->n * 4;
  TB_TRY(pr_alloc((void **)&W->e[0], b));
  TB_TRY(pr_alloc((void **)&W->e[1], b));
  TB_TRY(pr_alloc((void **)&W->prod32, b));
  TB_TRY(pr_alloc((void **)&W->r, b));
  return TBSLA_OK;
}

// one FP64 sweep x_in -> x_out (mode kSweepRef or kSweepDang) + finalize
static tbsla_status_t enqueue_f64_sweep(const tbsla_matrix *A, PrWork *W, const double *x_in, double *x_out,
                                        int mode, bool with_tmask, cudaStream_t s, bool accel = false) {
  PrEpi<double, double> epi{};
  epi.y = x_out;
  epi.xold = x_in;
  epi.rvec = nullptr;
  epi.dmask = mode == kSweepDang || mode == kSweepTele ? W->dmask : nullptr;
  epi.tmask = with_tmask ? W->tmask : nullptr;
  epi.tvec = mode == kSweepTele ? W->tvec : nullptr;
  epi.add = &W->ctl->add;
  epi.betap = &W->ctl->beta;
  epi.done = &W->ctl->done;
  epi.partials = W->partials;
  epi.n = W->n;
  epi.mode = mode;
  epi.part_base = 0;
  int nparts;
  if (fused_ok(A)) {
    TB_TRY(launch_product<double, double>(A, static_cast<const double *>(A->values[0]), x_in, epi, s));
    nparts = sweep_parts(A, true);
  } else {
    TB_TRY(spmv_dispatch(A, TBSLA_F64, TBSLA_F64, x_in, TBSLA_F64, W->prod, 0, s));
    pr_affine_kernel<double><<<kAffineBlocks, 256, 0, s>>>(W->prod, epi);
    nparts = kAffineBlocks;
  }
  if (mode == kSweepRef) {
    pr_finalize_kernel<<<1, 256, 0, s>>>(W->partials, nparts, W->ctl, 0);
    pr_normalize_kernel<<<kAffineBlocks, 256, 0, s>>>(x_out, x_in, W->n, W->ctl, W->partials);
    pr_finalize_kernel<<<1, 256, 0, s>>>(W->partials, kAffineBlocks, W->ctl, 1);
  } else {
    pr_finalize_kernel<<<1, 256, 0, s>>>(W->partials, nparts, W->ctl,
                                         mode == kSweepTele ? (accel ? 14 : 8) : (accel ? 12 : 2));
  }
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

// the ring buffers of the accelerated solves
static tbsla_status_t pr_aa_buffers(PrWork *W) {
  if (W->ag[0]) return TBSLA_OK;
  for (int i = 0; i < 3; ++i) {
    TB_TRY(pr_alloc((void **)&W->ag[i], (size_t)W->n * 8));
    TB_TRY(pr_alloc((void **)&W->ar[i], (size_t)W->n * 8));
  }
  return TBSLA_OK;
}

// after sweep k wrote g_k (slot k % 3) from x: residual dots, the Anderson
// step, x <- the combination
static tbsla_status_t enqueue_aa_step(PrWork *W, double *x, double *partials, int k, cudaStream_t s) {
  const int s0 = k % 3, s1 = (k + 2) % 3, s2 = (k + 1) % 3;
  pr_aa_dots_kernel<double><<<kAffineBlocks, 256, 0, s>>>(W->ag[s0], x, W->ar[s0], W->ar[s1], W->ar[s2], W->n,
                                                          W->ctl, 0, partials);
  pr_finalize_kernel<<<1, 256, 0, s>>>(partials, kAffineBlocks, W->ctl, 13);
  pr_aa_solve_kernel<<<1, 1, 0, s>>>(W->ctl, 0);
  pr_aa_combine_kernel<double><<<kAffineBlocks, 256, 0, s>>>(W->ag[s0], W->ag[s1], W->ag[s2], x, W->n, W->ctl, 0);
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

// the ring buffers of the accelerated inner solves
static tbsla_status_t pr_inner_aa_buffers(PrWork *W) {
  if (W->eg[0]) return TBSLA_OK;
  for (int i = 0; i < 3; ++i) {
    TB_TRY(pr_alloc((void **)&W->eg[i], (size_t)W->n * 4));
    TB_TRY(pr_alloc((void **)&W->er[i], (size_t)W->n * 4));
  }
  return TBSLA_OK;
}

// after inner sweep k wrote eg[k % 3] from e: the same step in FP32 vectors
// (dots summed in FP64)
static tbsla_status_t enqueue_inner_aa_step(PrWork *W, float *e, int k, cudaStream_t s) {
  const int s0 = k % 3, s1 = (k + 2) % 3, s2 = (k + 1) % 3;
  pr_aa_dots_kernel<float><<<kAffineBlocks, 256, 0, s>>>(W->eg[s0], e, W->er[s0], W->er[s1], W->er[s2], W->n,
                                                         W->ctl, 1, W->partials);
  pr_finalize_kernel<<<1, 256, 0, s>>>(W->partials, kAffineBlocks, W->ctl, 16);
  pr_aa_solve_kernel<<<1, 1, 0, s>>>(W->ctl, 1);
  pr_aa_combine_kernel<float><<<kAffineBlocks, 256, 0, s>>>(W->eg[s0], W->eg[s1], W->eg[s2], e, W->n, W->ctl, 1);
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

// one accelerated iteration k of the forward map (dangling or teleport mode)
static tbsla_status_t enqueue_aa_iteration(const tbsla_matrix *A, PrWork *W, int k, int mode, cudaStream_t s) {
  double *x = W->x[0];
  TB_TRY(enqueue_f64_sweep(A, W, x, W->ag[k % 3], mode, false, s, true));
  return enqueue_aa_step(W, x, W->partials, k, s);
}

// one low-precision inner sweep e_in -> e_out + finalize
static tbsla_status_t enqueue_inner_sweep(const tbsla_matrix *A, PrWork *W, tbsla_dtype_t store, const float *e_in,
                                          float *e_out, cudaStream_t s, bool accel = false) {
  PrEpi<float, float> epi{};
  epi.y = e_out;
  epi.xold = e_in;
  epi.rvec = W->r;
  epi.dmask = W->dmask;
  epi.tmask = nullptr;
  epi.add = &W->ctl->add_in;
  epi.betap = &W->ctl->beta;
  epi.done = &W->ctl->inner_done;
  epi.partials = W->partials;
  epi.n = W->n;
  epi.mode = kSweepInner;
  int nparts;
  if (fused_ok(A)) {
    if (store == TBSLA_F32)
      TB_TRY(launch_product<float, float>(A, static_cast<const float *>(A->values[1]), e_in, epi, s));
    else
      TB_TRY(launch_product<__nv_bfloat16, float>(A, static_cast<const __nv_bfloat16 *>(A->values[2]), e_in, epi, s));
    nparts = sweep_parts(A, true);
  } else {
    TB_TRY(spmv_dispatch(A, store, TBSLA_F32, e_in, TBSLA_F32, W->prod32, 0, s));
    pr_affine_kernel<float><<<kAffineBlocks, 256, 0, s>>>(W->prod32, epi);
    nparts = kAffineBlocks;
  }
  pr_finalize_kernel<<<1, 256, 0, s>>>(W->partials, nparts, W->ctl, accel ? 17 : 3);
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

// A graph of `sweeps` sweeps (kind 0: FP64 sweeps from x[0], alternating;
// kind 1: inner sweeps from e[0], alternating; kind 2: accelerated
// iterations, slots k % 3; kind 3: accelerated inner iterations from e[0],
// slots k % 3); sweeps is even (kinds 2 and 3: a multiple of 6) so that the
// buffers are back in place after each launch.
static tbsla_status_t get_graph(const tbsla_matrix *A, PrWork *W, int kind, int sweeps, int precision, int mode,
                                bool with_tmask, cudaGraphExec_t *exec) {
  for (auto &g : W->graphs)
    if (g.kind == kind * 16 + mode * 2 + (with_tmask ? 1 : 0) && g.sweeps == sweeps && g.precision == precision) {
      *exec = g.exec;
      return TBSLA_OK;
    }
  cudaStream_t s = W->stream;
  TB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  tbsla_status_t st = TBSLA_OK;
  for (int k = 0; k < sweeps && st == TBSLA_OK; ++k) {
    if (kind == 0) st = enqueue_f64_sweep(A, W, W->x[k & 1], W->x[(k + 1) & 1], mode, with_tmask, s);
    else if (kind == 1) st = enqueue_inner_sweep(A, W, (tbsla_dtype_t)precision, W->e[k & 1], W->e[(k + 1) & 1], s);
    else if (kind == 3) {
      st = enqueue_inner_sweep(A, W, (tbsla_dtype_t)precision, W->e[0], W->eg[k % 3], s, true);
      if (st == TBSLA_OK) st = enqueue_inner_aa_step(W, W->e[0], k, s);
    } else st = enqueue_aa_iteration(A, W, k, mode, s);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(s, &graph);
  if (st != TBSLA_OK) { if (graph) cudaGraphDestroy(graph); return st; }
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
  cudaGraphExec_t ex = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&ex, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate", __FILE__, __LINE__);
  W->graphs.push_back({kind * 16 + mode * 2 + (with_tmask ? 1 : 0), sweeps, precision, ex});
  *exec = ex;
  return TBSLA_OK;
}

static tbsla_status_t read_ctl(PrWork *W) {
  TB_CUDA(cudaMemcpyAsync(W->ctl_host, W->ctl, sizeof(PrCtl), cudaMemcpyDeviceToHost, W->stream));
  TB_CUDA(cudaStreamSynchronize(W->stream));
  return TBSLA_OK;
}

static tbsla_status_t write_ctl(PrWork *W) {
  TB_CUDA(cudaMemcpyAsync(W->ctl, W->ctl_host, sizeof(PrCtl), cudaMemcpyHostToDevice, W->stream));
  return TBSLA_OK;
}

// the FP64 power iteration (reference or dangling mode); result in x[iter % 2]
static tbsla_status_t run_f64(tbsla_matrix *A, PrWork *W, int mode, bool with_tmask, int check_every) {
  cudaGraphExec_t ex;
  TB_TRY(get_graph(A, W, 0, check_every, TBSLA_F64, mode, with_tmask, &ex));
  while (true) {
    TB_CUDA(cudaGraphLaunch(ex, W->stream));
    TB_TRY(read_ctl(W));
    if (W->ctl_host->done) break;
  }
  return TBSLA_OK;
}

// the Anderson-accelerated FP64 solve (dangling or teleport mode); result in
// ag[(iter-1) % 3]
static tbsla_status_t run_aa(tbsla_matrix *A, PrWork *W, int mode, int check_every) {
  TB_TRY(pr_aa_buffers(W));
  const int K = std::max(6, (check_every + 5) / 6 * 6);
  cudaGraphExec_t ex;
  TB_TRY(get_graph(A, W, 2, K, TBSLA_F64, mode, false, &ex));
  while (true) {
    TB_CUDA(cudaGraphLaunch(ex, W->stream));
    TB_TRY(read_ctl(W));
    if (W->ctl_host->done) break;
  }
  return TBSLA_OK;
}

static double *pr_result(PrWork *W) { return W->result; }

tbsla_status_t pr_relabelled(tbsla_matrix *A, tbsla_matrix **B);
tbsla_status_t pr_relabel_gather(const tbsla_matrix *A, const double *x, double *out, cudaStream_t s);

}  // namespace tbsla

using namespace tbsla;

static tbsla_status_t pagerank_impl(tbsla_matrix *A, const tbsla_pagerank_params_t *p, const int *nodes,
                                    int n_nodes, double *d_out, tbsla_pagerank_result_t *res, cudaStream_t user,
                                    const double *d_teleport = nullptr) {
  TB_CHECK(A && p, "NULL argument");
  TB_CHECK(A->n_row == A->n_col, "PageRank needs a square matrix (%d x %d)", A->n_row, A->n_col);
  TB_CHECK(A->n_col > 0, "empty matrix");
  TB_CHECK(p->max_iter >= 0, "max_iter < 0");
  TB_CHECK(p->mode == TBSLA_PR_REFERENCE || p->mode == TBSLA_PR_DANGLING || p->mode == TBSLA_PR_TELEPORT,
           "unknown PageRank mode %d", p->mode);
  TB_CHECK(p->mode != TBSLA_PR_TELEPORT || (d_teleport && p->precision == TBSLA_F64),
           "the teleport mode needs a teleport vector and FP64");
  TB_CHECK(p->precision == TBSLA_F64 || p->precision == TBSLA_F32 || p->precision == TBSLA_BF16, "bad precision");
  TB_CHECK(p->precision == TBSLA_F64 || p->mode == TBSLA_PR_DANGLING, "reduced precision needs TBSLA_PR_DANGLING");
  TB_CHECK(p->accel == 0 || (p->accel == 1 && p->mode != TBSLA_PR_REFERENCE && nodes == nullptr),
           "accel = %d: Anderson acceleration (1) is for the dangling and teleport modes", p->accel);
  TB_CHECK(A->values[0], "PageRank needs the F64 value store");
  TB_CHECK(p->precision == TBSLA_F64 || A->values[store_index((tbsla_dtype_t)p->precision)],
           "the requested reduced-precision value store is not present");
  TB_CHECK(nodes == nullptr || p->mode == TBSLA_PR_REFERENCE, "node lists are for the reference mode");
  TB_CUDA(cudaSetDevice(A->device));
  PrWork *W = nullptr;
  TB_TRY(pr_setup(A, &W));
  // kernel timing records events; none inside captured graphs
  struct TimingOff {
    tbsla_matrix *A;
    bool was;
    ~TimingOff() { A->timing = was; }
  } timing_off{A, A->timing};
  A->timing = false;
  // order after work the caller queued on its stream
  if (user) {
    cudaEvent_t ev;
    TB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, user);
    cudaStreamWaitEvent(W->stream, ev, 0);
    cudaEventDestroy(ev);
  }
  const int n = W->n;
  const int K = p->check_every > 0 ? (p->check_every + 1) / 2 * 2 : 8;
  PrCtl &c = *W->ctl_host;
  std::memset(&c, 0, sizeof c);
  c.beta = p->beta;
  c.tol = p->tol;
  c.inv_n = 1.0 / n;
  c.max_iter = p->max_iter;
  const bool with_tmask = nodes != nullptr;
  if (with_tmask) {
    TB_CHECK(n_nodes > 0, "empty node list");
    std::vector<unsigned char> m((size_t)n, 0);
    for (int k = 0; k < n_nodes; ++k)
      if (nodes[k] >= 0 && nodes[k] < n) m[(size_t)nodes[k]] = 1;
    TB_CUDA(cudaMemcpyAsync(W->tmask, m.data(), (size_t)n, cudaMemcpyHostToDevice, W->stream));
    TB_CUDA(cudaStreamSynchronize(W->stream));
    c.tele_scale = (1.0 - p->beta) / n_nodes;
  } else {
    c.tele_scale = (1.0 - p->beta) / n;
  }
  c.done = p->max_iter == 0;
  TB_TRY(write_ctl(W));
  const int g = kAffineBlocks;
  if (p->mode == TBSLA_PR_TELEPORT) {
    if (!W->tvec) TB_TRY(pr_alloc((void **)&W->tvec, (size_t)n * 8));
    TB_CUDA(cudaMemcpyAsync(W->tvec, d_teleport, (size_t)n * 8, cudaMemcpyDeviceToDevice, W->stream));
    TB_CUDA(cudaMemcpyAsync(W->x[0], d_teleport, (size_t)n * 8, cudaMemcpyDeviceToDevice, W->stream));
    pr_mass_kernel<double><<<g, 256, 0, W->stream>>>(W->x[0], n, W->dmask, W->partials);
    pr_finalize_kernel<<<1, 256, 0, W->stream>>>(W->partials, g, W->ctl, 9);
  } else if (p->mode == TBSLA_PR_REFERENCE) {
    pr_fill_kernel<<<g, 256, 0, W->stream>>>(W->x[0], n, with_tmask ? 0.25 : 1.0);
    pr_mass_kernel<double><<<g, 256, 0, W->stream>>>(W->x[0], n, nullptr, W->partials);
    pr_finalize_kernel<<<1, 256, 0, W->stream>>>(W->partials, g, W->ctl, 6);
  } else {
    pr_fill_kernel<<<g, 256, 0, W->stream>>>(W->x[0], n, 1.0 / n);
    pr_mass_kernel<double><<<g, 256, 0, W->stream>>>(W->x[0], n, W->dmask, W->partials);
    pr_finalize_kernel<<<1, 256, 0, W->stream>>>(W->partials, g, W->ctl, 4);
  }
  TB_CUDA(cudaGetLastError());

  int f64_sweeps = 0, inner_total = 0;
  const bool accel = p->accel != 0 && p->precision == TBSLA_F64 && p->mode != TBSLA_PR_REFERENCE;
  if (accel) {
    if (!c.done) TB_TRY(run_aa(A, W, p->mode == TBSLA_PR_TELEPORT ? kSweepTele : kSweepDang, K));
    else TB_TRY(read_ctl(W));
    f64_sweeps = c.iter;
  } else if (p->precision == TBSLA_F64) {
    const int sweep = p->mode == TBSLA_PR_REFERENCE ? kSweepRef : p->mode == TBSLA_PR_TELEPORT ? kSweepTele : kSweepDang;
    if (!c.done) TB_TRY(run_f64(A, W, sweep, with_tmask, K));
    else TB_TRY(read_ctl(W));
    f64_sweeps = c.iter;
  } else {
    // accel = 1: the inner solves are Anderson-accelerated (FP32 vectors)
    const bool inner_accel = p->accel != 0;
    TB_TRY(pr_inner_buffers(W));
    if (inner_accel) TB_TRY(pr_inner_aa_buffers(W));
    cudaGraphExec_t inner_ex;
    if (inner_accel) TB_TRY(get_graph(A, W, 3, std::max(6, (K + 5) / 6 * 6), p->precision, kSweepInner, false,
                                      &inner_ex));
    else TB_TRY(get_graph(A, W, 1, K, p->precision, kSweepInner, false, &inner_ex));
    // defect correction: FP64 sweep for r = G(x) - x, inner solve, x += e.
    // The inner tolerance relative to ||r||: with accelerated inner solves an
    // FP32 store is solved further (each correction then gains about four
    // decades; R-MAT 2^20: 3 FP64 + 11 FP32 sweeps against 26 plain FP64
    // sweeps), a BF16 store as before (its model error bounds the gain).
    const double eta = p->precision == TBSLA_BF16 ? 0.05 : inner_accel ? 1e-4 : 0.01;
    while (true) {
      TB_TRY(enqueue_f64_sweep(A, W, W->x[0], W->x[1], kSweepDang, false, W->stream));
      TB_TRY(read_ctl(W));
      ++f64_sweeps;
      if (c.done) break;
      // r = x1 - x0, e0 = r; inner solve to ||e_{j+1}-e_j|| < eta ||r||
      pr_residual_kernel<<<g, 256, 0, W->stream>>>(W->x[1], W->x[0], W->r, W->e[0], n);
      pr_mass_kernel<float><<<g, 256, 0, W->stream>>>(W->e[0], n, W->dmask, W->partials);
      c.inner_iter = 0;
      c.inner_done = 0;
      c.inner_tol = eta * c.resid;
      c.inner_max = 4 * K * 16;
      // only the inner fields change: copy the control block back
      TB_TRY(write_ctl(W));
      pr_finalize_kernel<<<1, 256, 0, W->stream>>>(W->partials, g, W->ctl, 5);
      while (true) {
        TB_CUDA(cudaGraphLaunch(inner_ex, W->stream));
        TB_TRY(read_ctl(W));
        if (c.inner_done) break;
      }
      inner_total += c.inner_iter;
      // the last inner output: eg[(iter - 1) % 3] (accelerated) or e[iter % 2]
      const float *e_last = inner_accel ? W->eg[(c.inner_iter - 1) % 3] : W->e[c.inner_iter & 1];
      pr_correct_kernel<<<g, 256, 0, W->stream>>>(W->x[0], e_last, n);
      // the next FP64 sweep needs the teleport term of the corrected x
      pr_mass_kernel<double><<<g, 256, 0, W->stream>>>(W->x[0], n, W->dmask, W->partials);
      pr_finalize_kernel<<<1, 256, 0, W->stream>>>(W->partials, g, W->ctl, 4);
      TB_CUDA(cudaGetLastError());
    }
  }
  // result buffer: FP64 runs end in x[iter % 2]; the mixed run in x[1], the
  // output G(x) of its last FP64 sweep
  W->result = accel ? (c.iter > 0 ? W->ag[(c.iter - 1) % 3] : W->x[0])
                    : p->precision == TBSLA_F64 ? W->x[c.iter & 1] : W->x[1];
  double *xr = W->result;
  if (p->mode == TBSLA_PR_REFERENCE || p->precision != TBSLA_F64) {
    // reference: b /= sum(b) (Matrix.cpp:52-59); mixed: sum-normalise
    const double keep_s = c.s;
    pr_mass_kernel<double><<<g, 256, 0, W->stream>>>(xr, n, nullptr, W->partials);
    pr_finalize_kernel<<<1, 256, 0, W->stream>>>(W->partials, g, W->ctl, 7);
    pr_scale_kernel<<<g, 256, 0, W->stream>>>(xr, n, &W->ctl->s);
    (void)keep_s;
  }
  if (d_out) TB_CUDA(cudaMemcpyAsync(d_out, xr, (size_t)n * 8, cudaMemcpyDeviceToDevice, W->stream));
  TB_CUDA(cudaGetLastError());
  TB_CUDA(cudaStreamSynchronize(W->stream));
  if (res) {
    TB_TRY(read_ctl(W));
    res->iterations = p->precision == TBSLA_F64 ? c.iter : f64_sweeps + inner_total;
    res->iterations_f64 = f64_sweeps;
    res->residual = c.resid;
    res->converged = c.converged;
  }
  return TBSLA_OK;
}

namespace tbsla {
tbsla_status_t ensure_transpose(tbsla_matrix *A, tbsla_matrix **T);
tbsla_status_t grad_values_f64(const tbsla_matrix *A, const double *a, const double *b, double scale, double *out,
                               cudaStream_t s);
}  // namespace tbsla

// The adjoint of the TBSLA_PR_TELEPORT fixed point (see tbsla_gb300.h).
static tbsla_status_t adjoint_impl(tbsla_matrix *A, const tbsla_pagerank_params_t *p, const double *d_v,
                                   const double *d_x, const double *d_w, double *d_gvals, double *d_gv,
                                   tbsla_pagerank_result_t *res, cudaStream_t user) {
  TB_CHECK(A && p && d_x && d_w, "NULL argument");
  TB_CHECK(A->format == TBSLA_FMT_CSR && A->csr_variant == 0, "the adjoint needs a CSR handle (default variant)");
  TB_CHECK(A->n_row == A->n_col && A->n_col > 0, "the adjoint needs a square matrix");
  TB_CHECK(A->values[0], "the adjoint needs the F64 value store");
  TB_CHECK(p->max_iter >= 0, "max_iter < 0");
  TB_CUDA(cudaSetDevice(A->device));
  PrWork *W = nullptr;
  TB_TRY(pr_setup(A, &W));
  tbsla_matrix *T = nullptr;
  TB_TRY(ensure_transpose(A, &T));
  TB_CHECK(fused_ok(T), "the transposed copy does not take the fused sweep");
  const int n = W->n;
  if (!W->lam[0]) {
    TB_TRY(pr_alloc((void **)&W->lam[0], (size_t)n * 8));
    TB_TRY(pr_alloc((void **)&W->lam[1], (size_t)n * 8));
  }
  const int nparts = std::max(sweep_parts(T, true), kAffineBlocks);
  if (W->adj_nparts < nparts) {
    if (W->adj_partials) cudaFree(W->adj_partials);
    W->adj_partials = nullptr;
    W->adj_nparts = 0;
    TB_TRY(pr_alloc((void **)&W->adj_partials, (size_t)nparts * 3 * 8));
    W->adj_nparts = nparts;
  }
  if (user) {
    cudaEvent_t ev;
    TB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, user);
    cudaStreamWaitEvent(W->stream, ev, 0);
    cudaEventDestroy(ev);
  }
  cudaStream_t s = W->stream;
  PrCtl &c = *W->ctl_host;
  std::memset(&c, 0, sizeof c);
  c.beta = p->beta;
  c.tol = p->tol;
  c.inv_n = 1.0 / n;
  c.max_iter = p->max_iter;
  c.done = p->max_iter == 0;
  TB_TRY(write_ctl(W));
  const int g = kAffineBlocks;
  TB_CUDA(cudaMemcpyAsync(W->lam[0], d_w, (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
  pr_dot_kernel<<<g, 256, 0, s>>>(W->lam[0], d_v, n, 1.0 / n, W->adj_partials);
  pr_finalize_kernel<<<1, 256, 0, s>>>(W->adj_partials, g, W->ctl, 11);
  TB_CUDA(cudaGetLastError());
  TB_CHECK(p->accel == 0 || p->accel == 1, "accel = %d not 0 or 1", p->accel);
  const bool accel = p->accel == 1;
  if (accel) TB_TRY(pr_aa_buffers(W));
  const int K = accel ? std::max(6, (p->check_every + 5) / 6 * 6) : p->check_every > 0 ? p->check_every : 8;
  int launched = 0;
  while (!c.done) {
    for (int k = 0; k < K; ++k, ++launched) {
      AdjEpi epi{};
      // accelerated: lambda stays in lam[0] (the combination), outputs go to
      // the ring slots; plain: ping-pong
      epi.y = accel ? W->ag[launched % 3] : W->lam[(launched + 1) & 1];
      epi.yold = accel ? W->lam[0] : W->lam[launched & 1];
      epi.w = d_w;
      epi.dmask = W->dmask;
      epi.v = d_v;
      epi.c1 = &W->ctl->add;
      epi.betap = &W->ctl->beta;
      epi.done = &W->ctl->done;
      epi.partials = W->adj_partials;
      epi.inv_n = 1.0 / n;
      epi.n = n;
      TB_TRY(launch_product<double, double>(T, static_cast<const double *>(T->values[0]), epi.yold, epi, s));
      pr_finalize_kernel<<<1, 256, 0, s>>>(W->adj_partials, sweep_parts(T, true), W->ctl, accel ? 15 : 10);
      if (accel) TB_TRY(enqueue_aa_step(W, W->lam[0], W->adj_partials, launched, s));
    }
    TB_CUDA(cudaGetLastError());
    TB_TRY(read_ctl(W));
  }
  const double *lam = accel ? (c.iter > 0 ? W->ag[(c.iter - 1) % 3] : W->lam[0]) : W->lam[c.iter & 1];
  if (d_gv) {
    // dL/dv = (beta * d . x + 1 - beta) * lambda (stage 9 leaves that factor in ctl->add)
    pr_mass_kernel<double><<<g, 256, 0, s>>>(d_x, n, W->dmask, W->adj_partials);
    pr_finalize_kernel<<<1, 256, 0, s>>>(W->adj_partials, g, W->ctl, 9);
    pr_scale_to_kernel<<<g, 256, 0, s>>>(lam, n, &W->ctl->add, d_gv);
    TB_CUDA(cudaGetLastError());
  }
  if (d_gvals) TB_TRY(grad_values_f64(A, lam, d_x, p->beta, d_gvals, s));
  TB_CUDA(cudaStreamSynchronize(s));
  if (res) {
    res->iterations = c.iter;
    res->iterations_f64 = c.iter;
    res->residual = c.resid;
    res->converged = c.converged;
  }
  return TBSLA_OK;
}

// PageRank of A, on its relabelled copy when there is one (pr_relabel.cu);
// *result points to the vector in A's labels (d_out, or a buffer of A's).
// The reference mode never takes the copy: relabelling reorders every row's
// sum and the block sums of the max-normalised residual, and the reference's
// iteration count (Matrix.cpp:13-114) moves with that order near epsilon.
static tbsla_status_t pagerank_entry(tbsla_matrix *A, const tbsla_pagerank_params_t *p, const int *nodes,
                                     int n_nodes, double *d_out, tbsla_pagerank_result_t *res, cudaStream_t user,
                                     const double **result, const double *d_teleport = nullptr) {
  TB_CHECK(A && p, "NULL argument");
  TB_CUDA(cudaSetDevice(A->device));
  tbsla_matrix *B = nullptr;
  if (!d_teleport && p->mode != TBSLA_PR_REFERENCE) TB_TRY(pr_relabelled(A, &B));
  if (!B) {
    TB_TRY(pagerank_impl(A, p, nodes, n_nodes, d_out, res, user, d_teleport));
    if (result) *result = d_out ? d_out : pr_result(static_cast<PrWork *>(A->pr_work));
    return TBSLA_OK;
  }
  const int n = A->n_row;
  std::vector<int> mapped;
  if (nodes) {
    mapped.resize((size_t)std::max(n_nodes, 0));
    for (int k = 0; k < n_nodes; ++k)
      mapped[(size_t)k] = nodes[k] >= 0 && nodes[k] < n ? A->pr_newid_host[(size_t)nodes[k]] : -1;
  }
  TB_TRY(pagerank_impl(B, p, nodes ? mapped.data() : nullptr, n_nodes, nullptr, res, user));
  PrWork *W = static_cast<PrWork *>(B->pr_work);
  double *out = d_out;
  if (!out) {
    if (!A->pr_out) TB_TRY(dev_alloc(A, (void **)&A->pr_out, (size_t)n * sizeof(double)));
    out = A->pr_out;
  }
  TB_TRY(pr_relabel_gather(A, pr_result(W), out, W->stream));
  TB_CUDA(cudaStreamSynchronize(W->stream));
  if (result) *result = out;
  return TBSLA_OK;
}

extern "C" {

tbsla_status_t tbsla_pagerank(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p, double *d_out,
                              tbsla_pagerank_result_t *result, void *stream) {
  return pagerank_entry(const_cast<tbsla_matrix *>(A), p, nullptr, 0, d_out, result, (cudaStream_t)stream,
                        nullptr);
}

tbsla_status_t tbsla_pagerank_teleport(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p,
                                       const double *d_v, double *d_out, tbsla_pagerank_result_t *result,
                                       void *stream) {
  TB_CHECK(p && d_v, "NULL argument");
  tbsla_pagerank_params_t q = *p;
  q.mode = TBSLA_PR_TELEPORT;
  q.precision = TBSLA_F64;
  return pagerank_entry(const_cast<tbsla_matrix *>(A), &q, nullptr, 0, d_out, result, (cudaStream_t)stream,
                        nullptr, d_v);
}

tbsla_status_t tbsla_pagerank_adjoint(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p,
                                      const double *d_v, const double *d_x, const double *d_w,
                                      double *d_grad_values, double *d_grad_v,
                                      tbsla_pagerank_result_t *result, void *stream) {
  return adjoint_impl(const_cast<tbsla_matrix *>(A), p, d_v, d_x, d_w, d_grad_values, d_grad_v, result,
                      (cudaStream_t)stream);
}

tbsla_status_t tbsla_pagerank_host(tbsla_matrix_t *A, const tbsla_pagerank_params_t *p, double *out,
                                   int64_t n_out, tbsla_pagerank_result_t *result) {
  TB_CHECK(A && out, "NULL argument");
  TB_CHECK(n_out >= A->n_col, "output has %lld entries, need %d", (long long)n_out, A->n_col);
  std::lock_guard<std::mutex> lk(A->host_mu);
  const double *r = nullptr;
  TB_TRY(pagerank_entry(A, p, nullptr, 0, nullptr, result, nullptr, &r));
  TB_CUDA(cudaMemcpy(out, r, (size_t)A->n_col * 8, cudaMemcpyDeviceToHost));
  return TBSLA_OK;
}

tbsla_status_t tbsla_personalized_pagerank_host(tbsla_matrix_t *A, const tbsla_pagerank_params_t *p,
                                                const int *nodes, int n_nodes, double *out, int64_t n_out,
                                                tbsla_pagerank_result_t *result) {
  TB_CHECK(A && out && nodes, "NULL argument");
  TB_CHECK(n_out >= A->n_col, "output has %lld entries, need %d", (long long)n_out, A->n_col);
  std::lock_guard<std::mutex> lk(A->host_mu);
  tbsla_pagerank_params_t q = *p;
  q.mode = TBSLA_PR_REFERENCE;
  q.precision = TBSLA_F64;
  const double *r = nullptr;
  TB_TRY(pagerank_entry(A, &q, nodes, n_nodes, nullptr, result, nullptr, &r));
  TB_CUDA(cudaMemcpy(out, r, (size_t)A->n_col * 8, cudaMemcpyDeviceToHost));
  return TBSLA_OK;
}

}  // extern "C"
