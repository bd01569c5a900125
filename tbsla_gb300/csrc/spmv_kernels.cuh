// spmv_kernels.cuh -- sm_103a SpMV kernels for the five TBSLA formats.
//
// COO uses a merge-path decomposition: every thread consumes exactly
// kMergeItems nonzeros from a tile of kMergeTile entries staged in shared
// memory, accumulating its rows sequentially with one FMA per nonzero.  A row that spans several threads
// is finished by the thread where it ends, which adds the partial sums of the
// earlier threads in path order; a row that spans tiles is finished by
// merge_fixup_kernel from the per-tile head/tail partials.  No atomics: the
// result does not depend on scheduling.
//
// ELL is stored column-major (slot-major) and read with 16-byte vector loads,
// four rows per thread, each row summed in slot order exactly as
// MatrixELL::Ax (src/cpp/matrix/MatrixELL.cpp:101-114) orders it.
// DENSE is a row-major GEMV, four rows per warp.
//
// The products are written through an epilogue functor `Epi` that receives
// each finished row once:  epi.emit(row, value, state).
#pragma once

#include "common.cuh"

namespace tbsla {

template <typename Acc> struct Carry {
  int *head_row;            // row continued from an earlier tile, or -1
  Acc *head_val;            // its partial sum over this tile
  Acc *tail_val;            // partial sum of the tile's last row
  unsigned char *emitted;   // the tile finished at least one row
};

// ------------------------------------------------------------ epilogues
template <typename YT, typename AccT> struct StoreEpi {
  using Acc = AccT;
  static constexpr bool kReduces = false;  // no per-block partials
  struct State {};
  YT *y;
  int n_out;   // rows that may be written
  int shift;   // output row = row + shift (COO vect_incr)
  __device__ __forceinline__ void emit(int row, Acc v, State &) const {
    int o = row + shift;
    if (o >= 0 && o < n_out) __stcs(y + o, (YT)v);  // streaming: keep L2 for x
  }
  __device__ __forceinline__ bool active() const { return true; }
  __host__ __device__ void set_part_base(int) {}
  __device__ __forceinline__ void block_done(State &, int) const {}
  __device__ __forceinline__ void fixup_done(State &, int) const {}
};

// y = A x + x  (the first half of Matrix::a_axpx_, Matrix.cpp:6-11)
template <typename AccT> struct AddXEpi {
  using Acc = AccT;
  static constexpr bool kReduces = false;
  struct State {};
  double *y;
  const double *x;
  int n_out;
  int shift;
  __device__ __forceinline__ void emit(int row, Acc v, State &) const {
    int o = row + shift;
    if (o >= 0 && o < n_out) __stcs(y + o, (double)v + x[o]);
  }
  __device__ __forceinline__ bool active() const { return true; }
  __host__ __device__ void set_part_base(int) {}
  __device__ __forceinline__ void block_done(State &, int) const {}
  __device__ __forceinline__ void fixup_done(State &, int) const {}
};

// --------------------------------------------------------- block helpers
// deterministic block-wide sum / max of one value per thread (fixed tree)
template <int NT, typename T> __device__ __forceinline__ T block_sum(T v, T *scratch) {
  #pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) scratch[w] = v;
  __syncthreads();
  T r = 0;
  if (threadIdx.x == 0) {
    #pragma unroll
    for (int k = 0; k < NT / 32; ++k) r += scratch[k];
  }
  return r;  // valid in thread 0
}

template <int NT> __device__ __forceinline__ int block_max_int(int v, int *scratch) {
  #pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) scratch[w] = v;
  __syncthreads();
  int r = scratch[0];
  #pragma unroll
  for (int k = 1; k < NT / 32; ++k) r = max(r, scratch[k]);
  return r;  // valid in every thread
}

// Resolves the rows that cross thread boundaries inside one tile and writes
// the tile's carries.  Called by all threads after each stored its tail
// partial (s_tail) and whether it finished a row (s_emit).
template <int NT, typename Epi>
__device__ __forceinline__ void resolve_tile(int tile, bool deferred, int first_row,
                                             typename Epi::Acc first_val, bool tile_starts_mid,
                                             typename Epi::Acc *s_tail, unsigned char *s_emit,
                                             int *s_misc, typename Epi::Acc *s_red,
                                             Carry<typename Epi::Acc> carry, const Epi &epi,
                                             typename Epi::State &es) {
  using Acc = typename Epi::Acc;
  if (threadIdx.x == 0) s_misc[0] = -1;
  __syncthreads();
  if (deferred) {
    int u = (int)threadIdx.x - 1;
    while (u >= 0 && !s_emit[u]) --u;
    Acc s = 0;
    for (int v = u < 0 ? 0 : u; v < (int)threadIdx.x; ++v) s += s_tail[v];
    s += first_val;
    if (u >= 0 || !tile_starts_mid) {
      epi.emit(first_row, s, es);
    } else {
      s_misc[0] = first_row;
      s_red[NT / 32] = s;  // head value (slot after the reduction scratch)
    }
  }
  // the tile's tail: sum of the partials from the last thread that finished a
  // row up to the end of the tile
  const int last = block_max_int<NT>(s_emit[threadIdx.x] ? (int)threadIdx.x : -1, s_misc + 1);
  Acc mine = ((int)threadIdx.x >= (last < 0 ? 0 : last)) ? s_tail[threadIdx.x] : Acc(0);
  Acc tail = block_sum<NT, Acc>(mine, s_red);
  if (threadIdx.x == 0) {
    const int hr = s_misc[0];
    carry.head_row[tile] = hr;
    if (hr >= 0) carry.head_val[tile] = s_red[NT / 32];
    carry.tail_val[tile] = tail;
    carry.emitted[tile] = last >= 0;
  }
}

// Stages n (<= NT*K) consecutive nonzeros of a tile in shared memory: the
// values, and the gathered x[col - f_col] in the accumulator type.  Thread k
// takes nonzeros k, k+NT, ...: the index and value loads are coalesced, all K
// gathers of a thread are in flight together, and neighbouring threads
// gather neighbouring columns of a row (band entries are consecutive).
template <int NT, int K, typename V, typename XT, typename Acc>
__device__ __forceinline__ void stage_tile(const V *__restrict__ vals, const int *__restrict__ cols,
                                           const XT *__restrict__ x, int f_col, int n, V *s_val,
                                           Acc *s_x) {
  const uint64_t keep = policy_evict_last();
  int c[K];
  #pragma unroll
  for (int u = 0; u < K; ++u) {
    const int k = threadIdx.x + u * NT;
    c[u] = k < n ? ld_stream(cols + k) : f_col;
  }
  #pragma unroll
  for (int u = 0; u < K; ++u) {
    const int k = threadIdx.x + u * NT;
    if (k < n) {
      s_val[k] = ld_stream(vals + k);
      s_x[k] = to_acc(ld_keep(x + (c[u] - f_col), keep), Acc());
    }
  }
}

// rows that span tiles: the tile where the row ends adds the tails of the
// tiles before it (path order) to its head partial
template <typename Epi>
__global__ void merge_fixup_kernel(int num_tiles, Carry<typename Epi::Acc> carry, Epi epi) {
  using Acc = typename Epi::Acc;
  if (!epi.active()) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  typename Epi::State es{};
  if (t < num_tiles) {
    const int r = carry.head_row[t];
    if (r >= 0) {
      int u = t - 1;
      while (u >= 0 && !carry.emitted[u]) --u;
      Acc s = 0;
      for (int v = u < 0 ? 0 : u; v < t; ++v) s += carry.tail_val[v];
      s += carry.head_val[t];
      epi.emit(r, s, es);
    }
  }
  epi.fixup_done(es, blockIdx.x);
}

// --------------------------------------------------------------- COO
// Row-sorted triplets.  Tile t holds entries [t*TILE, (t+1)*TILE).
template <int NT, int K, typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(NT) coo_merge_kernel(const int *__restrict__ rowv,
                                                       const int *__restrict__ colv,
                                                       const V *__restrict__ values,
                                                       const XT *__restrict__ x, int f_col,
                                                       int64_t nnz, Carry<typename Epi::Acc> carry,
                                                       Epi epi) {
  using Acc = typename Epi::Acc;
  constexpr int TILE = NT * K;
  __shared__ int s_row[TILE];
  __shared__ V s_val[TILE];
  __shared__ Acc s_x[TILE];
  __shared__ Acc s_tail[NT];
  __shared__ Acc s_red[NT / 32 + 1];
  __shared__ unsigned char s_emit[NT];
  __shared__ int s_misc[NT / 32 + 2];

  if (!epi.active()) return;
  const int t = blockIdx.x;
  const int64_t e0 = (int64_t)t * TILE;
  const int n_t = (int)min((int64_t)TILE, nnz - e0);
  for (int k = threadIdx.x; k < n_t; k += NT) s_row[k] = ld_stream(rowv + e0 + k);
  stage_tile<NT, K, V, XT, Acc>(values + e0, colv + e0, x, f_col, n_t, s_val, s_x);
  const int prev_row = e0 > 0 ? rowv[e0 - 1] : -1;
  __syncthreads();

  const int b = min((int)threadIdx.x * K, n_t);
  const int n_items = min(b + K, n_t) - b;
  // row of the entry after this tile (INT_MIN past the last entry)
  const int next_tile_row = (e0 + n_t < nnz) ? rowv[e0 + n_t] : INT_MIN;
  typename Epi::State es{};
  Acc acc = 0, first_val = 0;
  bool emitted = false, deferred = false;
  int first_row = -1;
  const int before = b > 0 ? s_row[b - 1] : prev_row;
  const bool starts_mid = n_items > 0 && before == s_row[b];
  #pragma unroll
  for (int k = 0; k < K; ++k) {
    if (k < n_items) {
      const int e = b + k;
      const int r = s_row[e];
      acc = fma_acc(to_acc(s_val[e], Acc()), s_x[e], acc);
      const int nr = (e + 1 < n_t) ? s_row[e + 1] : next_tile_row;
      if (nr != r) {  // the row ends at entry e
        if (!emitted && starts_mid) { deferred = true; first_row = r; first_val = acc; }
        else epi.emit(r, acc, es);
        emitted = true;
        acc = 0;
      }
    }
  }
  s_tail[threadIdx.x] = acc;
  s_emit[threadIdx.x] = emitted;
  const bool tile_starts_mid = n_t > 0 && prev_row == s_row[0];
  resolve_tile<NT, Epi>(t, deferred, first_row, first_val, tile_starts_mid, s_tail, s_emit, s_misc,
                        s_red, carry, epi, es);
  epi.block_done(es, t);
}

// --------------------------------------------------------------- ELL
// Column-major ELL: slot s of row i at [s*rows_pad + i].  Four rows per
// thread; padding (column 0, value 0) is multiplied like any entry, and a
// column below f_col reads x[0], as the reference does.
template <typename V> struct Vec4 { V v[4]; };

// Streaming (.cs, evict-first) loads when x stays in L2; default loads when
// x is larger than L2, where evict-first row data measured slower (ELL FP64
// cqmat 2^24: 3.6 vs 4.0 TB/s; 2^22: 5.95 vs 5.68 TB/s).
// ELL row data: streaming (.cs) or read-only loads, both asking for 256-byte
// L2 prefetches (streams stay wide at a 32-byte L2 fetch granularity)
template <bool CS> __device__ __forceinline__ double2 ld_row(const double2 *p) {
  double2 v;
  if constexpr (CS) asm("ld.global.cs.L2::256B.v2.f64 {%0,%1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  else asm("ld.global.nc.L2::256B.v2.f64 {%0,%1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  return v;
}
template <bool CS> __device__ __forceinline__ float4 ld_row(const float4 *p) {
  float4 v;
  if constexpr (CS)
    asm("ld.global.cs.L2::256B.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  else
    asm("ld.global.nc.L2::256B.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  return v;
}
template <bool CS> __device__ __forceinline__ uint2 ld_row(const uint2 *p) {
  uint2 v;
  if constexpr (CS) asm("ld.global.cs.L2::256B.v2.u32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
  else asm("ld.global.nc.L2::256B.v2.u32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
  return v;
}
template <bool CS> __device__ __forceinline__ int4 ld_row(const int4 *p) {
  int4 v;
  if constexpr (CS)
    asm("ld.global.cs.L2::256B.v4.s32 {%0,%1,%2,%3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
  else
    asm("ld.global.nc.L2::256B.v4.s32 {%0,%1,%2,%3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
  return v;
}

template <typename V, bool CS = true> __device__ __forceinline__ Vec4<V> ld4(const V *p) {
  Vec4<V> r;
  if constexpr (sizeof(V) == 8) {
    const double2 a = ld_row<CS>(reinterpret_cast<const double2 *>(p));
    const double2 b = ld_row<CS>(reinterpret_cast<const double2 *>(p) + 1);
    r.v[0] = a.x; r.v[1] = a.y; r.v[2] = b.x; r.v[3] = b.y;
  } else if constexpr (sizeof(V) == 4) {
    const float4 a = ld_row<CS>(reinterpret_cast<const float4 *>(p));
    r.v[0] = a.x; r.v[1] = a.y; r.v[2] = a.z; r.v[3] = a.w;
  } else {
    const uint2 a = ld_row<CS>(reinterpret_cast<const uint2 *>(p));
    r.v[0] = __ushort_as_bfloat16((unsigned short)(a.x & 0xffffu));
    r.v[1] = __ushort_as_bfloat16((unsigned short)(a.x >> 16));
    r.v[2] = __ushort_as_bfloat16((unsigned short)(a.y & 0xffffu));
    r.v[3] = __ushort_as_bfloat16((unsigned short)(a.y >> 16));
  }
  return r;
}

template <typename V, typename XT, typename Epi, bool CS>
__global__ void __launch_bounds__(256) ell_kernel(const int *__restrict__ cols,
                                                  const V *__restrict__ vals,
                                                  const XT *__restrict__ x, int f_col, int rows,
                                                  int rows_pad, int max_col, XKeep x_keep, Epi epi) {
  using Acc = typename Epi::Acc;
  if (!epi.active()) return;
  const int r0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
  typename Epi::State es{};
  if (r0 < rows) {
    const uint64_t keep = policy_keep(x_keep, x);
    Acc a[4] = {0, 0, 0, 0};
    #pragma unroll 4
    for (int s = 0; s < max_col; ++s) {
      const size_t off = (size_t)s * rows_pad + r0;
      const int4 c = ld_row<CS>(reinterpret_cast<const int4 *>(cols + off));
      const Vec4<V> v = ld4<V, CS>(vals + off);
      const int cc[4] = {c.x, c.y, c.z, c.w};
      #pragma unroll
      for (int q = 0; q < 4; ++q) {
        int idx = cc[q] - f_col;
        if (idx < 0) idx = 0;
        a[q] = fma_acc(to_acc(v.v[q], Acc()), to_acc(ld_keep(x + idx, keep), Acc()), a[q]);
      }
    }
    #pragma unroll
    for (int q = 0; q < 4; ++q)
      if (r0 + q < rows) epi.emit(r0 + q, a[q], es);
  }
  epi.block_done(es, blockIdx.x);
}

// Warp tiles of 128 rows: lane l of a warp sums rows base + l + 32 q
// (q = 0..3), slot by slot in stored order (the arithmetic of ell_kernel, so
// results are bit-identical).  Each load instruction covers 32 consecutive
// rows: the column and value loads stay coalesced (two 128-byte lines per
// FP64 instruction) and the gathers of a banded matrix touch the lines of 32
// neighbouring rows, a quarter of the lines of ell_kernel's four
// consecutive rows per thread (whose 32 lanes span 128 rows per gather).
template <bool CS, typename T> __device__ __forceinline__ T ld_ell(const T *p);
template <> __device__ __forceinline__ int ld_ell<true, int>(const int *p) { return ld_stream(p); }
template <> __device__ __forceinline__ double ld_ell<true, double>(const double *p) { return ld_stream(p); }
template <> __device__ __forceinline__ float ld_ell<true, float>(const float *p) { return ld_stream(p); }
template <> __device__ __forceinline__ __nv_bfloat16 ld_ell<true, __nv_bfloat16>(const __nv_bfloat16 *p) {
  return ld_stream(p);
}
template <> __device__ __forceinline__ int ld_ell<false, int>(const int *p) {
  int v;
  asm("ld.global.nc.L2::256B.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
template <> __device__ __forceinline__ double ld_ell<false, double>(const double *p) {
  double v;
  asm("ld.global.nc.L2::256B.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
template <> __device__ __forceinline__ float ld_ell<false, float>(const float *p) {
  float v;
  asm("ld.global.nc.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
template <> __device__ __forceinline__ __nv_bfloat16 ld_ell<false, __nv_bfloat16>(const __nv_bfloat16 *p) {
  unsigned short u;
  asm("ld.global.nc.L2::256B.u16 %0, [%1];" : "=h"(u) : "l"(p));
  return __ushort_as_bfloat16(u);
}

template <typename V, typename XT, typename Epi, bool CS, int R = 4>
__global__ void __launch_bounds__(256) ell_warp_kernel(const int *__restrict__ cols,
                                                       const V *__restrict__ vals,
                                                       const XT *__restrict__ x, int f_col, int rows,
                                                       int rows_pad, int max_col, XKeep x_keep, Epi epi) {
  using Acc = typename Epi::Acc;
  if (!epi.active()) return;
  const int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32 * (32 * R);
  const int lane = threadIdx.x & 31;
  typename Epi::State es{};
  if (base < rows) {
    const uint64_t keep = policy_keep(x_keep, x);
    const int r0 = (int)base + lane;
    bool in[R];
    #pragma unroll
    for (int q = 0; q < R; ++q) in[q] = r0 + 32 * q < rows;
    Acc a[R];
    #pragma unroll
    for (int q = 0; q < R; ++q) a[q] = 0;
    #pragma unroll 4
    for (int s = 0; s < max_col; ++s) {
      const size_t off = (size_t)s * rows_pad + r0;
      int c[R];
      V v[R];
      #pragma unroll
      for (int q = 0; q < R; ++q) {
        c[q] = in[q] ? ld_ell<CS>(cols + off + 32 * q) : 0;
        v[q] = in[q] ? ld_ell<CS>(vals + off + 32 * q) : V(0);
      }
      #pragma unroll
      for (int q = 0; q < R; ++q) {
        int idx = c[q] - f_col;
        if (idx < 0) idx = 0;
        if (in[q]) a[q] = fma_acc(to_acc(v[q], Acc()), to_acc(ld_keep(x + idx, keep), Acc()), a[q]);
      }
    }
    #pragma unroll
    for (int q = 0; q < R; ++q)
      if (in[q]) epi.emit(r0 + 32 * q, a[q], es);
  }
  epi.block_done(es, blockIdx.x);
}

// --------------------------------------------------------------- DENSE
// Row-major GEMV: each warp handles four rows at once so that every x chunk
// loaded serves four rows; lanes stride over the columns, then the warp
// reduces each row with a fixed shuffle tree.
template <typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(256) dense_kernel(const V *__restrict__ a,
                                                    const XT *__restrict__ x, int rows, int cols,
                                                    Epi epi) {
  using Acc = typename Epi::Acc;
  constexpr int RW = 4;
  if (!epi.active()) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int r0 = warp * RW;
  typename Epi::State es{};
  if (r0 < rows) {
    Acc acc[RW] = {0, 0, 0, 0};
    const V *rowp[RW];
    #pragma unroll
    for (int q = 0; q < RW; ++q) rowp[q] = a + (size_t)min(r0 + q, rows - 1) * cols;
    int j = lane;
    for (; j < cols; j += 32) {
      const Acc xv = to_acc(ld_vec(x + j), Acc());
      #pragma unroll
      for (int q = 0; q < RW; ++q) acc[q] = fma_acc(to_acc(ld_stream(rowp[q] + j), Acc()), xv, acc[q]);
    }
    #pragma unroll
    for (int q = 0; q < RW; ++q) {
      Acc v = acc[q];
      #pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0 && r0 + q < rows) epi.emit(r0 + q, v, es);
    }
  }
  epi.block_done(es, blockIdx.x);
}

}  // namespace tbsla
