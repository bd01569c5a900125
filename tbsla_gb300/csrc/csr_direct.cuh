// csr_direct.cuh -- direct CSR SpMV kernels for sm_103a (the default CSR path).
//
// Rows are binned at creation by length:
//   short (<= kShortRow nonzeros), plain FP64 products of rows averaging at
//     least kPairMinRow entries: two lanes per row (csr_pair_kernel, below).
//   short, otherwise: one thread per row, walking its row in
//     chunks of eight entries with 16-byte loads straight from global memory.
//     Lanes of a warp hold neighbouring rows; the loads of one chunk are
//     issued together, so a sector's second use hits the line already in
//     flight in L1: L1 does the coalescing, no shared memory and no block
//     barrier are involved.  The row is summed in
//     its stored order with one FMA per nonzero (the order of
//     MatrixCSR::Ax, src/cpp/matrix/MatrixCSR.cpp:133-139).
//   long (<= kChunk): a group of L lanes per row, L = 4, 8, 16 or 32 by
//     length class (kGroupLimit), lanes striding the row, partial sums
//     combined with a fixed shuffle tree inside the group.
//   huge (> kChunk): the row is cut into chunks of kChunk nonzeros, 32 lanes
//     per chunk writing a partial; csr_chunk_fixup_kernel adds the partials of
//     each row in chunk order.
// The groups exist for the FP64 pipe (2 lane-operations per clock per SM on
// GB300; a warp instruction costs the same with 1 or 32 lanes active): one
// warp per row would spend ~10 FP64 warp instructions per row on its
// reduction and epilogue, more than the products of a 100-entry row.
// Row data is read through L1 with the default cache policy, the gathered x
// with a fractional evict-last L2 policy, y written with streaming stores.
// No atomics: results do not depend on scheduling.
#pragma once

#include <type_traits>

#include "spmv_kernels.cuh"

namespace tbsla {

constexpr int kShortRow = 32;
constexpr int kChunk = 8192;
// length classes of the long rows: class c takes rows of at most
// kGroupLimit[c] entries with kGroupLanes[c] lanes each (chunks: class 3)
constexpr int kGroupClasses = 4;
constexpr int kGroupLimit[kGroupClasses] = {96, 256, 1024, kChunk};
constexpr int kGroupLanes[kGroupClasses] = {4, 8, 16, 32};

__device__ __forceinline__ float bf16_lo(unsigned w) { return __bfloat162float(__ushort_as_bfloat16((unsigned short)(w & 0xffffu))); }
__device__ __forceinline__ float bf16_hi(unsigned w) { return __bfloat162float(__ushort_as_bfloat16((unsigned short)(w >> 16))); }

// eight entries from an 8-aligned index with 16-byte loads through L1 and the
// default cache policy (arrays carry 64 bytes of padding, so a group may run
// past the last entry).  A lane reads each sector in two pieces; L1/L2 keep
// the line between them.  Explicit L2 eviction hints were measured worse
// here: an evict-first hint lets L2 drop the line between the two reads
// (DRAM traffic x2.5), and 32-byte loads with an evict-normal policy ran 20%
// slower.  FP64 values and the column indices ask for 256-byte L2 prefetches:
// neutral at the default L2 fetch granularity, and they keep the streams
// wide when the process lowers it to 32 bytes for the gathers
// (tbsla_set_l2_fetch_granularity).
__device__ __forceinline__ void ld_vals8(const double *p, double (&v)[8]) {
  #pragma unroll
  for (int h = 0; h < 4; ++h)
    asm("ld.global.nc.L2::256B.v2.f64 {%0,%1}, [%2];" : "=d"(v[2 * h]), "=d"(v[2 * h + 1]) : "l"(p + 2 * h));
}
__device__ __forceinline__ void ld_vals8(const float *p, float (&v)[8]) {
  asm("ld.global.nc.L2::256B.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]) : "l"(p));
  asm("ld.global.nc.L2::256B.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]) : "l"(p + 4));
}
__device__ __forceinline__ void ld_vals8(const __nv_bfloat16 *p, float (&v)[8]) {
  unsigned w[4];
  asm("ld.global.nc.L2::256B.v4.u32 {%0,%1,%2,%3}, [%4];" : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]) : "l"(p));
  #pragma unroll
  for (int h = 0; h < 4; ++h) { v[2 * h] = bf16_lo(w[h]); v[2 * h + 1] = bf16_hi(w[h]); }
}
__device__ __forceinline__ void ld_cols8(const int *c, int (&col)[8]) {
  asm("ld.global.nc.L2::256B.v4.s32 {%0,%1,%2,%3}, [%4];" : "=r"(col[0]), "=r"(col[1]), "=r"(col[2]), "=r"(col[3]) : "l"(c));
  asm("ld.global.nc.L2::256B.v4.s32 {%0,%1,%2,%3}, [%4];" : "=r"(col[4]), "=r"(col[5]), "=r"(col[6]), "=r"(col[7]) : "l"(c + 4));
}
// two entries from an even index
__device__ __forceinline__ void ld_vals2(const double *p, double (&v)[2]) {
  const double2 d = __ldg(reinterpret_cast<const double2 *>(p));
  v[0] = d.x; v[1] = d.y;
}
__device__ __forceinline__ void ld_vals2(const float *p, float (&v)[2]) {
  const float2 d = __ldg(reinterpret_cast<const float2 *>(p));
  v[0] = d.x; v[1] = d.y;
}
__device__ __forceinline__ void ld_vals2(const __nv_bfloat16 *p, float (&v)[2]) {
  const unsigned w = __ldg(reinterpret_cast<const unsigned *>(p));
  v[0] = bf16_lo(w); v[1] = bf16_hi(w);
}

// One row, one thread.  Rows of eight or more entries go in groups of eight
// aligned to eight, all loads of a group issued together; shorter rows go in
// aligned pairs, which neighbouring lanes read as contiguous 16-byte pieces.
// Entries outside [a, b) of a group are masked (no gather, no FMA).  The row
// is summed in stored order, one FMA per entry.
template <int G, typename V, typename XT, typename Acc>
__device__ __forceinline__ Acc row_groups(const int *__restrict__ colidx, const V *__restrict__ values,
                                          const XT *__restrict__ x, int f_col, int a, int b, uint64_t keep) {
  using Ld = typename std::conditional<sizeof(V) == 8, double, float>::type;
  Acc acc = 0;
  for (int base = a & ~(G - 1); base < b; base += G) {
    Ld v[G];
    int col[G];
    if constexpr (G == 2) {
      ld_vals2(values + base, v);
      const int2 c = __ldg(reinterpret_cast<const int2 *>(colidx + base));
      col[0] = c.x; col[1] = c.y;
    } else {
      ld_vals8(values + base, v);
      ld_cols8(colidx + base, col);
    }
    Acc xv[G];
    #pragma unroll
    for (int e = 0; e < G; ++e) {
      const int k = base + e;
      xv[e] = (k >= a && k < b) ? to_acc(ld_keep(x + (col[e] - f_col), keep), Acc()) : Acc(0);
    }
    #pragma unroll
    for (int e = 0; e < G; ++e) {
      const int k = base + e;
      if (k >= a && k < b) acc = fma_acc((Acc)v[e], xv[e], acc);
    }
  }
  return acc;
}

template <typename V, typename XT, typename Acc>
__device__ __forceinline__ Acc row_sum_thread(const int *__restrict__ colidx, const V *__restrict__ values,
                                              const XT *__restrict__ x, int f_col, int a, int b,
                                              uint64_t keep) {
  if (b - a >= 8) return row_groups<8, V, XT, Acc>(colidx, values, x, f_col, a, b, keep);
  return row_groups<2, V, XT, Acc>(colidx, values, x, f_col, a, b, keep);
}

// short rows: rows [0, n_rows) when `rows` is NULL, else rows[0..n_rows);
// grid-stride (one row per thread unless the epilogue caps the grid)
template <typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(256) csr_short_kernel(const int *__restrict__ rows, int n_rows,
                                                       const int *__restrict__ rowptr,
                                                       const int *__restrict__ colidx,
                                                       const V *__restrict__ values,
                                                       const XT *__restrict__ x, int f_col, XKeep x_keep,
                                                       Epi epi) {
  using Acc = typename Epi::Acc;
  if (!epi.active()) return;
  typename Epi::State es{};
  const uint64_t keep = policy_keep(x_keep, x);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if constexpr (!Epi::kReduces) {
    // one row per thread (uncapped grid)
    for (; t < n_rows; t += stride) {
      const int r = rows ? __ldg(rows + t) : (int)t;
      const int a = __ldg(rowptr + r), b = __ldg(rowptr + r + 1);
      epi.emit(r, row_sum_thread<V, XT, Acc>(colidx, values, x, f_col, a, b, keep), es);
    }
  } else {
    // the next row's bounds are loaded before the current row is summed, so
    // their latency overlaps the sum (capped grids give a thread many rows)
    int r = 0, a = 0, b = 0;
    if (t < n_rows) {
      r = rows ? __ldg(rows + t) : (int)t;
      a = __ldg(rowptr + r);
      b = __ldg(rowptr + r + 1);
    }
    for (; t < n_rows; t += stride) {
      const int64_t tn = t + stride;
      int rn = 0, an = 0, bn = 0;
      if (tn < n_rows) {
        rn = rows ? __ldg(rows + tn) : (int)tn;
        an = __ldg(rowptr + rn);
        bn = __ldg(rowptr + rn + 1);
      }
      epi.emit(r, row_sum_thread<V, XT, Acc>(colidx, values, x, f_col, a, b, keep), es);
      r = rn;
      a = an;
      b = bn;
    }
  }
  epi.block_done(es, blockIdx.x);
}

// Short rows, two adjacent lanes per row: the row's aligned groups (of eight
// entries, or of two for rows under eight) are split in halves, each lane
// sums its half in stored order, and the row is first half + second half (a
// fixed order: results do not depend on scheduling, but round differently
// from the one-lane sum).  A warp's load instruction touches 16 rows' lines
// instead of 32, for one more FP64 add per row.
// the default uses the pairs for FP64 plain products when short rows
// average at least this many entries (cqmat c=16: 4889 vs 4378 GB/s with
// 32-byte L2 fetches; cdiag, 2 per row: 2516 vs 4647 -- a lane idles)
constexpr int kPairMinRow = 8;

template <typename V, typename XT, typename Acc>
__device__ __forceinline__ Acc row_half(const int *__restrict__ colidx, const V *__restrict__ values,
                                        const XT *__restrict__ x, int f_col, int a, int b, int half,
                                        uint64_t keep) {
  const int sh = b - a >= 8 ? 3 : 1;
  const int g0 = a >> sh, g1 = (b + (1 << sh) - 1) >> sh, gm = g0 + ((g1 - g0 + 1) >> 1);
  const int lo = half ? max(a, gm << sh) : a, hi = half ? b : min(b, gm << sh);
  if (lo >= hi) return Acc(0);
  if (sh == 3) return row_groups<8, V, XT, Acc>(colidx, values, x, f_col, lo, hi, keep);
  return row_groups<2, V, XT, Acc>(colidx, values, x, f_col, lo, hi, keep);
}

template <typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(256) csr_pair_kernel(const int *__restrict__ rows, int n_rows,
                                                      const int *__restrict__ rowptr,
                                                      const int *__restrict__ colidx,
                                                      const V *__restrict__ values,
                                                      const XT *__restrict__ x, int f_col, XKeep x_keep,
                                                      Epi epi) {
  using Acc = typename Epi::Acc;
  if (!epi.active()) return;
  typename Epi::State es{};
  const uint64_t keep = policy_keep(x_keep, x);
  const int half = threadIdx.x & 1;
  const unsigned pair = 3u << ((threadIdx.x & 31) & ~1);  // both lanes of a pair always run together
  const int64_t stride = ((int64_t)gridDim.x * blockDim.x) >> 1;
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 1; t < n_rows; t += stride) {
    const int r = rows ? __ldg(rows + t) : (int)t;
    const int a = __ldg(rowptr + r), b = __ldg(rowptr + r + 1);
    const Acc mine = row_half<V, XT, Acc>(colidx, values, x, f_col, a, b, half, keep);
    const Acc other = __shfl_xor_sync(pair, mine, 1);
    if (!half) epi.emit(r, mine + other, es);
  }
  epi.block_done(es, blockIdx.x);
}

// Tiny rows: every row in order and at most T entries (T = 2 or 4).  A warp
// takes a tile of 32 R rows (R = 8 / T), lane l rows l, l + 32, ..., so
// each load instruction covers 32 consecutive rows; a lane has the bounds,
// entries and gathers of its R rows in flight together (one row per thread
// leaves three dependent loads per row in flight: cdiag rows of two entries
// stayed latency-bound at two thirds of the HBM rate).  Each row is summed
// in stored order, one FMA per entry: the one-thread-per-row arithmetic.
// (kTinyRow, the longest row it takes, is in common.cuh.)

template <int T, typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(256) csr_tiny_kernel(int n_rows, const int *__restrict__ rowptr,
                                                      const int *__restrict__ colidx,
                                                      const V *__restrict__ values,
                                                      const XT *__restrict__ x, int f_col, XKeep x_keep,
                                                      Epi epi) {
  using Acc = typename Epi::Acc;
  constexpr int R = 8 / T;
  if (!epi.active()) return;
  typename Epi::State es{};
  const int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32 * (32 * R);
  if (base < n_rows) {
    const uint64_t keep = policy_keep(x_keep, x);
    const int r0 = (int)base + (threadIdx.x & 31);
    int a[R], b[R];
    #pragma unroll
    for (int q = 0; q < R; ++q) {
      const int r = r0 + 32 * q;
      a[q] = r < n_rows ? __ldg(rowptr + r) : 0;
      b[q] = r < n_rows ? __ldg(rowptr + r + 1) : 0;
    }
    V v[R][T];
    int c[R][T];
    #pragma unroll
    for (int q = 0; q < R; ++q) {
      #pragma unroll
      for (int t = 0; t < T; ++t) {
        const int k = a[q] + t;
        const bool in = k < b[q];
        c[q][t] = in ? ld_ell<false>(colidx + k) : f_col;  // read-only, 256-byte L2 prefetch
        v[q][t] = in ? ld_ell<false>(values + k) : V(0);
      }
    }
    Acc xv[R][T];
    #pragma unroll
    for (int q = 0; q < R; ++q) {
      #pragma unroll
      for (int t = 0; t < T; ++t)
        xv[q][t] = a[q] + t < b[q] ? to_acc(ld_keep(x + (c[q][t] - f_col), keep), Acc()) : Acc(0);
    }
    #pragma unroll
    for (int q = 0; q < R; ++q) {
      Acc acc = 0;
      #pragma unroll
      for (int t = 0; t < T; ++t)
        if (a[q] + t < b[q]) acc = fma_acc(to_acc(v[q][t], Acc()), xv[q][t], acc);
      if (r0 + 32 * q < n_rows) epi.emit(r0 + 32 * q, acc, es);
    }
  }
  epi.block_done(es, blockIdx.x);
}

// Tiny rows from a list: rows[0..n) each hold at most T entries (empty ones
// included), in any order.  As csr_tiny_kernel, a warp takes 32 R list
// entries, lane l entries l, l + 32, ..., with the bounds, entries and
// gathers of its R rows in flight together, but grid-stride over tiles, so
// that a reducing epilogue's capped grid covers the list; one thread per row
// would wait on each row's load chain in turn (PageRank sweeps on R-MAT:
// four fifths of the rows).  Each row is summed in stored order, one FMA per
// entry: the one-thread-per-row arithmetic.
constexpr int kTinyListRows = 2;  // R: rows per lane
inline int tiny_list_grid(int n, bool reduces) {
  const int g = (int)(((int64_t)n + 256 * kTinyListRows - 1) / (256 * kTinyListRows));
  return std::max(1, reduces ? std::min(g, 152 * 16) : g);
}

template <typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(256) csr_tiny_list_kernel(const int *__restrict__ rows, int n,
                                                           const int *__restrict__ rowptr,
                                                           const int *__restrict__ colidx,
                                                           const V *__restrict__ values,
                                                           const XT *__restrict__ x, int f_col, XKeep x_keep,
                                                           Epi epi) {
  using Acc = typename Epi::Acc;
  constexpr int R = kTinyListRows, T = kTinyRow;
  if (!epi.active()) return;
  typename Epi::State es{};
  const uint64_t keep = policy_keep(x_keep, x);
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (32 * R); base < n;
       base += nwarps * (32 * R)) {
    int r[R], a[R], b[R];
    #pragma unroll
    for (int q = 0; q < R; ++q) {
      const int64_t idx = base + lane + 32 * q;
      r[q] = idx < n ? __ldg(rows + idx) : -1;
    }
    #pragma unroll
    for (int q = 0; q < R; ++q) {
      a[q] = r[q] >= 0 ? __ldg(rowptr + r[q]) : 0;
      b[q] = r[q] >= 0 ? __ldg(rowptr + r[q] + 1) : 0;
    }
    V v[R][T];
    int c[R][T];
    #pragma unroll
    for (int q = 0; q < R; ++q) {
      #pragma unroll
      for (int t = 0; t < T; ++t) {
        const int k = a[q] + t;
        const bool in = k < b[q];
        c[q][t] = in ? ld_ell<false>(colidx + k) : f_col;
        v[q][t] = in ? ld_ell<false>(values + k) : V(0);
      }
    }
    Acc xv[R][T];
    #pragma unroll
    for (int q = 0; q < R; ++q) {
      #pragma unroll
      for (int t = 0; t < T; ++t)
        xv[q][t] = a[q] + t < b[q] ? to_acc(ld_keep(x + (c[q][t] - f_col), keep), Acc()) : Acc(0);
    }
    #pragma unroll
    for (int q = 0; q < R; ++q) {
      Acc acc = 0;
      #pragma unroll
      for (int t = 0; t < T; ++t)
        if (a[q] + t < b[q]) acc = fma_acc(to_acc(v[q][t], Acc()), xv[q][t], acc);
      if (r[q] >= 0) epi.emit(r[q], acc, es);
    }
  }
  epi.block_done(es, blockIdx.x);
}

// sum of entries [a, b) by a group of L lanes of one warp (L a power of two
// <= 32, groups aligned in the warp): lanes stride the range, fixed shuffle
// tree within the group.  Valid in the group's first lane.
template <int L, typename V, typename XT, typename Acc>
__device__ __forceinline__ Acc range_sum_group(const int *__restrict__ colidx, const V *__restrict__ values,
                                               const XT *__restrict__ x, int f_col, int a, int b, uint64_t keep) {
  const int lane = threadIdx.x & (L - 1);
  const unsigned mask = L == 32 ? 0xffffffffu : ((1u << (L & 31)) - 1u) << ((threadIdx.x & 31) & ~(L - 1));
  Acc acc = 0;
  #pragma unroll 4
  for (int k = a + lane; k < b; k += L)
    acc = fma_acc(to_acc(ld_stream(values + k), Acc()), to_acc(ld_keep(x + (ld_stream(colidx + k) - f_col), keep), Acc()), acc);
  #pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) acc += __shfl_down_sync(mask, acc, o, L);
  return acc;
}

// Rows longer than kShortRow and chunks of huge rows, L lanes per item:
// items[i] = (row, begin, end, partial slot or -1).  A warp holds 32/L
// groups, so its FP64 reduction steps and the epilogue serve 32/L rows at
// once (every FP64 warp instruction costs the same on this part whatever
// its active lanes).  Items come in length classes, so the groups of a warp
// take similar trip counts.
template <int L, typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(256) csr_group_kernel(const int4 *__restrict__ items, int n_items,
                                                       const int *__restrict__ colidx,
                                                       const V *__restrict__ values,
                                                       const XT *__restrict__ x, int f_col, XKeep x_keep,
                                                       typename Epi::Acc *__restrict__ partials, Epi epi) {
  using Acc = typename Epi::Acc;
  if (!epi.active()) return;
  typename Epi::State es{};
  const uint64_t keep = policy_keep(x_keep, x);
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / L;
  // every lane of a group sees the same item sequence (same trip count)
  int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / L;
  int4 it = g < n_items ? items[g] : make_int4(0, 0, 0, -1);
  for (; g < n_items; g += ng) {
    // next item loaded ahead (its latency overlaps this item's sum)
    const int4 nx = g + ng < n_items ? items[g + ng] : make_int4(0, 0, 0, -1);
    const Acc s = range_sum_group<L, V, XT, Acc>(colidx, values, x, f_col, it.y, it.z, keep);
    if ((threadIdx.x & (L - 1)) == 0) {
      if (it.w < 0) epi.emit(it.x, s, es);
      else partials[it.w] = s;
    }
    it = nx;
  }
  epi.block_done(es, blockIdx.x);
}

// ---------------------------------------------------------------- staged
// Matrices whose rows are all short (<= kShortRow entries).  A warp takes
// tiles of 32 consecutive rows; a tile's entries are contiguous, and the warp
// copies them into its slice of shared memory with lane-per-entry copies
// (each line of row data read by one instruction, evict-first in L2 so that
// the streamed matrix leaves L2 to x).  Then each lane sums its own row from
// shared memory in stored order, one FMA per entry (the direct kernel's
// arithmetic: results are bit-identical), gathering x with the kept-fraction
// policy.  Slots are XOR-swizzled within groups of 16 entries, so lanes
// reading rows of 16 entries hit distinct banks.  Warps work independently;
// the block meets only in the epilogue's reduction.  (Per-element cp.async
// copies into two buffers per warp, overlapping the next tile's copies with
// the current sum, measured 1.5x slower than these register copies.)
constexpr int kStageWarps = 8;
constexpr int kStageBatch = 8;                // loads in flight per lane
constexpr int kStageCapMax = 32 * kShortRow;  // a tile's entries when every row is short

template <typename T> __device__ __forceinline__ T ld_first(const T *p, uint64_t pol);
template <> __device__ __forceinline__ double ld_first<double>(const double *p, uint64_t pol) {
  double v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
template <> __device__ __forceinline__ float ld_first<float>(const float *p, uint64_t pol) {
  float v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}
template <> __device__ __forceinline__ int ld_first<int>(const int *p, uint64_t pol) {
  int v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.s32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
template <> __device__ __forceinline__ __nv_bfloat16 ld_first<__nv_bfloat16>(const __nv_bfloat16 *p, uint64_t pol) {
  unsigned short v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.u16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(pol));
  return __ushort_as_bfloat16(v);
}

__device__ __forceinline__ int stage_swz(int k) { return k ^ ((k >> 4) & 15); }

// dynamic shared memory of csr_stage_kernel for value type V and `cap` slots
template <typename V> constexpr size_t csr_stage_smem(int cap) {
  return (size_t)kStageWarps * cap * (sizeof(V) + sizeof(int));
}

// lane bounds of tile t: row r0+lane spans [lo, hi); lanes past the matrix
// (or a tile past the end) see empty rows
__device__ __forceinline__ void stage_bounds(const int *__restrict__ rowptr, int rows, int n_tiles, int t, int lane,
                                             int &lo, int &hi) {
  lo = hi = 0;
  if (t < n_tiles) {
    const int r0 = t << 5, nr = min(32, rows - r0);
    lo = __ldg(rowptr + r0 + min(lane, nr));
    hi = __ldg(rowptr + r0 + min(lane + 1, nr));
  }
}

template <typename V, typename XT, typename Acc>
__device__ __forceinline__ Acc stage_row_sum(const V *sv, const int *sc, int a, int b, const XT *__restrict__ x,
                                             int f_col, uint64_t keep) {
  Acc acc = 0;
  #pragma unroll 8
  for (int k = a; k < b; ++k) {
    const int sk = stage_swz(k);
    acc = fma_acc(to_acc(sv[sk], Acc()), to_acc(ld_keep(x + (sc[sk] - f_col), keep), Acc()), acc);
  }
  return acc;
}

template <typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(kStageWarps * 32) csr_stage_kernel(int rows, const int *__restrict__ rowptr,
                                                                    const int *__restrict__ colidx,
                                                                    const V *__restrict__ values,
                                                                    const XT *__restrict__ x, int f_col,
                                                                    XKeep x_keep, int cap, Epi epi) {
  using Acc = typename Epi::Acc;
  extern __shared__ __align__(16) unsigned char stage_smem[];
  if (!epi.active()) return;
  typename Epi::State es{};
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  V *sv = reinterpret_cast<V *>(stage_smem) + (size_t)wib * cap;
  int *sc = reinterpret_cast<int *>(stage_smem + (size_t)kStageWarps * cap * sizeof(V)) + (size_t)wib * cap;
  const uint64_t keep = policy_keep(x_keep, x), first = policy_evict_first();
  const int n_tiles = (rows + 31) >> 5;
  const int nw = gridDim.x * kStageWarps;
  int t = blockIdx.x * kStageWarps + wib;
  for (; t < n_tiles; t += nw) {
    int lo, hi;
    stage_bounds(rowptr, rows, n_tiles, t, lane, lo, hi);
    const int e0 = __shfl_sync(0xffffffffu, lo, 0), e1 = __shfl_sync(0xffffffffu, hi, 31);
    const int n = e1 - e0;  // <= cap by construction
    for (int k0 = 0; k0 < n; k0 += 32 * kStageBatch) {
      V v[kStageBatch];
      int c[kStageBatch];
      #pragma unroll
      for (int u = 0; u < kStageBatch; ++u) {
        const int k = k0 + u * 32 + lane;
        if (k < n) {
          v[u] = ld_first(values + e0 + k, first);
          c[u] = ld_first(colidx + e0 + k, first);
        }
      }
      #pragma unroll
      for (int u = 0; u < kStageBatch; ++u) {
        const int k = k0 + u * 32 + lane;
        if (k < n) {
          sv[stage_swz(k)] = v[u];
          sc[stage_swz(k)] = c[u];
        }
      }
    }
    __syncwarp();
    const Acc acc = stage_row_sum<V, XT, Acc>(sv, sc, lo - e0, hi - e0, x, f_col, keep);
    if ((t << 5) + lane < rows) epi.emit((t << 5) + lane, acc, es);
    __syncwarp();  // the next tile's copies overwrite the slots
  }
  epi.block_done(es, blockIdx.x);
}

// y[row] = sum of the row's chunk partials in chunk order;
// huge[h] = (row, first slot), huge[n_huge].y = total slots
template <typename Epi>
__global__ void csr_chunk_fixup_kernel(const int2 *__restrict__ huge, int n_huge,
                                       const typename Epi::Acc *__restrict__ partials, Epi epi) {
  using Acc = typename Epi::Acc;
  if (!epi.active()) return;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  typename Epi::State es{};
  if (h < n_huge) {
    const int row = huge[h].x, first = huge[h].y, last = huge[h + 1].y;
    Acc s = partials[first];
    for (int c = first + 1; c < last; ++c) s += partials[c];
    epi.emit(row, s, es);
  }
  epi.fixup_done(es, blockIdx.x);
}


// ------------------------------------------------------- sliced copy
// Every row short, few padded slots: a copy of the entries in ELL layout,
// slot j of every row stored together (rows padded to a multiple of 128,
// width = the longest row; padded slots hold column -1).  One warp per 32 R
// rows, lane l taking rows l, l + 32, ...: each slot's indices and values
// are R fully used 32-entry runs, and the gathers of neighbouring rows' band
// entries fall on neighbouring addresses.  Padded slots are skipped.  R = 2
// by default (two independent loads per slot and thread).  Each row is summed in its stored order, one FMA per entry (the
// order of MatrixCSR::Ax, src/cpp/matrix/MatrixCSR.cpp:133-139).
constexpr int kSellRows = 128;

template <int R, typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(256) csr_sell_kernel(const int *__restrict__ cols, const V *__restrict__ vals,
                                                      int64_t stride, int width, const XT *__restrict__ x,
                                                      int f_col, int rows, XKeep x_keep, Epi epi) {
  using Acc = typename Epi::Acc;
  if (!epi.active()) return;
  const int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32 * (32 * R);
  const int lane = threadIdx.x & 31;
  typename Epi::State es{};
  if (base < rows) {
    const uint64_t keep = policy_keep(x_keep, x);
    const int r0 = (int)base + lane;
    Acc a[R];
    #pragma unroll
    for (int q = 0; q < R; ++q) a[q] = 0;
    #pragma unroll 4
    for (int j = 0; j < width; ++j) {
      const size_t off = (size_t)j * stride + r0;
      int c[R];
      V v[R];
      #pragma unroll
      for (int q = 0; q < R; ++q) {
        c[q] = ld_ell<false>(cols + off + 32 * q);
        v[q] = ld_ell<false>(vals + off + 32 * q);
      }
      #pragma unroll
      for (int q = 0; q < R; ++q)
        if (c[q] >= 0) a[q] = fma_acc(to_acc(v[q], Acc()), to_acc(ld_keep(x + (c[q] - f_col), keep), Acc()), a[q]);
    }
    #pragma unroll
    for (int q = 0; q < R; ++q)
      if (r0 + 32 * q < rows) epi.emit(r0 + 32 * q, a[q], es);
  }
  epi.block_done(es, blockIdx.x);
}

// the sliced copy of one array: entry rowptr[r] + j to slot j * stride + r
// (one thread per row)
template <typename T>
__global__ void sell_scatter_kernel(const int *__restrict__ rowptr, int64_t stride, int rows,
                                    const T *__restrict__ src, T *__restrict__ dst) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    const int a = rowptr[r], b = rowptr[r + 1];
    for (int j = 0; j < b - a; ++j) dst[(size_t)j * stride + r] = src[a + j];
  }
}

}  // namespace tbsla
