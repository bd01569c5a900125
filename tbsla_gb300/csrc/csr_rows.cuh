// csr_rows.cuh -- row-block CSR SpMV for sm_103a (kernel variant 1 of CSR handles,
// tbsla_matrix_set_variant; the direct kernels of csr_direct.cuh are the default).
//
// The matrix is cut at creation into blocks of whole rows holding at most
// kRowsMax rows, kRowsMax segments (a segment: at most kSeg consecutive
// nonzeros of one row) and kRowsCap nonzeros; a row longer than kRowsCap is
// a "huge" row cut into chunks of kRowsCap nonzeros, one block each.
//
// Per block (one CTA):
//   1. stage: the block's contiguous nonzero range is read with coalesced
//      loads (matrix data evict-first in L2), every thread's loads in flight
//      together, then x[col] is gathered (x kept evict-last in L2); values
//      and gathered x go to shared memory under an XOR swizzle (swz) that
//      keeps rows kSeg apart in different banks;
//   2. consume: each thread sums its segments sequentially (one FMA per
//      nonzero, the row's own order); a row of several segments adds its
//      segment sums in order; y is written with streaming stores.
// Huge-row chunks write their sum to a partials array; csr_huge_fixup_kernel
// adds the chunks of each huge row in order.  No atomics anywhere.
#pragma once

#include "spmv_kernels.cuh"

namespace tbsla {

constexpr int kRowsNT = 256;                 // threads per block
constexpr int kRowsPT = 4;                   // rows and segments per thread
constexpr int kRowsMax = kRowsNT * kRowsPT;  // rows and segments per block
constexpr int kSeg = 16;                     // nonzeros per segment
constexpr int kRowsEPT = 16;                 // staged nonzeros per thread
constexpr int kRowsCap = kRowsNT * kRowsEPT; // nonzeros per block

// dynamic shared memory of csr_rows_kernel for accumulator type Acc
template <typename Acc> constexpr size_t csr_rows_smem() {
  return 2 * kRowsCap * sizeof(Acc) + (2 * (kRowsMax + 1) + kRowsNT / 32) * sizeof(int);
}

// Shared-memory slot of staged entry k: an XOR swizzle inside each group of
// 16 entries, so that threads reading entries 16 apart (rows of one segment
// each) hit different banks while consecutive entries stay a permutation of
// one 16-entry group.
__device__ __forceinline__ int swz(int k) { return k ^ ((k >> 4) & 15); }

// block descriptor: rows [x, y), nonzeros from z; w = -1 for a block of
// whole rows, else the partials slot of this chunk of huge row x
using RowBlock = int4;

template <typename V, typename XT, typename Epi>
__global__ void __launch_bounds__(kRowsNT, 3) csr_rows_kernel(const RowBlock *__restrict__ blocks,
                                                             const int *__restrict__ rowptr,
                                                             const int *__restrict__ colidx,
                                                             const V *__restrict__ values,
                                                             const XT *__restrict__ x, int f_col,
                                                             typename Epi::Acc *__restrict__ partials, Epi epi) {
  using Acc = typename Epi::Acc;
  constexpr int NT = kRowsNT, CAP = kRowsCap, RPT = kRowsPT;
  extern __shared__ __align__(16) unsigned char rows_smem[];
  Acc *s_val = reinterpret_cast<Acc *>(rows_smem);
  Acc *s_x = s_val + CAP;
  int *s_rp = reinterpret_cast<int *>(s_x + CAP);
  int *s_seg = s_rp + kRowsMax + 1;   // first segment of each row (exclusive scan)
  int *s_wsum = s_seg + kRowsMax + 1;
  Acc *s_part = s_val;                // segment sums, after the staged data is consumed

  if (!epi.active()) return;
  const RowBlock d = blocks[blockIdx.x];
  const int r0 = d.x, r1 = d.y, j0 = d.z, huge = d.w;
  const int nrows = r1 - r0;
  int j1;
  if (huge < 0) {
    for (int k = threadIdx.x; k <= nrows; k += NT) s_rp[k] = rowptr[r0 + k];
    j1 = rowptr[r1];
  } else {
    j1 = min(j0 + CAP, rowptr[r0 + 1]);
  }
  const int n = j1 - j0;

  // ---- stage: entry k = t + u*NT of the block.  Column indices come to
  // registers (coalesced); values and the gathered x[col] go straight to
  // shared memory with cp.async, so every copy of a thread is in flight at
  // once without holding registers (values evict-first, x evict-last in L2).
  {
    const uint64_t keep = policy_evict_last();
    int c[kRowsEPT];
    #pragma unroll
    for (int u = 0; u < kRowsEPT; ++u) {
      const int k = threadIdx.x + u * NT;
      c[u] = k < n ? ld_stream(colidx + j0 + k) : f_col;
    }
    if constexpr (sizeof(V) == sizeof(Acc) && sizeof(XT) == sizeof(Acc)) {
      const uint64_t stream = policy_evict_first();
      #pragma unroll
      for (int u = 0; u < kRowsEPT; ++u) {
        const int k = threadIdx.x + u * NT;
        if (k < n) cp_async(s_val + swz(k), values + j0 + k, stream, (int)sizeof(Acc));
      }
      #pragma unroll
      for (int u = 0; u < kRowsEPT; ++u) {
        const int k = threadIdx.x + u * NT;
        if (k < n) cp_async(s_x + swz(k), x + (c[u] - f_col), keep, (int)sizeof(Acc));
      }
      cp_async_wait_all();
    } else {
      #pragma unroll
      for (int u = 0; u < kRowsEPT; ++u) {
        const int k = threadIdx.x + u * NT;
        if (k < n) {
          const int sk = swz(k);
          s_x[sk] = to_acc(ld_keep(x + (c[u] - f_col), keep), Acc());
          s_val[sk] = to_acc(ld_stream(values + j0 + k), Acc());
        }
      }
    }
  }
  __syncthreads();
  typename Epi::State es{};

  if (huge >= 0) {
    // one chunk of a huge row: segments of kSeg, summed in order by thread 0
    const int a = threadIdx.x * kSeg, b = min(a + kSeg, n);
    Acc acc = 0;
    for (int k = a; k < b; ++k) acc = fma_acc(s_val[swz(k)], s_x[swz(k)], acc);
    __syncthreads();
    s_part[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      const int nseg = (n + kSeg - 1) / kSeg;
      Acc s = s_part[0];
      for (int t = 1; t < nseg; ++t) s += s_part[t];
      partials[huge] = s;
    }
    epi.block_done(es, blockIdx.x);
    return;
  }

  // ---- segments: thread t owns rows RPT*t .. RPT*t+RPT-1 for the scan
  int nseg[RPT], sum = 0;
  #pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int i = threadIdx.x * RPT + q;
    nseg[q] = 0;
    if (i < nrows) {
      const int len = s_rp[i + 1] - s_rp[i];
      nseg[q] = len > kSeg ? (len + kSeg - 1) / kSeg : 1;
    }
    sum += nseg[q];
  }
  int incl = sum;
  #pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if ((threadIdx.x & 31) >= o) incl += t;
  }
  if ((threadIdx.x & 31) == 31) s_wsum[threadIdx.x >> 5] = incl;
  __syncthreads();
  int base = incl - sum;
  #pragma unroll
  for (int w = 0; w < NT / 32; ++w) base += (w < (int)(threadIdx.x >> 5)) ? s_wsum[w] : 0;
  #pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int i = threadIdx.x * RPT + q;
    if (i < nrows) s_seg[i] = base;
    base += nseg[q];
  }
  if (threadIdx.x == NT - 1) s_seg[nrows] = base;
  __syncthreads();
  const int total_seg = s_seg[nrows];

  // ---- thread t sums segments t, t+NT, ... sequentially (the row's order)
  Acc acc[RPT];
  #pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int g = threadIdx.x + q * NT;
    acc[q] = 0;
    if (g < total_seg) {
      int lo = 0, hi = nrows - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_seg[mid] <= g) lo = mid; else hi = mid - 1;
      }
      const int a = s_rp[lo] - j0 + (g - s_seg[lo]) * kSeg;
      const int b = min(a + kSeg, s_rp[lo + 1] - j0);
      Acc t = 0;
      #pragma unroll 4
      for (int k = a; k < b; ++k) t = fma_acc(s_val[swz(k)], s_x[swz(k)], t);
      acc[q] = t;
    }
  }
  __syncthreads();
  #pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int g = threadIdx.x + q * NT;
    if (g < total_seg) s_part[g] = acc[q];
  }
  __syncthreads();
  // ---- rows t, t+NT, ...: add the row's segment sums in order
  #pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int i = threadIdx.x + q * NT;
    if (i < nrows) {
      const int b0 = s_seg[i], b1 = s_seg[i + 1];
      Acc s = s_part[b0];
      for (int t = b0 + 1; t < b1; ++t) s += s_part[t];
      epi.emit(r0 + i, s, es);
    }
  }
  epi.block_done(es, blockIdx.x);
}

// y[row] = sum of the row's chunk partials, in chunk order
template <typename Epi>
__global__ void csr_huge_fixup_kernel(const int2 *__restrict__ huge_rows, int n_huge,
                                      const typename Epi::Acc *__restrict__ partials, Epi epi) {
  using Acc = typename Epi::Acc;
  if (!epi.active()) return;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  typename Epi::State es{};
  if (h < n_huge) {
    const int row = huge_rows[h].x, first = huge_rows[h].y, last = huge_rows[h + 1].y;
    Acc s = partials[first];
    for (int c = first + 1; c < last; ++c) s += partials[c];
    epi.emit(row, s, es);
  }
  epi.fixup_done(es, blockIdx.x);
}

}  // namespace tbsla
