// common.cuh -- shared definitions of the tbsla_gb300 library: the matrix
// handle, error reporting, and small device helpers.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/tbsla_gb300.h"

namespace tbsla {

// ---------------------------------------------------------------- errors
tbsla_status_t fail(tbsla_status_t s, const char *fmt, ...);
tbsla_status_t cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define TB_CUDA(call)                                                           \
  do {                                                                          \
    cudaError_t tb_e_ = (call);                                                 \
    if (tb_e_ != cudaSuccess) return ::tbsla::cuda_fail(tb_e_, #call, __FILE__, __LINE__); \
  } while (0)

#define TB_CHECK(cond, ...)                                                     \
  do {                                                                          \
    if (!(cond)) return ::tbsla::fail(TBSLA_ERR_INVALID_ARG, __VA_ARGS__);      \
  } while (0)

#define TB_TRY(...)                                                             \
  do {                                                                          \
    tbsla_status_t tb_s_ = (__VA_ARGS__);                                       \
    if (tb_s_ != TBSLA_OK) return tb_s_;                                        \
  } while (0)

// ------------------------------------------------------------- constants
// merge-path tiling of CSR / COO: threads per CTA and items per thread.
// Items per thread is odd so that consecutive-item shared-memory reads of 4-
// and 8-byte words are free of bank conflicts.
constexpr int kMergeThreads = 256;
constexpr int kMergeItems = 9;
constexpr int kMergeTile = kMergeThreads * kMergeItems;

// -------------------------------------------------------------- handle
struct DeviceBuffer {
  void *ptr = nullptr;
  size_t bytes = 0;
};

}  // namespace tbsla

namespace tbsla {
// rows of at most this many entries, all in order: csr_tiny_kernel
constexpr int kTinyRow = 4;
}  // namespace tbsla

// The opaque matrix handle of the C ABI.
struct tbsla_matrix {
  int format = 0;
  int n_row = 0, n_col = 0;
  int f_row = 0, f_col = 0;
  int rows = 0;          // rows visited by the kernels
  int cols = 0;          // DENSE: ln_col
  int max_col = 0;       // ELL width
  int64_t stored = 0;    // stored entries
  int stores = 0;        // TBSLA_STORE_* bits
  int device = 0;

  // values in up to three precisions (F64, F32, BF16), same positions
  void *values[3] = {nullptr, nullptr, nullptr};
  // CSR: rowptr (rows+1 ints, base removed); ELL: column-major columns
  // (rows_pad * max_col); COO: row (stored)
  int *idx0 = nullptr;
  // CSR: colidx; COO: col
  int *idx1 = nullptr;
  int rows_pad = 0;      // ELL: padded row count of the column-major arrays
  int64_t x_extent = 0;  // entries of x the kernels read (max column - f_col + 1)

  // CSR kernel variant: 0 = direct (row bins), 1 = row blocks.  COO / SCOO:
  // 0 = the direct CSR kernels over coo_rowptr, 1 = merge path
  int csr_variant = 0;
  // COO / SCOO: row pointer of the row-sorted entries (n_row + 1), with the
  // row bins of the direct kernels built from it
  int *coo_rowptr = nullptr;
  // fraction of the gathered vector's lines loaded with L2 evict-last
  // priority by the direct CSR kernels (tbsla_matrix_tune)
  float x_keep = 0.6f;
  // 1: the kept fraction is the leading part of x by address (range policy)
  int x_keep_range = 0;
  // CSR direct bins (csr_direct.cuh): short rows (NULL = all rows), warp
  // items (long rows and chunks of huge rows), huge rows, chunk partials
  int *short_rows = nullptr;
  int n_short = 0;
  // the first n_tiny entries of short_rows hold every short row of at most
  // kTinyRow entries (empty ones included), when there are many of them:
  // reducing epilogues (PageRank sweeps) run them in warp tiles
  int n_tiny = 0;
  int64_t short_nnz = 0;  // entries of the short rows
  int short_max = 0;      // entries of the longest short row (<= kTinyRow, all rows
                          // short and in order: the tiny-row warp tiles)
  // all rows short: shared-memory slots per warp of the staged kernel (the
  // entries of the largest 32-row tile, a multiple of 16); 0 otherwise
  int stage_cap = 0;
  // short-row kernel (tbsla_matrix_tune): 0 one thread per row, 1 staged
  // tiles (every row short), 2 two lanes per row, 3 the sliced copy, -1
  // (default) the sliced copy for plain products when it exists, else two
  // lanes for plain products of FP64 values when short rows average at least
  // kPairMinRow entries, one thread per row otherwise
  int short_mode = -1;
  // sliced copy of the entries (csr_sell_kernel): ELL layout, slot j of row
  // r at j * sell_stride + r, sell_width slots, padding column -1; built when
  // every row is short and padding adds little (csr_bins), kept for the F64
  // and F32 value stores (sell_vals[k] mirrors values[k]; [2] stays NULL)
  int *sell_cols = nullptr;
  void *sell_vals[3] = {nullptr, nullptr, nullptr};
  int64_t sell_stride = 0;  // rows rounded up to a multiple of 128
  int sell_width = 0;       // slots per row (the longest row); 0: no copy
  int sell_rows = 0;        // rows per thread of csr_sell_kernel (1, 2, 4; 0: by size)
  int4 *warp_items = nullptr;
  int n_warp_items = 0;
  int item_class_start[5] = {0, 0, 0, 0, 0};  // items of length class c: [start[c], start[c+1])
  int2 *chunk_rows = nullptr;
  int n_chunk_rows = 0;
  double *chunk_partials = nullptr;
  float *chunk_partials32 = nullptr;

  // CSR row blocks (csr_rows_kernel): descriptors, huge rows, chunk partials
  int num_blocks = 0;
  int4 *row_blocks = nullptr;
  int num_huge = 0;
  int2 *huge_rows = nullptr;         // (row, first partial slot), num_huge + 1
  double *huge_partials = nullptr;
  float *huge_partials32 = nullptr;

  // merge-path tiles (COO): tile count and carries
  int num_tiles = 0;
  int2 *tile_start = nullptr;
  int *tile_head_row = nullptr; // per tile: row continued from an earlier tile, or -1
  double *tile_head_val = nullptr;
  double *tile_tail_val = nullptr;
  unsigned char *tile_emitted = nullptr;
  float *tile_head_val32 = nullptr;  // FP32-accumulating variants
  float *tile_tail_val32 = nullptr;
  int *d_err = nullptr;              // set by a kernel whose bounded wait gave up
  int tc_split = 0;                  // DENSE tensor-core product: K splits (0: chosen per call)

  // PageRank workspace built on first use (pagerank.cu)
  void *pr_work = nullptr;
  void (*pr_work_free)(void *) = nullptr;
  unsigned char *dangling = nullptr;
  double *pr_scratch = nullptr;
  // PageRank on a relabelled copy (pr_relabel.cu): vertices in decreasing
  // out-degree order, so that the hot entries of the gathered iterate share
  // cache lines
  int pr_relabel_mode = -1;          // tbsla_matrix_tune: -1 auto, 0 off, 1 on
  int pr_relabel_state = 0;          // 0 undecided, 1 built, 2 declined
  tbsla_matrix *pr_relabel = nullptr;
  int *pr_newid = nullptr;           // new label of each vertex (device)
  std::vector<int> pr_newid_host;    // the same on the host (node lists)
  double *pr_out = nullptr;          // result in the original labels (device)
  // transposed copy (transpose.cu), built on first use: entry k' of the copy
  // holds entry transpose_perm[k'] of this matrix
  tbsla_matrix *transpose = nullptr;
  int *transpose_perm = nullptr;
  // batched PageRank tile width chosen by tbsla_autotune_ppr (F64, F32); 0: none
  int ppr_tile[2] = {0, 0};
  // batched PageRank work list built on first use (ppr_batch.cu; depends on
  // the row structure only)
  void *ppr_plan = nullptr;
  void (*ppr_plan_free)(void *) = nullptr;

  // host-path staging
  cudaStream_t stream = nullptr;
  double *d_x = nullptr, *d_y = nullptr, *d_t = nullptr;
  int64_t cap_x = 0, cap_y = 0, cap_t = 0;

  int64_t device_bytes = 0;
  std::mutex host_mu;

  // optional per-launch timing of the main product kernel
  bool timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending_events;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> free_events;
  double timed_ms = 0;
  int64_t timed_launches = 0;
};

namespace tbsla {

tbsla_status_t dev_alloc(tbsla_matrix *A, void **p, size_t bytes);
// brackets the main kernel of a product when A->timing is set
struct KernelTimer {
  tbsla_matrix *A;
  cudaStream_t s;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  KernelTimer(const tbsla_matrix *A_, cudaStream_t s_);
  void stop();
};
tbsla_status_t ensure_host_buffers(tbsla_matrix *A, int64_t nx, int64_t ny, int64_t nt);
int current_device();

inline int store_index(tbsla_dtype_t t) { return t == TBSLA_F64 ? 0 : (t == TBSLA_F32 ? 1 : 2); }

// ------------------------------------------------------- device helpers
template <typename T> struct AccOf { using type = float; };
template <> struct AccOf<double> { using type = double; };

__device__ __forceinline__ double to_acc(double v, double) { return v; }
__device__ __forceinline__ float to_acc(float v, float) { return v; }
__device__ __forceinline__ float to_acc(__nv_bfloat16 v, float) { return __bfloat162float(v); }
__device__ __forceinline__ float to_acc(double v, float) { return (float)v; }
__device__ __forceinline__ double to_acc(float v, double) { return (double)v; }

// fused multiply-add in the accumulator type
__device__ __forceinline__ double fma_acc(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_acc(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// streaming loads of matrix data (read once: evict-first in L2 so that the
// gathered vector stays resident)
// (256-byte L2 prefetches: streams stay wide when the process lowers the L2
// fetch granularity for gathers, tbsla_set_l2_fetch_granularity)
template <typename T> __device__ __forceinline__ T ld_stream(const T *p);
template <> __device__ __forceinline__ double ld_stream(const double *p) {
  double v;
  asm("ld.global.cs.L2::256B.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
template <> __device__ __forceinline__ float ld_stream(const float *p) {
  float v;
  asm("ld.global.cs.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
template <> __device__ __forceinline__ int ld_stream(const int *p) {
  int v;
  asm("ld.global.cs.L2::256B.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
template <> __device__ __forceinline__ __nv_bfloat16 ld_stream(const __nv_bfloat16 *p) {
  unsigned short u;
  asm("ld.global.cs.L2::256B.u16 %0, [%1];" : "=h"(u) : "l"(p));
  return __ushort_as_bfloat16(u);
}

// L2 cache policies (createpolicy): evict-last for the gathered vector
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// evict-last for a fraction f of the lines it touches (the others keep their
// priority); f <= 0 gives normal priority throughout.  Used on the gathered
// vector: when x is about as large as L2, protecting all of it leaves no room
// for the streamed matrix lines, which are then fetched again.
__device__ __forceinline__ uint64_t policy_keep(float f) {
  uint64_t p;
  if (f >= 1.f)
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  else if (f > 0.f)
    asm volatile("createpolicy.fractional.L2::evict_last.L2::evict_unchanged.b64 %0, %1;" : "=l"(p) : "f"(f));
  else
    asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// What the kernels keep of the gathered vector: a fraction of its lines
// (fractional policy), or, when `range` is the vector's size in bytes, the
// first `frac` of its addresses (range policy: the same lines every time).
struct XKeep {
  float frac;
  uint32_t range;
};
__device__ __forceinline__ uint64_t policy_keep(XKeep k, const void *x) {
  if (k.range == 0 || k.frac <= 0.f) return policy_keep(k.frac);
  const uint32_t primary = (uint32_t)fminf((float)k.range, k.frac * (float)k.range);
  uint64_t p;
  asm volatile("createpolicy.range.global.L2::evict_last.L2::evict_unchanged.b64 %0, [%1], %2, %3;"
               : "=l"(p)
               : "l"(x), "r"(primary), "r"(k.range));
  return p;
}

__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ uint64_t policy_evict_normal() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// asynchronous 4/8-byte copies global -> shared (cp.async), with an L2 policy
__device__ __forceinline__ void cp_async(void *smem, const void *gmem, uint64_t pol, int bytes) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
  if (bytes == 8)
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 8, %2;" ::"r"(d), "l"(gmem), "l"(pol)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 4, %2;" ::"r"(d), "l"(gmem), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most N of this thread's committed groups are pending
template <int N> __device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <typename T> __device__ __forceinline__ T ld_keep(const T *p, uint64_t pol);
template <> __device__ __forceinline__ double ld_keep<double>(const double *p, uint64_t pol) {
  double v;
  asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
template <> __device__ __forceinline__ float ld_keep<float>(const float *p, uint64_t pol) {
  float v;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}

// gathered vector loads (read-only path)
template <typename T> __device__ __forceinline__ T ld_vec(const T *p) { return __ldg(p); }

template <typename T> __device__ __forceinline__ void st_out(T *p, double v) { *p = (T)v; }
template <typename T> __device__ __forceinline__ void st_out(T *p, float v) { *p = (T)v; }

}  // namespace tbsla
