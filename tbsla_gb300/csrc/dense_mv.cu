// dense_mv.cu -- the multi-vector DENSE product Y = A X (k right-hand
// sides, each a product MatrixDENSE::Ax of src/cpp/matrix/MatrixDENSE.cpp:64-73).
//
// F32 and BF16 value stores run on the 5th-generation tensor cores with a
// kernel written here (dense_tc_kernel): per CTA a tile of 128 rows of A
// times up to 256 vectors, A and X staged in shared memory by TMA
// (cp.async.bulk.tensor, 128-byte swizzle, a ring of stages guarded by
// mbarriers), tcgen05.mma kind::f16 (BF16 A and X) or kind::tf32 (F32 A and
// X) issued by one thread with FP32 accumulation in TMEM, read back with
// tcgen05.ld by four epilogue warps.  A is streamed once; at k <= 64 vectors
// the product is bound by HBM (64 flops per byte of BF16 A), not by the
// tensor cores.  K is split into parts when the row tiles alone do not fill
// the GPU; the parts' FP32 partial sums are added in part order by a second
// kernel, so results do not depend on scheduling.
//
// The F64 store stays on the FP64 pipe: cuBLAS DGEMM (a plain library GEMM;
// GB300's FP64 tensor rate is no faster than its FP64 pipe).
#include <cublas_v2.h>
#include <cuda.h>

#include <algorithm>
#include <map>
#include <mutex>

#include "common.cuh"
#include "driver.cuh"
#include "tc_ptx.cuh"

namespace {

using namespace tbsla;

std::mutex g_mu;
std::map<int, cublasHandle_t> g_handles;

tbsla_status_t handle_for(int device, cublasHandle_t *h) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_handles.find(device);
  if (it != g_handles.end()) {
    *h = it->second;
    return TBSLA_OK;
  }
  cublasHandle_t c = nullptr;
  if (cublasCreate(&c) != CUBLAS_STATUS_SUCCESS) return tbsla::fail(TBSLA_ERR_CUDA, "cublasCreate failed");
  g_handles[device] = c;
  *h = c;
  return TBSLA_OK;
}

// ----------------------------------------------------------- tensor cores
constexpr int kTileM = 128;    // rows of A per CTA (the MMA's M)
constexpr int kRowBytes = 128; // K bytes per stage row: one 128-byte swizzle span
constexpr int kTcThreads = 192;

struct TcParams {
  int M;                // rows of A
  int nvec;             // vectors (columns of Y) in total
  int kb_total;         // K blocks of kRowBytes
  int kb_per_split;     // K blocks per part (every part holds at least one)
  float *out;           // Y (one part) or the parts' partial sums
  int64_t ld_out;       // distance between vectors in out
  int64_t split_stride; // distance between parts in out
  int *err;             // raised when a bounded wait gave up
  int a_early;          // A is not written by the stream's previous kernels:
                        // its first stages load before the dependency wait
};

template <int N> struct TcShape {
  static constexpr int kA = kTileM * kRowBytes;  // bytes of A per stage
  static constexpr int kB = N * kRowBytes;       // bytes of X per stage
  // stages: about 96 KB (two CTAs per SM) up to N = 64, about 192 KB above
  static constexpr int kStages = N <= 64 ? (96 * 1024) / (kA + kB) : (192 * 1024) / (kA + kB);
  static constexpr int kTmemCols = N < 32 ? 32 : N;
  static constexpr int kSmem = kStages * (kA + kB) + 1024 + 256;
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "MMA N for M = 128: a multiple of 16 in [16, 256]");
  static_assert(kStages >= 2, "at least two stages");
};

// Y[:, panel] (or part blockIdx.y's partial sums) for the row tile blockIdx.x
// and the vector panel blockIdx.z.  Warp 0 lane 0 loads (TMA), warp 1 owns
// TMEM and its lane 0 issues the MMAs, warps 2-5 move the accumulators out.
template <int N, uint32_t Fmt>
__global__ void __launch_bounds__(kTcThreads, 1)
    dense_tc_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_x,
                    TcParams p) {
  using S = TcShape<N>;
  constexpr int ST = S::kStages;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *sa = smem;
  uint8_t *sx = smem + ST * S::kA;
  uint64_t *full = reinterpret_cast<uint64_t *>(sx + ST * S::kB);
  uint64_t *empty = full + ST;
  uint64_t *done = empty + ST;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int m0 = blockIdx.x * kTileM;
  const int part = blockIdx.y;
  const int vec0 = blockIdx.z * N;
  const int kb0 = part * p.kb_per_split;
  const int nkb = min(p.kb_total - kb0, p.kb_per_split);

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      tc::mbar_init(full + s, 1);
      tc::mbar_init(empty + s, 1);
    }
    tc::mbar_init(done, 1);
    *abort = 0;
    tc::fence_barrier_init();
    tc::tma_prefetch_map(&map_a);
    tc::tma_prefetch_map(&map_x);
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, S::kTmemCols);
  tc::tc_fence_before_sync();
  __syncthreads();
  tc::tc_fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer: stage s holds K block i (i % ST == s) of A's row tile and of
    // the vector panel
    const uint64_t pol_a = tc::policy_evict_first(), pol_x = tc::policy_evict_last();
    constexpr int kElems = kRowBytes / (Fmt == tc::kFmtBF16 ? 2 : 4);
    // A of the first stages may load while the kernel that writes X (or any
    // earlier kernel of the stream) finishes; X only after the dependency wait
    const int pre = p.a_early ? min(ST, nkb) : 0;
    for (int i = 0; i < pre; ++i) {
      tc::mbar_arrive_expect_tx(full + i, S::kA + S::kB);
      tc::tma_load_2d(sa + i * S::kA, &map_a, full + i, (kb0 + i) * kElems, m0, pol_a);
    }
    tc::grid_dependency_wait();
    int issued = 0;
    for (int i = 0; i < nkb; ++i) {
      const int s = i % ST;
      const int kx = (kb0 + i) * kElems;
      if (i >= pre) {
        if (i >= ST && !tc::mbar_wait(empty + s, ((i / ST) - 1) & 1, abort)) break;
        tc::mbar_arrive_expect_tx(full + s, S::kA + S::kB);
        tc::tma_load_2d(sa + s * S::kA, &map_a, full + s, kx, m0, pol_a);
      }
      tc::tma_load_2d(sx + s * S::kB, &map_x, full + s, kx, vec0, pol_x);
      ++issued;
    }
    if (*abort)  // let the loads already issued land before the CTA leaves
      for (int j = max(0, issued - ST); j < issued; ++j) tc::mbar_wait(full + j % ST, (j / ST) & 1, abort, true);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: four 32-byte K steps per stage into the TMEM accumulator
    constexpr uint32_t idesc = tc::mma_idesc(Fmt, kTileM, N);
    for (int i = 0; i < nkb; ++i) {
      const int s = i % ST;
      if (!tc::mbar_wait(full + s, (i / ST) & 1, abort)) break;
      tc::tc_fence_after_sync();
      const uint32_t a = tc::smem_addr(sa + s * S::kA), x = tc::smem_addr(sx + s * S::kB);
#pragma unroll
      for (int k = 0; k < kRowBytes / 32; ++k)
        tc::mma<Fmt>(tmem, tc::sw128_kmajor_desc(a + 32 * k), tc::sw128_kmajor_desc(x + 32 * k), idesc,
                     (i > 0 || k > 0) ? 1u : 0u);
      tc::mma_commit(empty + s);  // stage s is free once these MMAs have read it
    }
    tc::mma_commit(done);  // every MMA issued has completed
  } else if (warp >= 2) {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 = rows of the tile
    const int q = warp & 3;
    const bool ok = tc::mbar_wait(done, 0, abort, true);
    tc::tc_fence_after_sync();
    tc::grid_dependency_wait();  // the stream's earlier kernels are done with Y
    const int go = __shfl_sync(0xffffffffu, (ok && !*abort) ? 1 : 0, 0);
    if (go) {
      const int row = m0 + q * 32 + lane;
      float *out = p.out + (int64_t)part * p.split_stride;
#pragma unroll 1
      for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        tc::tmem_load16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
        if (row < p.M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int c = vec0 + c0 + j;
            if (c < p.nvec) out[(int64_t)c * p.ld_out + row] = v[j];
          }
        }
      }
    }
  }
  tc::tc_fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after_sync();
    tc::tmem_dealloc(tmem, S::kTmemCols);
  }
  if (threadIdx.x == 0 && *abort && p.err) atomicExch(p.err, 1);
}

// Y[c*ldy + r] = sum over parts (in part order) of P[part][c*M + r]
__global__ void split_sum_kernel(const float *__restrict__ P, int parts, int M, int nvec, int64_t part_stride,
                                 float *__restrict__ Y, int64_t ldy) {
  const int64_t total = (int64_t)M * nvec;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    float s = P[t];
    for (int k = 1; k < parts; ++k) s += P[(int64_t)k * part_stride + t];
    const int64_t c = t / M, r = t % M;
    Y[c * ldy + r] = s;
  }
}

// X (FP32 column-major, ldx) rounded to BF16, vector c at out + c * ldo:
// blockIdx.y walks the vectors, x four entries per thread (one 16-byte load
// and one 8-byte store when both vectors start on such boundaries).  Lets the
// next kernel launch at once (it waits for this one before reading X).
__global__ void x_to_bf16_kernel(const float *__restrict__ x, int rows, int k, int64_t ldx,
                                 __nv_bfloat16 *__restrict__ out, int64_t ldo, int vec4) {
  tc::grid_launch_dependents();
  for (int c = blockIdx.y; c < k; c += gridDim.y) {
    const float *xc = x + (int64_t)c * ldx;
    __nv_bfloat16 *oc = out + (int64_t)c * ldo;
    for (int r = 4 * (blockIdx.x * blockDim.x + threadIdx.x); r < rows; r += 4 * gridDim.x * blockDim.x) {
      if (vec4 && r + 4 <= rows) {
        const float4 v = *reinterpret_cast<const float4 *>(xc + r);
        __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
        uint2 w;
        w.x = *reinterpret_cast<uint32_t *>(&lo);
        w.y = *reinterpret_cast<uint32_t *>(&hi);
        *reinterpret_cast<uint2 *>(oc + r) = w;
      } else {
        for (int j = r; j < min(r + 4, rows); ++j) oc[j] = __float2bfloat16_rn(xc[j]);
      }
    }
  }
}

// rows x cols row-major (ld src_ld) copied to ld dst_ld (element size es)
__global__ void pad_rows_kernel(const uint8_t *__restrict__ src, int64_t rows, int64_t row_bytes, int64_t src_ld,
                                uint8_t *__restrict__ dst, int64_t dst_ld) {
  const int64_t total = rows * row_bytes;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / row_bytes, b = t % row_bytes;
    dst[r * dst_ld + b] = src[r * src_ld + b];
  }
}

tbsla_status_t encode_map(CUtensorMap *map, bool bf16, const void *base, int64_t inner, int64_t outer,
                          int64_t ld_bytes, int box_outer) {
  const DriverApi *d = nullptr;
  TB_TRY(driver_api(&d));
  const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  const cuuint64_t strides[1] = {(cuuint64_t)ld_bytes};
  const cuuint32_t box[2] = {(cuuint32_t)(kRowBytes / (bf16 ? 2 : 4)), (cuuint32_t)box_outer};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = d->tensor_map_encode_tiled(
      map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base),
      dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(TBSLA_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return TBSLA_OK;
}

template <int N, uint32_t Fmt>
tbsla_status_t launch_tc(const CUtensorMap &ma, const CUtensorMap &mx, const TcParams &p, int m_tiles, int parts,
                         int panels, cudaStream_t s) {
  using Sh = TcShape<N>;
  static std::once_flag once[2];
  static cudaError_t attr_err[2];
  std::call_once(once[Fmt == tc::kFmtBF16 ? 0 : 1], [] {
    attr_err[Fmt == tc::kFmtBF16 ? 0 : 1] =
        cudaFuncSetAttribute(dense_tc_kernel<N, Fmt>, cudaFuncAttributeMaxDynamicSharedMemorySize, Sh::kSmem);
  });
  TB_CUDA(attr_err[Fmt == tc::kFmtBF16 ? 0 : 1]);
  // programmatic dependent launch: the kernel may start while the stream's
  // previous kernel finishes; it waits for it (griddepcontrol.wait) before
  // loading X or storing Y
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(m_tiles, parts, panels);
  cfg.blockDim = dim3(kTcThreads);
  cfg.dynamicSmemBytes = Sh::kSmem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  TB_CUDA(cudaLaunchKernelEx(&cfg, dense_tc_kernel<N, Fmt>, ma, mx, p));
  return TBSLA_OK;
}

template <uint32_t Fmt>
tbsla_status_t launch_tc_n(int n_pad, const CUtensorMap &ma, const CUtensorMap &mx, const TcParams &p, int m_tiles,
                           int parts, int panels, cudaStream_t s) {
  switch (n_pad) {
  case 16: return launch_tc<16, Fmt>(ma, mx, p, m_tiles, parts, panels, s);
  case 32: return launch_tc<32, Fmt>(ma, mx, p, m_tiles, parts, panels, s);
  case 64: return launch_tc<64, Fmt>(ma, mx, p, m_tiles, parts, panels, s);
  case 128: return launch_tc<128, Fmt>(ma, mx, p, m_tiles, parts, panels, s);
  default: return launch_tc<256, Fmt>(ma, mx, p, m_tiles, parts, panels, s);
  }
}

// K parts: doubled only while the row tiles and panels leave SMs idle and
// every part keeps at least 16 K blocks.  A split costs a pass over the
// parts' partial sums; with every SM holding a tile the stages already keep
// HBM busy (n = 32768, k = 64, BF16: 0.350 ms whole, 0.358 / 0.371 / 0.388 ms
// in 2 / 4 / 8 parts)
int choose_parts(int m_tiles, int panels, int kb_total, int sms) {
  int parts = 1;
  while ((int64_t)m_tiles * panels * parts < sms && kb_total / (parts * 2) >= 16 && parts < 16) parts *= 2;
  return parts;
}

// Y = A X on the tensor cores for the F32 (TF32 MMA) or BF16 store
tbsla_status_t dense_spmm_tc(tbsla_matrix *A, bool bf16, int k, const float *X, int64_t ldx, float *Y, int64_t ldy,
                             cudaStream_t s) {
  const int M = A->rows, K = A->cols;
  const int es = bf16 ? 2 : 4;
  const int align = 16 / es;  // elements per 16 bytes: TMA strides are multiples of 16 bytes
  if (!A->d_err) {
    TB_TRY(dev_alloc(A, (void **)&A->d_err, sizeof(int)));
    TB_CUDA(cudaMemsetAsync(A->d_err, 0, sizeof(int), s));
  }
  // A: the value store itself when its rows start on 16-byte boundaries,
  // else a copy with padded rows
  const void *a = A->values[bf16 ? 2 : 1];
  int64_t lda = K;
  void *a_pad = nullptr, *x_buf = nullptr, *parts_buf = nullptr;
  struct Release {
    cudaStream_t s;
    void **p[3];
    ~Release() {
      for (void **q : p)
        if (*q) cudaFreeAsync(*q, s);
    }
  } release{s, {&a_pad, &x_buf, &parts_buf}};
  if ((K % align) != 0 || (reinterpret_cast<uintptr_t>(a) & 15) != 0) {
    lda = (K + align - 1) / align * align;
    TB_CUDA(cudaMallocAsync(&a_pad, (size_t)M * lda * es, s));
    pad_rows_kernel<<<152 * 8, 256, 0, s>>>(static_cast<const uint8_t *>(a), M, (int64_t)K * es, (int64_t)K * es,
                                             static_cast<uint8_t *>(a_pad), lda * es);
    a = a_pad;
  }
  // X: BF16 copy for the BF16 store; for F32 the caller's X when its vectors
  // start on 16-byte boundaries
  const void *x = X;
  int64_t ldxe = ldx;
  if (bf16 || (ldx % align) != 0 || (reinterpret_cast<uintptr_t>(X) & 15) != 0) {
    ldxe = (K + align - 1) / align * align;
    TB_CUDA(cudaMallocAsync(&x_buf, (size_t)k * ldxe * es, s));
    if (bf16) {
      const int vec4 = (ldx % 4) == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
      const int gx = std::max(1, std::min((K + 1023) / 1024, 64));
      x_to_bf16_kernel<<<dim3(gx, std::min(k, 65535)), 256, 0, s>>>(X, K, k, ldx,
                                                                    static_cast<__nv_bfloat16 *>(x_buf), ldxe, vec4);
    } else {
      pad_rows_kernel<<<152 * 8, 256, 0, s>>>(reinterpret_cast<const uint8_t *>(X), k, (int64_t)K * 4, ldx * 4,
                                               static_cast<uint8_t *>(x_buf), ldxe * 4);
    }
    x = x_buf;
  }
  const int n_pad = k <= 16 ? 16 : k <= 32 ? 32 : k <= 64 ? 64 : k <= 128 ? 128 : 256;
  const int panels = (k + n_pad - 1) / n_pad;
  const int m_tiles = (M + kTileM - 1) / kTileM;
  const int kb_total = (int)(((int64_t)K * es + kRowBytes - 1) / kRowBytes);
  int sms = 0;
  TB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, A->device));
  int parts = A->tc_split > 0 ? A->tc_split : choose_parts(m_tiles, panels, kb_total, sms);
  parts = std::max(1, std::min(parts, kb_total));
  const int kb_per = (kb_total + parts - 1) / parts;
  parts = (kb_total + kb_per - 1) / kb_per;  // every part holds at least one K block
  CUtensorMap ma, mx;
  TB_TRY(encode_map(&ma, bf16, a, K, M, lda * es, kTileM));
  TB_TRY(encode_map(&mx, bf16, x, K, k, ldxe * es, n_pad));
  TcParams p{};
  p.M = M;
  p.nvec = k;
  p.kb_total = kb_total;
  p.kb_per_split = kb_per;
  p.err = A->d_err;
  p.a_early = a_pad == nullptr;  // the handle's own store: written at creation only
  if (parts == 1) {
    p.out = Y;
    p.ld_out = ldy;
    p.split_stride = 0;
  } else {
    TB_CUDA(cudaMallocAsync(&parts_buf, (size_t)parts * M * k * sizeof(float), s));
    p.out = static_cast<float *>(parts_buf);
    p.ld_out = M;
    p.split_stride = (int64_t)M * k;
  }
  if (bf16) TB_TRY(launch_tc_n<tc::kFmtBF16>(n_pad, ma, mx, p, m_tiles, parts, panels, s));
  else TB_TRY(launch_tc_n<tc::kFmtTF32>(n_pad, ma, mx, p, m_tiles, parts, panels, s));
  if (parts > 1) {
    split_sum_kernel<<<sms * 8, 256, 0, s>>>(static_cast<const float *>(parts_buf), parts, M, k, (int64_t)M * k, Y,
                                             ldy);
    TB_CUDA(cudaGetLastError());
  }
  return TBSLA_OK;
}

}  // namespace

extern "C" tbsla_status_t tbsla_dense_spmm(const tbsla_matrix_t *A_, tbsla_dtype_t store, int k, const void *d_X,
                                           int64_t ldx, void *d_Y, int64_t ldy, void *stream) {
  tbsla_matrix *A = const_cast<tbsla_matrix *>(A_);
  TB_CHECK(A && A->format == TBSLA_FMT_DENSE, "tbsla_dense_spmm needs a DENSE handle");
  TB_CHECK(k >= 0 && d_X && d_Y, "bad argument");
  const int m = A->rows, n = A->cols;
  TB_CHECK(ldx >= n && ldy >= A->n_row, "leading dimensions too small (ldx %lld < %d or ldy %lld < %d)",
           (long long)ldx, n, (long long)ldy, A->n_row);
  const void *vals = A->values[store_index(store)];
  TB_CHECK(vals, "value store %d not present", (int)store);
  TB_CUDA(cudaSetDevice(A->device));
  cudaStream_t s = (cudaStream_t)stream;
  const size_t el = store == TBSLA_F64 ? 8 : 4;
  // rows past ln_row give 0 (the one-vector product's rule)
  if (A->n_row > m && k > 0)
    TB_CUDA(cudaMemset2DAsync(static_cast<char *>(d_Y) + (size_t)m * el, (size_t)ldy * el, 0,
                              (size_t)(A->n_row - m) * el, (size_t)k, s));
  if (m == 0 || k == 0) return TBSLA_OK;
  if (n == 0) {
    TB_CUDA(cudaMemset2DAsync(d_Y, (size_t)ldy * el, 0, (size_t)m * el, (size_t)k, s));
    return TBSLA_OK;
  }
  if (store != TBSLA_F64)
    return dense_spmm_tc(A, store == TBSLA_BF16, k, static_cast<const float *>(d_X), ldx, static_cast<float *>(d_Y),
                         ldy, s);
  cublasHandle_t h = nullptr;
  TB_TRY(handle_for(A->device, &h));
  if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS) return fail(TBSLA_ERR_CUDA, "cublasSetStream failed");
  const double one = 1.0, zero = 0.0;
  const cublasStatus_t cs =
      cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, m, k, n, &one, static_cast<const double *>(vals), n,
                  static_cast<const double *>(d_X), (int)ldx, &zero, static_cast<double *>(d_Y), (int)ldy);
  if (cs != CUBLAS_STATUS_SUCCESS) return fail(TBSLA_ERR_CUDA, "cuBLAS DGEMM failed (status %d)", (int)cs);
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

extern "C" tbsla_status_t tbsla_matrix_device_status(const tbsla_matrix_t *A_, int *status) {
  tbsla_matrix *A = const_cast<tbsla_matrix *>(A_);
  TB_CHECK(A && status, "NULL argument");
  *status = 0;
  if (!A->d_err) return TBSLA_OK;
  TB_CUDA(cudaSetDevice(A->device));
  TB_CUDA(cudaDeviceSynchronize());
  TB_CUDA(cudaMemcpy(status, A->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  TB_CUDA(cudaMemset(A->d_err, 0, sizeof(int)));
  return TBSLA_OK;
}
