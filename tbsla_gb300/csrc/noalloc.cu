// noalloc.cu -- a COO SpMV entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc: their device memory is owned by
// another allocator (a framework's caching pool or a fixed arena that has
// already reserved it), or they cannot afford the device-wide
// synchronisation that cudaMalloc and cudaFree may cause in the middle of a
// pipeline.  tbsla_coo_spmv_noalloc serves them: the caller passes the
// row-sorted triplets, x and y as device pointers, and the only scratch the
// product needs -- the per-tile carries of the merge-path COO kernel -- lives
// in the file-scope device array below, which every GPU that loads this
// library holds until the process exits.
//
// Set-up: the first call on a device, with that device current, looks the
// array's device address up with cudaGetSymbolAddress (in host code the
// array's name is only a host-side stand-in, not a device address).  That
// first call should therefore come before any stream capture on the device.
// The address is kept per device with the id of the context it belongs to;
// a call in another context (after cudaDeviceReset, say) looks it up again.
//
// Sharing: every call uses the same array.  Each call overwrites every carry
// it reads before reading it (nothing has to start at zero; y is cleared by
// the call), but two calls that overlap on the GPU -- on different streams,
// or from different host threads -- race on the array and must be ordered by
// the caller.
//
// Checked input: a first kernel verifies that the rows are nondecreasing and
// inside [0, n_row) and the columns inside [0, n_col), into a flag in the
// same array.  The product's kernels read the flag before touching x or y
// and stand down when it is set; y is then filled with NaN, and
// tbsla_coo_spmv_noalloc_status reports the failure to a caller that
// synchronises.  No call waits on the GPU.
#include <mutex>

#include "driver.cuh"
#include "product.cuh"

namespace tbsla {

// at most kNoAllocMaxTiles tiles of kMergeTile stored entries
constexpr int kNoAllocMaxTiles = 16384;
constexpr int64_t kNoAllocMaxEntries = (int64_t)kNoAllocMaxTiles * kMergeTile;  // 37,748,736

// carries: head_row (int), emitted (byte), head_val and tail_val (double)
constexpr size_t kOffHeadRow = 0;
constexpr size_t kOffEmitted = kOffHeadRow + (size_t)kNoAllocMaxTiles * sizeof(int);
constexpr size_t kOffHeadVal = (kOffEmitted + (size_t)kNoAllocMaxTiles + 255) / 256 * 256;
constexpr size_t kOffTailVal = kOffHeadVal + (size_t)kNoAllocMaxTiles * sizeof(double);
constexpr size_t kOffCheck = kOffTailVal + (size_t)kNoAllocMaxTiles * sizeof(double);
constexpr size_t kNoAllocBytes = kOffCheck + 256;  // 344,320 B

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
// per device: the context the address was looked up in, and the address
static unsigned long long g_noalloc_ctx[kMaxDevices] = {0};
static unsigned char *g_noalloc_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array in the current device's current
// context.  Looked up once per context: after cudaDeviceReset the runtime
// makes a new context, whose id differs, and the array is looked up again.
static tbsla_status_t noalloc_scratch(unsigned char **out) {
  int dev = 0;
  TB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(TBSLA_ERR_UNSUPPORTED, "device %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  unsigned long long ctx = 0;
  TB_TRY(current_context_id(&ctx));
  if (!g_noalloc_addr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
    // the lookup made the device's context current if none was
    TB_TRY(current_context_id(&ctx));
    g_noalloc_ctx[dev] = ctx;
    g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
  }
  *out = g_noalloc_addr[dev];
  return TBSLA_OK;
}

// *bad = 1 when a row decreases or leaves [0, n_row), or a column leaves
// [0, n_col) (the flag is cleared before the launch)
__global__ void noalloc_check_kernel(int64_t nnz, const int *__restrict__ row, const int *__restrict__ col,
                                     int n_row, int n_col, int *bad) {
  bool ok = true;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = row[i], c = col[i];
    ok = ok && r >= 0 && r < n_row && c >= 0 && c < n_col && (i + 1 == nnz || r <= row[i + 1]);
  }
  if (!ok) atomicOr(bad, 1);
}

// the product's epilogue, standing down when the input check failed
struct CheckedStoreEpi : StoreEpi<double, double> {
  const int *bad;
  __device__ __forceinline__ bool active() const { return *(volatile const int *)bad == 0; }
};

// y = NaN when the input check failed
__global__ void noalloc_poison_kernel(double *y, int n, const int *bad) {
  if (*(volatile const int *)bad == 0) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __longlong_as_double(0x7ff8000000000000ll);
}

}  // namespace tbsla

using namespace tbsla;

extern "C" tbsla_status_t tbsla_coo_spmv_noalloc_status(int *bad, void *stream) {
  TB_CHECK(bad, "bad is NULL");
  unsigned char *scratch = nullptr;
  TB_TRY(noalloc_scratch(&scratch));
  TB_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  TB_CUDA(cudaMemcpy(bad, scratch + kOffCheck, sizeof(int), cudaMemcpyDeviceToHost));
  return TBSLA_OK;
}

extern "C" tbsla_status_t tbsla_coo_spmv_noalloc(int n_row, int n_col, int64_t nnz, const int *d_row,
                                                 const int *d_col, const double *d_values, const double *d_x,
                                                 double *d_y, void *stream) {
  TB_CHECK(n_row >= 0 && n_col >= 0 && nnz >= 0, "negative size");
  TB_CHECK(nnz <= kNoAllocMaxEntries,
           "nnz %lld exceeds the %lld stored entries the allocation-free COO product can hold "
           "(%d tiles of %d); use tbsla_coo_create + tbsla_spmv",
           (long long)nnz, (long long)kNoAllocMaxEntries, kNoAllocMaxTiles, kMergeTile);
  TB_CHECK(nnz == 0 || (d_row && d_col && d_values && d_x), "NULL input array");
  TB_CHECK(d_y || n_row == 0, "y is NULL");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char *scratch = nullptr;
  TB_TRY(noalloc_scratch(&scratch));
  int *bad = reinterpret_cast<int *>(scratch + kOffCheck);
  TB_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
  if (n_row > 0) TB_CUDA(cudaMemsetAsync(d_y, 0, (size_t)n_row * sizeof(double), s));
  if (nnz == 0) return TBSLA_OK;
  noalloc_check_kernel<<<152 * 8, 256, 0, s>>>(nnz, d_row, d_col, n_row, n_col, bad);
  const int tiles = (int)((nnz + kMergeTile - 1) / kMergeTile);
  const Carry<double> carry{reinterpret_cast<int *>(scratch + kOffHeadRow),
                            reinterpret_cast<double *>(scratch + kOffHeadVal),
                            reinterpret_cast<double *>(scratch + kOffTailVal), scratch + kOffEmitted};
  CheckedStoreEpi epi;
  epi.y = d_y;
  epi.n_out = n_row;
  epi.shift = 0;
  epi.bad = bad;
  coo_merge_kernel<kMergeThreads, kMergeItems, double, double, CheckedStoreEpi>
      <<<tiles, kMergeThreads, 0, s>>>(d_row, d_col, d_values, d_x, 0, nnz, carry, epi);
  merge_fixup_kernel<CheckedStoreEpi><<<(tiles + 255) / 256, 256, 0, s>>>(tiles, carry, epi);
  if (n_row > 0) noalloc_poison_kernel<<<152 * 4, 256, 0, s>>>(d_y, n_row, bad);
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}
