// driver.cu -- driver entry points resolved through the runtime (driver.cuh).
#include <mutex>

#include "driver.cuh"

namespace tbsla {

namespace {
std::once_flag g_once;
DriverApi g_api;
tbsla_status_t g_status = TBSLA_OK;

template <typename F> bool resolve(const char *name, F *fn) {
  void *p = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !p)
    return false;
  *fn = reinterpret_cast<F>(p);
  return true;
}
}  // namespace

tbsla_status_t driver_api(const DriverApi **out) {
  std::call_once(g_once, [] {
    const bool ok = resolve("cuCtxGetCurrent", &g_api.ctx_get_current) &&
                    resolve("cuCtxGetId", &g_api.ctx_get_id) &&
                    resolve("cuTensorMapEncodeTiled", &g_api.tensor_map_encode_tiled);
    g_status = ok ? TBSLA_OK : fail(TBSLA_ERR_CUDA, "the CUDA driver lacks an entry point the library needs");
  });
  if (g_status != TBSLA_OK) return fail(TBSLA_ERR_CUDA, "the CUDA driver lacks an entry point the library needs");
  *out = &g_api;
  return TBSLA_OK;
}

tbsla_status_t current_context_id(unsigned long long *id) {
  const DriverApi *d = nullptr;
  TB_TRY(driver_api(&d));
  CUcontext ctx = nullptr;
  *id = 0;
  if (d->ctx_get_current(&ctx) != CUDA_SUCCESS) return fail(TBSLA_ERR_CUDA, "cuCtxGetCurrent failed");
  if (!ctx) return TBSLA_OK;
  if (d->ctx_get_id(ctx, id) != CUDA_SUCCESS) return fail(TBSLA_ERR_CUDA, "cuCtxGetId failed");
  return TBSLA_OK;
}

}  // namespace tbsla
