// driver.cuh -- CUDA driver functions the library needs beside the runtime
// (the current context's identity, TMA tensor maps), resolved once through
// cudaGetDriverEntryPointByVersion so that the library does not link
// libcuda directly.
#pragma once

#include <cuda.h>

#include "common.cuh"

namespace tbsla {

struct DriverApi {
  CUresult (*ctx_get_current)(CUcontext *) = nullptr;
  CUresult (*ctx_get_id)(CUcontext, unsigned long long *) = nullptr;
  CUresult (*tensor_map_encode_tiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                      const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                      CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                      CUtensorMapFloatOOBfill) = nullptr;
};

// the resolved functions (TBSLA_ERR_CUDA if the driver lacks one)
tbsla_status_t driver_api(const DriverApi **out);

// unique id of the calling thread's current context (0 when there is none)
tbsla_status_t current_context_id(unsigned long long *id);

}  // namespace tbsla
