// Thread-local error reporting and small helpers of the C ABI.
#include <cstdio>
#include <cstring>

#include "../../include/lbm_gb300.h"
#include "capi_util.cuh"

namespace lbm {

static thread_local char g_last_error[512] = "";

int set_error(int status, const char* msg) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s", msg ? msg : "");
  return status;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return LBM_OK;
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s)", what, cudaGetErrorString(e),
                cudaGetErrorName(e));
  cudaGetLastError();  // clear a sticky launch error so later calls are not poisoned
  return e == cudaErrorMemoryAllocation ? LBM_ERR_NOMEM : LBM_ERR_CUDA;
}

int dev_alloc(void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 1;
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_check(e, "cudaMalloc");
  }
  return LBM_OK;
}

int check_align(const void* p, size_t align, const char* name) {
  if (p && (reinterpret_cast<uintptr_t>(p) % align) != 0) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "pointer '%s' is not %zu-byte aligned", name, align);
    return set_error(LBM_ERR_ALIGN, buf);
  }
  return LBM_OK;
}

}  // namespace lbm

extern "C" {

const char* lbm_last_error(void) { return lbm::g_last_error; }

size_t lbm_struct_size(int which) {
  switch (which) {
    case 0: return sizeof(lbm_params);
    case 1: return sizeof(lbm_sphere);
    case 2: return sizeof(lbm_xla_desc);
    case 3: return sizeof(lbm_xla_fused_desc);
    case 4: return sizeof(lbm_adam);
    default: return 0;
  }
}

const char* lbm_status_string(int s) {
  switch (s) {
    case LBM_OK: return "LBM_OK";
    case LBM_ERR_ARG: return "LBM_ERR_ARG";
    case LBM_ERR_ALIGN: return "LBM_ERR_ALIGN";
    case LBM_ERR_UNSUPPORTED: return "LBM_ERR_UNSUPPORTED";
    case LBM_ERR_TIMEOUT: return "LBM_ERR_TIMEOUT";
    case LBM_ERR_CUDA: return "LBM_ERR_CUDA";
    case LBM_ERR_NOMEM: return "LBM_ERR_NOMEM";
    case LBM_ERR_STATE: return "LBM_ERR_STATE";
    default: return "LBM_ERR_UNKNOWN";
  }
}

}  // extern "C"
