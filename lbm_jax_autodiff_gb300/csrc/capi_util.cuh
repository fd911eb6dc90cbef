// Error handling helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace lbm {

// Records `msg` as the calling thread's last error and returns `status`.
int set_error(int status, const char* msg);
// LBM_OK for cudaSuccess, else LBM_ERR_CUDA (or LBM_ERR_NOMEM) with the CUDA message.
int cuda_check(cudaError_t e, const char* what);
// cudaMalloc wrapper: LBM_ERR_NOMEM on failure.
int dev_alloc(void** p, size_t bytes);
// LBM_ERR_ALIGN when p is not a multiple of `align` (NULL passes).
int check_align(const void* p, size_t align, const char* name);

}  // namespace lbm

#define LBM_TRY(expr)              \
  do {                             \
    const int lbm_rc_ = (expr);    \
    if (lbm_rc_ != 0) return lbm_rc_; \
  } while (0)
