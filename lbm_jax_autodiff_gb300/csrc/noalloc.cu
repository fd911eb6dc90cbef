// Momentum-exchange force that allocates no device memory.
//
// lbm_momentum_exchange sums the per-block partial forces through a scratch
// buffer it takes from the CUDA stream-ordered allocator on every call.  Some
// callers of this library cannot let a library call allocate:
//  - code embedded in a host framework that owns all device memory and hands
//    out only the operand and result buffers (for example an XLA custom call
//    registered without a workspace);
//  - loops that run under a fixed device-memory budget, or that must never
//    enter the allocator (it can synchronise, fail under pressure, or fragment
//    a pool that the caller manages itself).
// lbm_momentum_exchange_noalloc computes the same force with its scratch in a
// fixed array compiled into this library (kNoAllocMaxBlocks x 3 doubles,
// 1.5 MiB).  Every GPU that loads the library holds that array until the
// process exits.
#include <cuda.h>   // CUcontext / CUresult types; the driver calls go through
                    // cudaGetDriverEntryPointByVersion, so no -lcuda is needed
#include <mutex>

#include "../../include/lbm_gb300.h"
#include "capi_util.cuh"
#include "sim.cuh"

namespace lbm {
namespace {

constexpr int kNoAllocBlock = 256;
constexpr int kNoAllocMaxCells = 1 << 24;                          // 16,777,216 cells
constexpr int kNoAllocMaxBlocks = kNoAllocMaxCells / kNoAllocBlock;  // 65,536 partials
constexpr int kMaxDevices = 64;

// One (Fx, Fy, Fz) partial per block of the current call.  Shared by every
// call on a device; a call writes slots [0, its block count) before reading
// them, so nothing needs clearing between calls.
static __device__ __align__(256) double g_force_scratch[kNoAllocMaxBlocks * 3];

// Device address of g_force_scratch per device, with the id of the CUDA
// context it was looked up in.  A module's globals live in a context: after
// cudaDeviceReset (or any teardown and re-creation of the primary context)
// the library's module is loaded again at a new address, so an address
// cached under the old context id is looked up again instead of reused.
struct ScratchSlot {
  unsigned long long ctx_id;
  double* addr;
};
std::mutex g_scratch_mu;
ScratchSlot g_scratch[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Id of the calling thread's current context (cuCtxGetId: unique over the
// life of the process), 0 when no context is current yet.
int current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static int resolved = 0;   // guarded by g_scratch_mu
  *id = 0;
  if (!resolved) {
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    LBM_TRY(cuda_check(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void**)&get_current,
                                                        12000, cudaEnableDefault, &q1),
                       "cudaGetDriverEntryPointByVersion(cuCtxGetCurrent)"));
    LBM_TRY(cuda_check(cudaGetDriverEntryPointByVersion("cuCtxGetId", (void**)&get_id, 12000,
                                                        cudaEnableDefault, &q2),
                       "cudaGetDriverEntryPointByVersion(cuCtxGetId)"));
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !get_current ||
        !get_id)
      return set_error(LBM_ERR_CUDA, "lbm_momentum_exchange_noalloc: driver lacks cuCtxGetId");
    resolved = 1;
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS)
    return set_error(LBM_ERR_CUDA, "lbm_momentum_exchange_noalloc: cuCtxGetCurrent failed");
  if (ctx && get_id(ctx, id) != CUDA_SUCCESS)
    return set_error(LBM_ERR_CUDA, "lbm_momentum_exchange_noalloc: cuCtxGetId failed");
  return LBM_OK;
}

// Device address of g_force_scratch on the current device.  Looked up with
// cudaGetSymbolAddress, with that device current, the first time a device
// calls in and again whenever the device's context has changed since; host
// code must not use the symbol itself as a device pointer.
int scratch_address(double** out) {
  int dev = 0;
  LBM_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(LBM_ERR_UNSUPPORTED, "lbm_momentum_exchange_noalloc: device ordinal >= 64");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  unsigned long long id = 0;
  LBM_TRY(current_context_id(&id));
  if (id != 0 && g_scratch[dev].addr && g_scratch[dev].ctx_id == id) {
    *out = g_scratch[dev].addr;
    return LBM_OK;
  }
  void* p = nullptr;
  // binds the device's primary context to this thread if none was current
  LBM_TRY(cuda_check(cudaGetSymbolAddress(&p, g_force_scratch), "cudaGetSymbolAddress"));
  if (id == 0) LBM_TRY(current_context_id(&id));
  g_scratch[dev].ctx_id = id;
  g_scratch[dev].addr = static_cast<double*>(p);
  *out = static_cast<double*>(p);
  return LBM_OK;
}

// Per-block partial of F = sum over links of e_i (f*_i + f_opp(i)) (forces.py:95-118).
template <class Re>
__global__ void __launch_bounds__(kNoAllocBlock)
    k_force_partials_noalloc(int n, const Re* __restrict__ fp, const Re* __restrict__ fs,
                             const Re* __restrict__ q, double* __restrict__ part) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double ax = 0.0, ay = 0.0, az = 0.0;
  if (c < n) {
    const size_t N = size_t(n);
#pragma unroll
    for (int i = 1; i < Q; ++i) {
      if (q[i * N + c] >= Re(0)) {
        const double t = double(fp[i * N + c]) + double(fs[opp(i) * N + c]);
        ax += ex(i) * t;
        ay += ey(i) * t;
        az += ez(i) * t;
      }
    }
  }
  block_sum3_store(ax, ay, az, part);
}

// Fixed-order sum of the partials into force[3].
__global__ void __launch_bounds__(kNoAllocBlock)
    k_force_total_noalloc(const double* __restrict__ part, int nblocks,
                          double* __restrict__ force) {
  __shared__ double sh[3][kNoAllocBlock];
  double a = 0.0, b = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
    a += part[3 * i];
    b += part[3 * i + 1];
    c += part[3 * i + 2];
  }
  sh[0][threadIdx.x] = a;
  sh[1][threadIdx.x] = b;
  sh[2][threadIdx.x] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
      sh[2][threadIdx.x] += sh[2][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    force[0] = sh[0][0];
    force[1] = sh[1][0];
    force[2] = sh[2][0];
  }
}

}  // namespace
}  // namespace lbm

using namespace lbm;

extern "C" int lbm_momentum_exchange_noalloc(int dtype, const void* f_post,
                                             const void* f_streamed, const void* q, double* force,
                                             int nx, int ny, int nz, void* stream) {
  if (dtype != LBM_F32 && dtype != LBM_F64)
    return set_error(LBM_ERR_UNSUPPORTED,
                     "lbm_momentum_exchange_noalloc: dtype must be LBM_F32 or LBM_F64");
  if (!f_post || !f_streamed || !q || !force)
    return set_error(LBM_ERR_ARG, "lbm_momentum_exchange_noalloc: null pointer");
  if (nx < 1 || ny < 1 || nz < 1)
    return set_error(LBM_ERR_ARG, "lbm_momentum_exchange_noalloc: dimensions must be >= 1");
  LBM_TRY(check_align(force, 8, "force"));
  const long long cells = (long long)nx * ny * nz;
  if (cells > kNoAllocMaxCells)
    return set_error(LBM_ERR_UNSUPPORTED,
                     "lbm_momentum_exchange_noalloc: grid exceeds the fixed scratch "
                     "(at most 16777216 cells); use lbm_momentum_exchange");
  double* scratch = nullptr;
  LBM_TRY(scratch_address(&scratch));
  const int n = int(cells);
  const int nb = (n + kNoAllocBlock - 1) / kNoAllocBlock;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == LBM_F64)
    k_force_partials_noalloc<double><<<nb, kNoAllocBlock, 0, st>>>(
        n, static_cast<const double*>(f_post), static_cast<const double*>(f_streamed),
        static_cast<const double*>(q), scratch);
  else
    k_force_partials_noalloc<float><<<nb, kNoAllocBlock, 0, st>>>(
        n, static_cast<const float*>(f_post), static_cast<const float*>(f_streamed),
        static_cast<const float*>(q), scratch);
  LBM_TRY(cuda_check(cudaGetLastError(), "momentum_exchange_noalloc partials"));
  k_force_total_noalloc<<<1, kNoAllocBlock, 0, st>>>(scratch, nb, force);
  return cuda_check(cudaGetLastError(), "momentum_exchange_noalloc total");
}
