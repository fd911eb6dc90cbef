// Device-side tables of the batched solver: many independent instances
// (grids of different sizes, own geometry and boundary modes) advanced by one
// kernel launch per step.  Block b of a batched launch works on sub-blocks
// map[b].y .. map[b].y + kBatchChunk - 1 of instance map[b].x; each instance's kernel arguments live in
// device memory, so a launch captured in a CUDA graph stays valid when the
// host rebuilds an instance's geometry between replays.
#pragma once

#include "sim.cuh"

namespace lbm {

// Population buffers of one instance, addressed by slot number in the
// batched launches: SLOT_F0 (reference-layout f_0), SLOT_S0 / SLOT_S1 (the
// ping-pong states), SLOT_NU0 / SLOT_NU1 (adjoint states), and j >= 0 for
// workspace state j (checkpoints, then the recompute stash).
enum : int { SLOT_F0 = -1, SLOT_S0 = -2, SLOT_S1 = -3, SLOT_NU0 = -4, SLOT_NU1 = -5 };

// Sub-blocks (one block's worth of cells each) that one block of a batched
// launch walks after staging its instance's arguments once: map[b].y is the
// first of them.
#ifndef LBM_BATCH_CHUNK
#define LBM_BATCH_CHUNK 4
#endif
constexpr int kBatchChunk = LBM_BATCH_CHUNK;

// The same for the batched pair adjoint (sub-blocks of 128 pairs): one, so
// the grid has the most blocks (measured 0.88 s per 400-step evaluation of
// the 64-instance batch against 0.93 s with four).
#ifndef LBM_PAIR_BATCH_CHUNK
#define LBM_PAIR_BATCH_CHUNK 1
#endif
constexpr int kPairBatchChunk = LBM_PAIR_BATCH_CHUNK;

struct BatchInst {
  void* f0;
  void* S[2];
  void* nu[2];
  char* states;
  unsigned long long state_bytes;
  double* force_part;      // [nblk][3]
  double* gr_part;         // [ngr] dJ/dr partials: per-block slots, then per-warp list slots
  int ngr;
  double* gq;              // [ngq] per-link dJ/dq
  int ngq;
  int nblk;                // blocks of this instance at the batch block size
  double* out;             // [8]: Fx, Fy, Fz, Cd, dJ/dFx, dCd/dr, loss, dloss/dr
  const double* dyn_area;  // 0.5 rho U^2 A
};

__device__ __forceinline__ void* batch_slot(const BatchInst& b, int slot) {
  switch (slot) {
    case SLOT_F0: return b.f0;
    case SLOT_S0: return b.S[0];
    case SLOT_S1: return b.S[1];
    case SLOT_NU0: return b.nu[0];
    case SLOT_NU1: return b.nu[1];
    default: return b.states + size_t(slot) * b.state_bytes;
  }
}

// Adam on the radius (optax.adam defaults b1 0.9, b2 0.999, eps 1e-8) and
// the loss: Cd, or (Cd - target_cd)^2 when target != 0.
struct AdamP {
  double lr, b1, b2, eps, r_min, r_max, target_cd;
  int target;
};

// Copy an argument block into shared memory with the whole thread block.
template <class T>
__device__ __forceinline__ void copy_to_shared(T* dst, const T* src) {
  static_assert(sizeof(T) % 4 == 0, "argument blocks are 4-byte multiples");
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  for (int i = threadIdx.x; i < int(sizeof(T) / 4); i += blockDim.x) d[i] = s[i];
}

}  // namespace lbm
