// Fused forward time step (one HBM read + one HBM write of the 19
// populations per cell).
//
// The stored state between launches is the post-collision, post-solid
// population S_k ("f_post" of the reference drivers, examples/11:152-160).
// One launch of k_step for step k does, per cell, in registers:
//   pull S_{k-1} from the upstream neighbours            streaming.py:109-142
//   Bouzidi bounce-back on the cell's wall links         streaming.py:148-183
//   Zou-He inlet (x=0) and outlet (x=nx-1)               boundary.py:35-200
//   post-BC guard (state.py:161-169)     -> f_k (the reference's state after k steps)
//   momentum-exchange force of (S_{k-1}, f_k), if sampled  forces.py:95-118
//   pre-collision guard (examples/10:163-168)
//   Smagorinsky tau, BGK/MRT collide                     collision.py:46-270
//   hard bounce-back or sigmoid-porosity blend          state.py:146-149, smooth.py:151-155
//   store S_k
// SF_COLLIDE_ONLY (step 0) reads f_0 instead of pulling; SF_STREAM_ONLY stops
// after f_k and writes it in the reference layout.
//
// k_step_pair does the same for two z-adjacent cells per thread (FP32
// arithmetic, nz even): the 19 populations of both cells live in packed
// float2 registers and the collision runs on the FP32x2 pipe, the z-aligned
// directions move as one 4-byte access of two 16-bit values, and the per-cell
// index and conversion work is shared by the pair; the pairs with a boundary
// record, on an x face, on a non-periodic edge or straddling the storage-
// offset box are listed and run lane by lane in the first blocks of the same
// launch.  It serves 16-bit storage; k_step serves FP32 / FP64, odd nz, the
// COLLIDE_ONLY / STREAM_ONLY launches and the sampled steps that also sum the
// momentum-exchange force (SF_FORCE).
#include <type_traits>

#include "batch.cuh"
#include "sim.cuh"
#include "vec2.cuh"

namespace lbm {

// One block of the fused step: cells [block * blockDim.x, +blockDim.x) of the
// grid `a` describes; the force partial of the block goes to slot `block`.
// Per-direction pointers of a k_step launch: pull[i] + idx is the interior
// pull source x - e_i of cell idx (before y / z wrap), out[i] + idx its slot
// in S_k.
template <class St> struct CellTabs {
  const St* pull[Q];
  St* out[Q];
};

template <class St, bool MRT>
__device__ __forceinline__ void step_body(const StepArgs<typename Storage<St>::Re>& a, int block,
                                          const CellTabs<St>* T = nullptr) {
  using Re = typename Storage<St>::Re;
  using S = Storage<St>;
  const Grid& g = a.g;
  const int n = g.n;
  const int idx = block * blockDim.x + threadIdx.x;
  const int fl = a.flags;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  unsigned resets = 0;

  if (idx < n) {
    int x, y, z;
    decode(g, idx, x, y, z);
    const uint32_t tag = a.tag ? __ldg(a.tag + idx) : 0u;
    const size_t N = size_t(n);
    Re f[Q];

    if (fl & SF_COLLIDE_ONLY) {
      const Re* f0 = static_cast<const Re*>(a.src);
#pragma unroll
      for (int i = 0; i < Q; ++i) f[i] = __ldg(f0 + i * N + idx);
    } else {
      pull_post_bc<St>(a, static_cast<const St*>(a.src), idx, x, y, z, tag, f,
                       T ? T->pull : nullptr);
    }

    Re rho = density<Re>(f);
    Re jx, jy, jz;
    momentum<Re>(f, jx, jy, jz);

    if (!(fl & SF_COLLIDE_ONLY)) {
      if ((fl & SF_GUARD_POST) && unstable_rj<Re>(rho, jx, jy, jz)) {
#pragma unroll
        for (int i = 0; i < Q; ++i) f[i] = a.guard_reset[i];
        rho = density<Re>(f);
        momentum<Re>(f, jx, jy, jz);
        ++resets;
      }
      if ((fl & SF_FORCE) && (tag & TAG_INDEX)) {
        const St* src = static_cast<const St*>(a.src);
        const LinkRec& r = a.rec[(tag & TAG_INDEX) - 1];
        const uint32_t lm = r.linkmask;
#pragma unroll
        for (int j = 1; j < Q; ++j) {
          if (lm & (1u << j)) {
            const double tot =
                double(S::ld(src + j * N + idx, soff_at(a, x, y, z, j))) + double(f[opp(j)]);
            fx += ex(j) * tot;
            fy += ey(j) * tot;
            fz += ez(j) * tot;
          }
        }
      }
    }

    if ((fl & SF_EMIT_F) && !(fl & SF_COLLIDE_ONLY)) {
      // the reference f of this step, as a stream-only pass would write it
      Re* fe = static_cast<Re*>(a.f_emit);
#pragma unroll
      for (int i = 0; i < Q; ++i) fe[i * N + idx] = f[i];
    }

    if (fl & SF_STREAM_ONLY) {
      // (a null dst: only the force of this pass is wanted)
      Re* fo = static_cast<Re*>(a.dst);
      if (fo) {
#pragma unroll
        for (int i = 0; i < Q; ++i) fo[i * N + idx] = f[i];
      }
    } else {
      if ((fl & SF_GUARD_PRE) && unstable_rj<Re>(rho, jx, jy, jz)) {
#pragma unroll
        for (int i = 0; i < Q; ++i) f[i] = a.guard_reset[i];
        rho = density<Re>(f);
        momentum<Re>(f, jx, jy, jz);
        ++resets;
      }
      Re c[Q];
      if constexpr (sizeof(Re) == 4)
        collide_cell_rj<Re>(f, rho, jx, jy, jz, a.tau, MRT, (fl & SF_SMAG) != 0, a.c18cs2,
                            FixedConstsF{}, c);
      else
        collide_cell_rj<Re>(f, rho, jx, jy, jz, a.tau, MRT, (fl & SF_SMAG) != 0, a.c18cs2, a.K, c);

      St* dst = static_cast<St*>(a.dst);
      auto out = [&](int i) { return T ? T->out[i] + idx : dst + i * N + idx; };
      const bool nr = in_near(a.near, x, y, z);
      if ((fl & SF_SOLID_HARD) && (tag & TAG_SOLID)) {
#pragma unroll
        for (int i = 0; i < Q; ++i) S::st(out(i), c[opp(i)], nr ? a.soff_near[i] : a.soff[i]);
      } else if (fl & (SF_SOLID_SPHERE | SF_SOLID_FIELD)) {
        const Re p = a.porosity[idx];   // field, or the sigmoid sphere's precomputed one
        const Re omp = Re(1) - p;
#pragma unroll
        for (int i = 0; i < Q; ++i)
          S::st(out(i), omp * c[i] + p * c[opp(i)], nr ? a.soff_near[i] : a.soff[i]);
      } else {
#pragma unroll
        for (int i = 0; i < Q; ++i) S::st(out(i), c[i], nr ? a.soff_near[i] : a.soff[i]);
      }
    }
  }

  if (fl & SF_FORCE) block_sum3_store_at(fx, fy, fz, a.force_partials, block);
  if ((fl & (SF_GUARD_PRE | SF_GUARD_POST)) && a.guard_count) {
    const unsigned tot = __reduce_add_sync(0xffffffffu, resets);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd(a.guard_count, (unsigned long long)tot);
  }
}

// LBM_STEP_TABLES 1: k_step takes per-direction pointer tables (CellTabs)
// for its interior pulls and its stores.
#ifndef LBM_STEP_TABLES
#define LBM_STEP_TABLES 1
#endif

#ifndef LBM_STEP_MINB
#define LBM_STEP_MINB 4
#endif

template <class St, bool MRT>
__global__ void __launch_bounds__(256, sizeof(St) == 8 ? 2 : LBM_STEP_MINB)
    k_step(const StepArgs<typename Storage<St>::Re> a, const CellTabs<St> T) {
  step_body<St, MRT>(a, blockIdx.x, LBM_STEP_TABLES ? &T : nullptr);
}

// Per-direction pointers of one pair launch: pull[i] + idx is the interior
// pull source x - e_i of cell idx in direction i; out[i] + idx its slot in S_k.
template <class St> struct PairArgs {
  StepArgs<float> a;
  const St* pull[Q];
  St* out[Q];
  // storage offsets (both lanes): [0] outside the body box, [1] inside; the
  // box's z bounds are even, so the two cells of a pair share the class
  float2 soff2[2][Q];
};

constexpr int kPairBlock = 128;   // 256 cells per block

// Per-direction base pointers of a pair launch.  LBM_PAIR_PTR_ARITH 0 (the
// default): read from the argument block's per-direction pointer tables; 1:
// formed from the two population pointers and the grid sizes.  Measured at
// 256x128x128: 92.9 us (tables) against 96.2 us per FP16 step, 0.554 s
// against 0.563 s per FP16 gradient evaluation.
#ifndef LBM_PAIR_PTR_ARITH
#define LBM_PAIR_PTR_ARITH 0
#endif
template <class St>
__device__ __forceinline__ const St* pair_pull(const PairArgs<St>& P, int i) {
#if LBM_PAIR_PTR_ARITH
  const Grid& g = P.a.g;
  return static_cast<const St*>(P.a.src) + (long long)i * g.n -
         (ex(i) * g.ny * g.nz + ey(i) * g.nz + ez(i));
#else
  return P.pull[i];
#endif
}
template <class St>
__device__ __forceinline__ St* pair_out(const PairArgs<St>& P, int i) {
#if LBM_PAIR_PTR_ARITH
  return static_cast<St*>(P.a.dst) + (long long)i * P.a.g.n;
#else
  return P.out[i];
#endif
}

// Pre/post guard of state.py:161-169 on both lanes; returns the number of
// lanes reset (to `reset`, with rho and j recomputed).
__device__ __forceinline__ unsigned guard_pair(V2 f[Q], V2& rho, V2& jx, V2& jy, V2& jz,
                                               const float reset[Q]) {
  const V2 j2 = jx * jx + jy * jy + jz * jz;
  const V2 lim = V2(0.16f) * rho * rho;
  const bool b0 = !(rho.x() >= 0.3f && rho.x() <= 2.0f) || j2.x() > lim.x();
  const bool b1 = !(rho.y() >= 0.3f && rho.y() <= 2.0f) || j2.y() > lim.y();
  if (b0 || b1) {
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = V2(b0 ? reset[i] : f[i].x(), b1 ? reset[i] : f[i].y());
    rho = density<V2>(f);
    momentum<V2>(f, jx, jy, jz);
  }
  return unsigned(b0) + unsigned(b1);
}

// Everything after the pull for a pair of cells (idx even, z even): guards,
// Smagorinsky + BGK/MRT collision on the FP32x2 pipe, hard bounce-back or
// porosity blend, store of S_k through out[i] + idx.
// CLS: the pair's storage offset class when the caller knows it at compile
// time (0 outside the body box), -1 to test the pair here.
template <class St, bool MRT, int CLS = -1>
__device__ __forceinline__ unsigned finish_pair(const PairArgs<St>& P, int idx, int x, int y,
                                                int z, uint32_t t0, uint32_t t1, V2 f[Q]) {
  using Pr = Pair<St>;
  const StepArgs<float>& a = P.a;
  constexpr FixedConstsF K{};
  const int fl = a.flags;
  unsigned resets = 0;
  V2 rho = density<V2>(f);
  V2 jx, jy, jz;
  momentum<V2>(f, jx, jy, jz);
  if (fl & SF_GUARD_POST) resets += guard_pair(f, rho, jx, jy, jz, a.guard_reset);
  if (fl & SF_GUARD_PRE) resets += guard_pair(f, rho, jx, jy, jz, a.guard_reset);

  // storage offset class of the pair
  const int nc = CLS >= 0 ? CLS : (in_near(a.near, x, y, z) ? 1 : 0);
  auto off = [&](int i) { return V2(P.soff2[nc][i]); };
  const bool s0 = (t0 & TAG_SOLID) != 0, s1 = (t1 & TAG_SOLID) != 0;
  const bool blend = (fl & (SF_SOLID_SPHERE | SF_SOLID_FIELD)) != 0;
  if (!blend && !((fl & SF_SOLID_HARD) && (s0 || s1))) {
    // plain fluid pair: each post-collision population is stored as it is
    // produced, no output array stays live
    auto store = [&](int i, V2 v) { Pr::st2(pair_out(P, i) + idx, v, off(i)); };
    collide_cell_rj<V2>(f, rho, jx, jy, jz, V2(a.tau), MRT, (fl & SF_SMAG) != 0, V2(a.c18cs2), K,
                        store);
    return resets;
  }
  V2 c[Q];
  collide_cell_rj<V2>(f, rho, jx, jy, jz, V2(a.tau), MRT, (fl & SF_SMAG) != 0, V2(a.c18cs2), K, c);
  if ((fl & SF_SOLID_HARD) && (s0 || s1)) {
#pragma unroll
    for (int i = 0; i < Q; ++i)
      Pr::st2(pair_out(P, i) + idx,
              V2(s0 ? c[opp(i)].x() : c[i].x(), s1 ? c[opp(i)].y() : c[i].y()),
              off(i));
  } else if (fl & (SF_SOLID_SPHERE | SF_SOLID_FIELD)) {
    // porosity field, or the sigmoid sphere's precomputed one
    const V2 p(__ldg(reinterpret_cast<const float2*>(a.porosity + idx)));
    const V2 omp = V2(1.0f) - p;
#pragma unroll
    for (int i = 0; i < Q; ++i)
      Pr::st2(pair_out(P, i) + idx, omp * c[i] + p * c[opp(i)], off(i));
  }
  return resets;
}

// Global-memory pull of the lanes marked in `lanes` (bit 0: cell idx, bit 1:
// idx + 1), with the Bouzidi, Zou-He and fallback rules of pull_post_bc.
template <class St>
__device__ __forceinline__ void pull_lanes(const StepArgs<float>& a, int idx, int x, int y, int z,
                                           uint32_t t0, uint32_t t1, unsigned lanes, V2 f[Q]) {
  const St* src = static_cast<const St*>(a.src);
#pragma unroll 1
  for (int l = 0; l < 2; ++l) {
    if (!(lanes & (1u << l))) continue;
    float fl1[Q];
    pull_post_bc<St>(a, src, idx + l, x, y, z + l, l ? t1 : t0, fl1);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      if (l) f[i].v.y = fl1[i];
      else f[i].v.x = fl1[i];
    }
  }
}

__device__ __forceinline__ void add_resets(const StepArgs<float>& a, unsigned resets) {
  if ((a.flags & (SF_GUARD_PRE | SF_GUARD_POST)) && a.guard_count) {
    const unsigned tot = __reduce_add_sync(__activemask(), resets);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd(a.guard_count, (unsigned long long)tot);
  }
}

// The boundary pairs (pair_special, listed in spec_pairs): the per-cell
// pull with Bouzidi, Zou-He, fallback and per-direction storage offsets,
// then the same packed collision and store.
template <class St, bool MRT>
__device__ __forceinline__ void step_pair_list_part(const PairArgs<St>& P, int nlist_block) {
  const StepArgs<float>& a = P.a;
  const Grid& g = a.g;
  const int t = nlist_block * blockDim.x + threadIdx.x;
  unsigned resets = 0;
  if (t < a.spec_count) {
    const int idx = __ldg(a.spec_pairs + t) << 1;
    int x, y, z;
    decode(g, idx, x, y, z);
    const uint32_t t0 = a.tag ? __ldg(a.tag + idx) : 0u;
    const uint32_t t1 = a.tag ? __ldg(a.tag + idx + 1) : 0u;
    V2 f[Q];
    pull_lanes<St>(a, idx, x, y, z, t0, t1, 3u, f);
    resets = finish_pair<St, MRT>(P, idx, x, y, z, t0, t1, f);
  }
  add_resets(a, resets);
}

// Pull (packed, y wrap shared by both lanes, z wrap per lane) and finish of
// one interior pair; CLS as for finish_pair, `cls` the tested class when
// CLS < 0.  The x faces are listed pairs, so every source lies in the grid.
template <class St, bool MRT, int CLS>
__device__ __forceinline__ unsigned step_pair_interior(const PairArgs<St>& P, int idx, int x,
                                                       int y, int z, uint32_t t0, uint32_t t1,
                                                       int cls) {
  using Pr = Pair<St>;
  const StepArgs<float>& a = P.a;
  const Grid& g = a.g;
  if (CLS >= 0) cls = CLS;
  V2 f[Q];
  const int nyz = g.ny * g.nz;
  const int iym = idx + (y == 0 ? nyz : 0);          // e_y = +1 pulls y - 1
  const int iyp = idx - (y == g.ny - 1 ? nyz : 0);   // e_y = -1 pulls y + 1
  const int zw0 = z == 0 ? g.nz : 0;                 // lane 0, e_z = +1 pulls z - 1
  const int zw1 = z + 2 == g.nz ? -g.nz : 0;         // lane 1, e_z = -1 pulls z + 2
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const V2 so(P.soff2[cls][i]);
    const int b = ey(i) == 1 ? iym : (ey(i) == -1 ? iyp : idx);
    const St* p = pair_pull(P, i) + b;
    if (ez(i) == 0) f[i] = Pr::ld2(p, so);
    else if (ez(i) == 1) f[i] = Pr::ld2s(p + zw0, p + 1, so);
    else f[i] = Pr::ld2s(p, p + 1 + zw1, so);
  }
  return finish_pair<St, MRT, CLS>(P, idx, x, y, z, t0, t1, f);
}

// Five 128-thread blocks per SM (96 registers): the extra resident warps hide
// more load latency than the few spilled registers of the list path cost
// (measured 104 us per 16-bit step at 256x128x128 against 110 us at four).
#ifndef LBM_STEP_PAIR_MINB
#define LBM_STEP_PAIR_MINB 5
#endif

// One launch in two parts: blocks [0, nlist) run the boundary pairs, the
// rest the interior pairs (the list blocks first, so their longer latency
// overlaps the interior blocks).
template <class St, bool MRT>
__global__ void __launch_bounds__(kPairBlock, LBM_STEP_PAIR_MINB) k_step_pair(const PairArgs<St> P, int nlist) {
  if (int(blockIdx.x) < nlist) {
    step_pair_list_part<St, MRT>(P, blockIdx.x);
    return;
  }
  const StepArgs<float>& a = P.a;
  const Grid& g = a.g;
  const int pidx = (blockIdx.x - nlist) * blockDim.x + threadIdx.x;
  unsigned resets = 0;

  int idx = 0, x = 0, y = 0, z = 0;
  uint32_t t0 = 0u, t1 = 0u;
  bool active = pidx < (g.n >> 1);
  if (active) {
    idx = pidx << 1;
    decode(g, idx, x, y, z);
    t0 = a.tag ? __ldg(a.tag + idx) : 0u;
    t1 = a.tag ? __ldg(a.tag + idx + 1) : 0u;
    // listed pairs run in the list blocks
    active = !pair_special(g, a.near, sizeof(St) == 2, x, y, z, t0, t1);
  }
  // storage offset class per pair (0 outside the body box, 1 inside; listed
  // pairs straddle it).  FP16: a warp whose pairs are all outside runs a
  // copy with the outside offsets fixed at compile time (measured 98 us
  // against 104 us per step at 256x128x128; neutral to slower for bf16,
  // whose loads take the mixed-precision add instead).
  const int cls = active && sizeof(St) == 2 ? near_class(g, a.near, x, y, z, 2) : 0;
  constexpr bool kWarpClass = std::is_same<St, __half>::value;
  const bool far = kWarpClass ? __all_sync(0xffffffffu, cls == 0) : false;
  if (active) {
    if (far)
      resets = step_pair_interior<St, MRT, 0>(P, idx, x, y, z, t0, t1, 0);
    else
      resets = step_pair_interior<St, MRT, -1>(P, idx, x, y, z, t0, t1, cls);
  }
  add_resets(a, resets);
}

// Per pair: 1 if pair_special (the pair kernels' own skip test), else 0.
__global__ void k_pair_flags(Grid g, const uint32_t* __restrict__ tag, Near nb, int use_class,
                             uint8_t* __restrict__ flags) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (g.n >> 1)) return;
  const int idx = p << 1;
  int x, y, z;
  decode(g, idx, x, y, z);
  const uint32_t t0 = tag ? tag[idx] : 0u, t1 = tag ? tag[idx + 1] : 0u;
  flags[p] = pair_special(g, nb.b, use_class != 0, x, y, z, t0, t1) ? 1 : 0;
}

cudaError_t launch_pair_flags(const Grid& g, const uint32_t* tag, const int near[6], int use_class,
                              uint8_t* flags, cudaStream_t st) {
  Near nb;
  for (int k = 0; k < 6; ++k) nb.b[k] = near[k];
  const int np = g.n >> 1;
  k_pair_flags<<<(np + 255) / 256, 256, 0, st>>>(g, tag, nb, use_class, flags);
  return cudaGetLastError();
}

// Deterministic reduction of the per-block force partials (fixed order) and
// the drag coefficient Cd = |Fx| / (0.5 rho U^2 A + 1e-10) (forces.py:274-276).
// Writes out[0..2] = F, out[3] = Cd.
__global__ void k_force_finalize(const double* __restrict__ part, int nblocks, double dyn_area,
                                 double* __restrict__ out, int with_cd) {
  __shared__ double sh[3][256];
  double a = 0, b = 0, c = 0;
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
    out[0] = sh[0][0];
    out[1] = sh[1][0];
    out[2] = sh[2][0];
    if (with_cd) out[3] = fabs(sh[0][0]) / (dyn_area + 1e-10);
  }
}

// FP32 storage runs k_step, the fastest form for it when measured at
// 256x128x128 (113-114 us vs 115-117 us for k_step_pair); 16-bit storage runs
// k_step_pair (91-92 us vs ~117 us for k_step), the pair layout halving its
// conversion and address work per cell.
template <class St>
cudaError_t launch_step(const StepArgs<typename Storage<St>::Re>& a, bool mrt,
                        cudaStream_t stream) {
  if constexpr (sizeof(St) == 2) {
    if ((a.g.nz % 2) == 0 && a.spec_pairs &&
        !(a.flags & (SF_COLLIDE_ONLY | SF_STREAM_ONLY | SF_FORCE | SF_EMIT_F))) {
      PairArgs<St> P;
      P.a = a;
      const Grid& g = a.g;
      const long long N = g.n, nyz = (long long)g.ny * g.nz;
      for (int i = 0; i < Q; ++i) {
        P.pull[i] = static_cast<const St*>(a.src) + i * N - (ex(i) * nyz + ey(i) * g.nz + ez(i));
        P.out[i] = static_cast<St*>(a.dst) + i * N;
        P.soff2[0][i] = make_float2(a.soff[i], a.soff[i]);
        P.soff2[1][i] = make_float2(a.soff_near[i], a.soff_near[i]);
      }
      const int nb = (g.n / 2 + kPairBlock - 1) / kPairBlock;
      const int nlist = (a.spec_count + kPairBlock - 1) / kPairBlock;
      if (mrt)
        k_step_pair<St, true><<<nlist + nb, kPairBlock, 0, stream>>>(P, nlist);
      else
        k_step_pair<St, false><<<nlist + nb, kPairBlock, 0, stream>>>(P, nlist);
      return cudaGetLastError();
    }
  }
  const int bs = 256;
  const int nb = (a.g.n + bs - 1) / bs;
  CellTabs<St> T;
  {
    const Grid& g = a.g;
    const long long N = g.n, nyz = (long long)g.ny * g.nz;
    for (int i = 0; i < Q; ++i) {
      // pull bases are formed only when there is a source state (a
      // collide-only launch reads f_0 through a.src itself)
      T.pull[i] = a.src && !(a.flags & SF_COLLIDE_ONLY)
                      ? static_cast<const St*>(a.src) + i * N - (ex(i) * nyz + ey(i) * g.nz + ez(i))
                      : nullptr;
      T.out[i] = a.dst ? static_cast<St*>(a.dst) + i * N : nullptr;
    }
  }
  if (mrt)
    k_step<St, true><<<nb, bs, 0, stream>>>(a, T);
  else
    k_step<St, false><<<nb, bs, 0, stream>>>(a, T);
  return cudaGetLastError();
}

cudaError_t launch_force_finalize(const double* part, int nblocks, double dyn_area, double* out,
                                  cudaStream_t stream) {
  k_force_finalize<<<1, 256, 0, stream>>>(part, nblocks, dyn_area, out, 1);
  return cudaGetLastError();
}

// force only (3 doubles), for the per-op momentum_exchange
cudaError_t launch_force_sum(const double* part, int nblocks, double* out3, cudaStream_t stream) {
  k_force_finalize<<<1, 256, 0, stream>>>(part, nblocks, 0.0, out3, 0);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Batched forms: one launch covers every instance of a batch.
// ---------------------------------------------------------------------------
template <class St, bool MRT>
__global__ void __launch_bounds__(256, 4)
    k_step_batch(const StepArgs<float>* __restrict__ args, const BatchInst* __restrict__ inst,
                 const int2* __restrict__ map, int src_slot, int dst_slot, int extra_flags) {
  __shared__ StepArgs<float> sa;
  const int2 m = map[blockIdx.x];
  copy_to_shared(&sa, args + m.x);
  __syncthreads();
  const BatchInst& b = inst[m.x];
  if (threadIdx.x == 0) {
    sa.src = batch_slot(b, src_slot);
    sa.dst = batch_slot(b, dst_slot);
    sa.flags |= extra_flags;
    sa.force_partials = b.force_part;
  }
  __syncthreads();
  const int end = m.y + kBatchChunk < b.nblk ? m.y + kBatchChunk : b.nblk;
  for (int sb = m.y; sb < end; ++sb) step_body<St, MRT>(sa, sb);
}

// Per instance (one block each): F from the block partials, Cd, and with
// with_dj the objective's dJ/dFx = sign(Fx) / (0.5 rho U^2 A + 1e-10)
// (forces.py:274-276).  With `samples`, (F, Cd) also go to samples[i*4..].
__global__ void __launch_bounds__(256)
    k_force_finalize_batch(const BatchInst* __restrict__ inst, int with_dj,
                           double* __restrict__ samples) {
  __shared__ double sh[3][256];
  const BatchInst& b = inst[blockIdx.x];
  double x = 0, y = 0, z = 0;
  for (int i = threadIdx.x; i < b.nblk; i += blockDim.x) {
    x += b.force_part[3 * i];
    y += b.force_part[3 * i + 1];
    z += b.force_part[3 * i + 2];
  }
  sh[0][threadIdx.x] = x;
  sh[1][threadIdx.x] = y;
  sh[2][threadIdx.x] = z;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + o];
      sh[2][threadIdx.x] += sh[2][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double fx = sh[0][0], den = *b.dyn_area + 1e-10;
    b.out[0] = fx;
    b.out[1] = sh[1][0];
    b.out[2] = sh[2][0];
    b.out[3] = fabs(fx) / den;
    if (with_dj) b.out[4] = (fx > 0.0 ? 1.0 : (fx < 0.0 ? -1.0 : 0.0)) / den;
    if (samples) {
      samples[4 * blockIdx.x + 0] = fx;
      samples[4 * blockIdx.x + 1] = sh[1][0];
      samples[4 * blockIdx.x + 2] = sh[2][0];
      samples[4 * blockIdx.x + 3] = fabs(fx) / den;
    }
  }
}

template <class St>
cudaError_t launch_step_batch(const StepArgs<float>* args, const BatchInst* inst, const int2* map,
                              int nblocks, int block, bool mrt, int src_slot, int dst_slot,
                              int extra_flags, cudaStream_t stream) {
  if (mrt)
    k_step_batch<St, true><<<nblocks, block, 0, stream>>>(args, inst, map, src_slot, dst_slot,
                                                         extra_flags);
  else
    k_step_batch<St, false><<<nblocks, block, 0, stream>>>(args, inst, map, src_slot, dst_slot,
                                                          extra_flags);
  return cudaGetLastError();
}

cudaError_t launch_force_finalize_batch(const BatchInst* inst, int count, int with_dj,
                                        double* samples, cudaStream_t stream) {
  k_force_finalize_batch<<<count, 256, 0, stream>>>(inst, with_dj, samples);
  return cudaGetLastError();
}

template cudaError_t launch_step_batch<float>(const StepArgs<float>*, const BatchInst*,
                                              const int2*, int, int, bool, int, int, int,
                                              cudaStream_t);

template cudaError_t launch_step<float>(const StepArgs<float>&, bool, cudaStream_t);
template cudaError_t launch_step<double>(const StepArgs<double>&, bool, cudaStream_t);
template cudaError_t launch_step<__half>(const StepArgs<float>&, bool, cudaStream_t);
template cudaError_t launch_step<__nv_bfloat16>(const StepArgs<float>&, bool, cudaStream_t);

}  // namespace lbm
