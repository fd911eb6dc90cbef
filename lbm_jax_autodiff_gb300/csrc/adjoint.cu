// Adjoint (reverse-mode) time step of the fused solver: the hand-derived
// transpose of one forward step, giving dCd/dr and dCd/dq without storing
// any per-step intermediate beyond the populations S_k.
//
// Forward (one step k):  f_k = Z(T_q(S_{k-1})),  S_k = B_p(C(f_k))
//   T_q : pull streaming + Bouzidi with wall distances q   streaming.py:40-185
//   Z   : Zou-He inlet / outlet (affine in f)              boundary.py:35-200
//   C   : BGK / MRT collision (+ Smagorinsky)               collision.py:46-270
//   B_p : hard bounce-back or sigmoid-porosity blend        smooth.py:118-155
// Objective: Cd(F(S_{N-1}, f_N)) with the momentum-exchange force F
// (forces.py:37-120, 237-276) -- the reference drivers' simulate_cd
// (examples/11:139-165) whose gradient jax.grad derives.
//
// Adjoint state stored between launches: nu_k = Z^T lambda_k, the cotangent
// of the streamed (pre-boundary) populations of step k.  One launch of
// k_adjoint for step k does, per cell y:
//   mu_k(y)  = (T_q^T nu_{k+1})(y)      gather form of the transposed stream
//   f_k(y)   = recomputed from the stashed S_{k-1}
//   dJ/dp   += mu_k . dB/dp  (sigmoid porosity, dp/dr = alpha p (1-p))
//   dJ/dq   += nu_{k+1} . dT/dq (S_k), per wall link, times dq/dr
//   lambda_k = C^T B^T mu_k;  nu_k = Z^T lambda_k on the inlet/outlet faces
#include "batch.cuh"
#include "capi_util.cuh"
#include "sim.cuh"
#include "vec2.cuh"

namespace lbm {

template <class Re> struct AdjArgs {
  StepArgs<Re> s;          // forward description; s.src = S_{k-1} (or f_0 when first)
  const void* S_k;         // stashed S_k (storage type), for q < 0.5 neighbour reads
  const Re* nu_in;         // nu_{k+1}
  Re* nu_out;              // nu_k (lambda_0 when first)
  int first;               // k == 0
  int last;                // k == N-1: add dJ/dS_{N-1} of the momentum exchange
  const double* dj_dfx;    // device scalar dJ/dFx
  double* gr_partials;     // [gridDim.x] running dJ/dr per block
  double* gq;              // [nrec][19] running dJ/dq per link
};

// Zou-He transposes (affine maps; see boundary.py:95-122 and :176-198).
template <class Re>
__device__ __forceinline__ void zou_he_inlet_T(Re l[Q], Re ux, Re uy, Re uz) {
  const Re c3 = Re(1.0 / 3.0), c6 = Re(1.0 / 6.0);
  const Re grho = c3 * ux * l[1] + c6 * (ux + uy) * l[7] + c6 * (ux - uy) * l[9] +
                  c6 * (ux + uz) * l[11] + c6 * (ux - uz) * l[13];
  const Re d = grho / (Re(1) - ux);
  Re o[Q];
#pragma unroll
  for (int j = 0; j < Q; ++j) o[j] = l[j];
  o[1] = o[7] = o[9] = o[11] = o[13] = Re(0);
  o[2] += l[1];
  o[10] += l[7];
  o[8] += l[9];
  o[14] += l[11];
  o[12] += l[13];
  o[0] += d; o[3] += d; o[4] += d; o[5] += d; o[6] += d;
  o[15] += d; o[16] += d; o[17] += d; o[18] += d;
  o[2] += Re(2) * d; o[8] += Re(2) * d; o[10] += Re(2) * d; o[12] += Re(2) * d;
  o[14] += Re(2) * d;
#pragma unroll
  for (int j = 0; j < Q; ++j) l[j] = o[j];
}

template <class Re>
__device__ __forceinline__ void zou_he_outlet_T(Re l[Q], Re rho_out) {
  const Re c3 = Re(1.0 / 3.0), c6 = Re(1.0 / 6.0);
  const Re gu = -rho_out * (c3 * l[2] + c6 * (l[10] + l[8] + l[14] + l[12]));
  const Re d = gu / rho_out;
  Re o[Q];
#pragma unroll
  for (int j = 0; j < Q; ++j) o[j] = l[j];
  o[2] = o[10] = o[8] = o[14] = o[12] = Re(0);
  o[1] += l[2];
  o[7] += l[10];
  o[9] += l[8];
  o[11] += l[14];
  o[13] += l[12];
  o[0] += d; o[3] += d; o[4] += d; o[5] += d; o[6] += d;
  o[15] += d; o[16] += d; o[17] += d; o[18] += d;
  o[1] += Re(2) * d; o[7] += Re(2) * d; o[9] += Re(2) * d; o[11] += Re(2) * d;
  o[13] += Re(2) * d;
#pragma unroll
  for (int j = 0; j < Q; ++j) l[j] = o[j];
}

// dJ/dq of the wall links owned by a cell at this step, d T(S_k)/dq with
// S_k = B(c) (c = C(f_k)); accumulates per link and returns the dJ/dr part.
template <class St>
__device__ __forceinline__ double link_q_grad(const AdjArgs<typename Storage<St>::Re>& A,
                                              const typename Storage<St>::Re c[Q],
                                              typename Storage<St>::Re p, bool soft, bool hard,
                                              uint32_t ri, int idx, int x, int y, int z) {
  using Re = typename Storage<St>::Re;
  using S = Storage<St>;
  const StepArgs<Re>& a = A.s;
  const Grid& g = a.g;
  const size_t N = size_t(g.n);
  const LinkRec& r = a.rec[ri - 1];
  const uint32_t lm = r.linkmask;
  const St* Sk = static_cast<const St*>(A.S_k);
  const NearMask M(g, a.near, x, y, z, 1);
  double* gq = A.gq + size_t(ri - 1) * Q;
  double gr = 0.0;
#pragma unroll
  for (int i = 1; i < Q; ++i) {
    const int io = opp(i);
    if ((lm >> io) & 1u) {
      const Re qv = Re(r.q[io]);
      const Re nv = __ldg(A.nu_in + i * N + idx);
      const Re s_io = soft ? (Re(1) - p) * c[io] + p * c[i] : (hard ? c[i] : c[io]);
      Re dout;
      if (qv >= Re(0.5)) {
        // a = 1 / (2 clip(q, 0.5, 1)); clip passes half the cotangent at a tie
        const Re s_i = soft ? (Re(1) - p) * c[i] + p * c[io] : (hard ? c[io] : c[i]);
        const Re wc = clip_weight<Re>(qv, Re(0.5), Re(1));
        const Re qc = fmin(qv, Re(1));
        dout = wc * (-(s_io - s_i) / (Re(2) * qc * qc));
      } else {
        // b = 2 clip(q, 0, 0.5)
        const int nb = ahead_wrap(g, x, y, z, ex(i), ey(i), ez(i));
        const Re s_nb = S::ld(Sk + io * N + nb, M.nbr_in(i) ? a.soff_near[io] : a.soff[io]);
        dout = clip_weight<Re>(qv, Re(0), Re(0.5)) * Re(2) * (s_io - s_nb);
      }
      const double gqv = double(nv) * double(dout);
      gq[io] += gqv;
      gr += gqv * r.dqdr[io];
    }
  }
  return gr;
}

// mu_k(y) = (T_q^T nu_{k+1})(y) for one cell: the gather form of the
// transposed pull (x + e_j pulled S_j(y)), the fallback terms of out-of-range
// sources, and on boundary cells the transposed Bouzidi terms and, at the
// last step, the seed dJ/dS_{N-1} of the momentum exchange.
template <class Re>
__device__ __forceinline__ void gather_mu(const AdjArgs<Re>& A, int idx, int x, int y, int z,
                                          uint32_t tag, Re mu[Q]) {
  const StepArgs<Re>& a = A.s;
  const Grid& g = a.g;
  const size_t N = size_t(g.n);
  const uint32_t ri = tag & TAG_INDEX;
  const Re* nu = A.nu_in;
  // ---- mu_k = T^T nu_{k+1}: normal-stream part (gather from x + e_j) ---
  mu[0] = __ldg(nu + idx);
  {
    const NbrOff O(g, x, y, z);
    if (!O.face) {
#pragma unroll
      for (int j = 1; j < Q; ++j) mu[j] = __ldg(nu + j * N + O.push(j, idx));
    } else {
      const PullIdx P(g, x, y, z);
#pragma unroll
      for (int j = 1; j < Q; ++j) {
        // (a) output (y + e_j, j) pulls S_j(y) when that neighbour is in range
        Re v = P.valid(opp(j)) ? __ldg(nu + j * N + P.raw(opp(j))) : Re(0);
        // (b) output (y, j) keeps S_j(y) when its own source is out of range
        if (!P.valid(j)) v += __ldg(nu + j * N + idx);
        mu[j] = v;
      }
    }
  }

  // ---- boundary-cell corrections of T^T, force seed --------------------
  if (ri) {
    const PullIdx P(g, x, y, z);
    const LinkRec& r = a.rec[ri - 1];
    const uint32_t lm = r.linkmask, nbw = r.nb_wall, nbl = r.nb_low;
#pragma unroll
    for (int j = 1; j < Q; ++j) {
      const bool wall_out = (lm >> opp(j)) & 1u;
      const bool a_ok = P.valid(opp(j)) && !((nbw >> j) & 1u);
      Re v = a_ok ? __ldg(nu + j * N + P.raw(opp(j))) : Re(0);
      if (!P.valid(j) && !wall_out) v += __ldg(nu + j * N + idx);
      if ((nbl >> j) & 1u) {
        const int w = ahead_wrap(g, x, y, z, ex(j), ey(j), ez(j));
        v += (Re(1) - Re(2) * Re(r.qnb[j])) * __ldg(nu + opp(j) * N + w);
      }
      mu[j] = v;
    }
#pragma unroll
    for (int i = 1; i < Q; ++i) {
      const int io = opp(i);
      if ((lm >> io) & 1u) {
        const Re qv = Re(r.q[io]);
        const Re nv = __ldg(nu + i * N + idx);
        if (qv >= Re(0.5)) {
          const Re a2 = Re(1) / (Re(2) * fmin(qv, Re(1)));
          mu[io] += a2 * nv;
          mu[i] += (Re(1) - a2) * nv;
        } else {
          mu[io] += Re(2) * fmax(qv, Re(0)) * nv;
        }
      }
    }
    if (A.last) {
      const Re gfx = Re(*A.dj_dfx);
#pragma unroll
      for (int j = 1; j < Q; ++j)
        if (ex(j) != 0 && ((lm >> j) & 1u)) mu[j] += Re(ex(j)) * gfx;
    }
  }
}

// resident 256-thread blocks per SM the register allocation is sized for
#ifndef LBM_ADJ_MINB
#define LBM_ADJ_MINB 3
#endif

// The adjoint step of one cell; returns its dJ/dr contribution.
template <class St, bool MRT>
__device__ __forceinline__ double adjoint_cell(const AdjArgs<typename Storage<St>::Re>& A,
                                               int idx) {
  using Re = typename Storage<St>::Re;
  using S = Storage<St>;
  const StepArgs<Re>& a = A.s;
  const Grid& g = a.g;
  const int n = g.n;
  const int fl = a.flags;
  double gr = 0.0;

  if (idx < n) {
    int x, y, z;
    decode(g, idx, x, y, z);
    const uint32_t tag = a.tag ? __ldg(a.tag + idx) : 0u;
    const uint32_t ri = tag & TAG_INDEX;
    const size_t N = size_t(n);
    const Re* nu = A.nu_in;

    Re mu[Q];
    gather_mu<Re>(A, idx, x, y, z, tag, mu);

    // ---- f_k (recompute) --------------------------------------------------
    Re f[Q];
    if (A.first) {
      const Re* f0 = static_cast<const Re*>(a.src);
#pragma unroll
      for (int i = 0; i < Q; ++i) f[i] = __ldg(f0 + i * N + idx);
    } else {
      pull_post_bc<St>(a, static_cast<const St*>(a.src), idx, x, y, z, tag, f);
    }

    const bool soft = (fl & (SF_SOLID_SPHERE | SF_SOLID_FIELD)) != 0;
    const bool hard = (fl & SF_SOLID_HARD) && (tag & TAG_SOLID);
    Re p = Re(0);
    if (soft) {
      // porosity field, or the sigmoid sphere's precomputed p and dp/dr
      p = a.porosity[idx];
      const Re dpdr = (fl & SF_SOLID_SPHERE) ? a.dpdr[idx] : Re(0);
      // dJ/dr gets mu . dB/dp dp/dr; dp/dr = alpha p (1 - p) is below
      // alpha 2^-40 (2^-70 in FP64) outside a shell a few cells thick around
      // the surface, 4e-12 of its peak alpha / 4, so the collision recompute
      // is skipped there
      const Re tiny = sizeof(Re) == 8 ? Re(8.470329472543003e-22) : Re(9.094947017729282e-13);
      if (ri || ((fl & SF_SOLID_SPHERE) && dpdr > a.sph.alpha * tiny)) {
        // dJ/dp = mu . (c[opp] - c) with c = C(f_k)
        Re c[Q];
        collide_cell<Re>(f, a.tau, MRT, (fl & SF_SMAG) != 0, a.c18cs2, a.K, c);
        if (fl & SF_SOLID_SPHERE) {
          Re gp = Re(0);
#pragma unroll
          for (int i = 0; i < Q; ++i) gp += mu[i] * (c[opp(i)] - c[i]);
          gr += double(gp) * double(dpdr);
        }
        if (ri) gr += link_q_grad<St>(A, c, p, true, false, ri, idx, x, y, z);
      }
    } else if (ri) {
      Re c[Q];
      collide_cell<Re>(f, a.tau, MRT, (fl & SF_SMAG) != 0, a.c18cs2, a.K, c);
      gr += link_q_grad<St>(A, c, p, false, hard, ri, idx, x, y, z);
    }

    // ---- B^T -------------------------------------------------------------
    if (soft) {
      Re m2[Q];
#pragma unroll
      for (int i = 0; i < Q; ++i) m2[i] = (Re(1) - p) * mu[i] + p * mu[opp(i)];
#pragma unroll
      for (int i = 0; i < Q; ++i) mu[i] = m2[i];
    } else if (hard) {
      Re m2[Q];
#pragma unroll
      for (int i = 0; i < Q; ++i) m2[i] = mu[opp(i)];
#pragma unroll
      for (int i = 0; i < Q; ++i) mu[i] = m2[i];
    }

    // ---- lambda_k = C^T mu (in place) --------------------------------------
    CellScalars<Re> cs;
    cell_scalars<Re>(f, cs);
    collide_vjp_s<Re>(cs, f, mu, a.tau, MRT, (fl & SF_SMAG) != 0, a.c18cs2, a.K, nullptr);

    // ---- nu_k = Z^T lambda_k on the faces ---------------------------------
    if (!A.first) {
      if (x == g.nx - 1 && !(fl & SF_NO_OUTLET)) zou_he_outlet_T<Re>(mu, a.rho_out);
      if (x == 0 && !(fl & SF_NO_INLET)) {
        Re ux = a.u_in[0], uy = a.u_in[1], uz = a.u_in[2];
        if (fl & SF_INLET_FACE) {
          const int fi = y * g.nz + z, fn = g.ny * g.nz;
          ux = a.u_face[fi];
          uy = a.u_face[fn + fi];
          uz = a.u_face[2 * fn + fi];
        }
        zou_he_inlet_T<Re>(mu, ux, uy, uz);
      }
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) A.nu_out[i * N + idx] = mu[i];
  }
  return gr;
}

// One block of the adjoint step: cells [block * blockDim.x, +blockDim.x);
// the block's dJ/dr goes to gr_partials[block * 8 + warp].
template <class St, bool MRT>
__device__ __forceinline__ void adjoint_body(const AdjArgs<typename Storage<St>::Re>& A,
                                             int block) {
  double gr = adjoint_cell<St, MRT>(A, block * blockDim.x + threadIdx.x);
  // deterministic per-warp accumulation of dJ/dr across steps
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) gr += __shfl_down_sync(0xffffffffu, gr, o);
  if ((threadIdx.x & 31) == 0) A.gr_partials[block * 8 + (threadIdx.x >> 5)] += gr;
}

template <class St, bool MRT>
__global__ void __launch_bounds__(256, sizeof(St) == 8 ? 1 : LBM_ADJ_MINB)
    k_adjoint(const AdjArgs<typename Storage<St>::Re> A) {
  adjoint_body<St, MRT>(A, blockIdx.x);
}

// ---------------------------------------------------------------------------
// k_adjoint_pair: the same adjoint step for two z-adjacent cells per thread
// (FP32 arithmetic, nz even): the interior gather of nu_{k+1}, the recomputed
// f_k, the bounce-back or porosity-blend transpose and the collision transpose
// run on packed float2 values (FP32x2 pipe).  Pairs with a boundary record, on
// an x face, on a non-periodic y/z edge or (16-bit storage) straddling the
// storage-offset box are listed and take the per-cell path of k_adjoint.
// ---------------------------------------------------------------------------
template <class St> struct AdjPairArgs {
  AdjArgs<float> A;
  const St* pull[Q];      // S_{k-1} + i N - (e_x nyz + e_y nz + e_z): pull source of cell 0
  const float* push[Q];   // nu_{k+1} + j N + (e_x nyz + e_y nz + e_z): cell 0 + e_j
  float* out[Q];          // nu_k + i N
  float2 soff2[2][Q];     // storage offsets outside / inside the body box (as PairArgs)
};

constexpr int kAdjPairBlock = 128;   // 256 cells per block, as k_adjoint

// Per-direction base pointers of a pair launch (as pair_pull / pair_out of
// the forward step): from the argument block's pointer tables, or with
// LBM_PAIR_PTR_ARITH 1 from the state pointers and grid sizes.
#ifndef LBM_PAIR_PTR_ARITH
#define LBM_PAIR_PTR_ARITH 0
#endif
template <class St>
__device__ __forceinline__ long long dir_off(const AdjPairArgs<St>& P, int i) {
  const Grid& g = P.A.s.g;
  return (long long)(ex(i) * g.ny * g.nz + ey(i) * g.nz + ez(i));
}
// ARITH (a template argument): formed from the state pointers and grid sizes
// regardless of LBM_PAIR_PTR_ARITH -- the batched kernel's argument block
// sits in shared memory, where a table entry costs a shared load per use.
template <bool ARITH, class St>
__device__ __forceinline__ const St* adj_pull(const AdjPairArgs<St>& P, int i) {
  if (ARITH || LBM_PAIR_PTR_ARITH)
    return static_cast<const St*>(P.A.s.src) + (long long)i * P.A.s.g.n - dir_off(P, i);
  return P.pull[i];
}
template <bool ARITH, class St>
__device__ __forceinline__ const float* adj_push(const AdjPairArgs<St>& P, int j) {
  if (ARITH || LBM_PAIR_PTR_ARITH) return P.A.nu_in + (long long)j * P.A.s.g.n + dir_off(P, j);
  return P.push[j];
}
template <bool ARITH, class St>
__device__ __forceinline__ float* adj_out(const AdjPairArgs<St>& P, int i) {
  if (ARITH || LBM_PAIR_PTR_ARITH) return P.A.nu_out + (long long)i * P.A.s.g.n;
  return P.out[i];
}

#ifndef LBM_ADJ_PAIR_MINB
#define LBM_ADJ_PAIR_MINB 4
#endif

// The part of an interior pair's adjoint step after mu and f_k: the
// transpose B^T of the hard bounce-back or (SOFT) of the porosity blend, with
// dJ/dp for a sigmoid sphere; lambda_k = C^T mu on the packed values; store
// of nu_k.  Returns the pair's dJ/dr contribution
// (nonzero only for a sigmoid sphere).
template <class St, bool MRT, bool SOFT, bool ARITH = false>
__device__ __forceinline__ double adj_pair_finish(const AdjPairArgs<St>& P, int idx, int x, int y,
                                                  int z, uint32_t t0, uint32_t t1, V2 mu[Q],
                                                  V2 f[Q]) {
  const AdjArgs<float>& A = P.A;
  const StepArgs<float>& a = A.s;
  const Grid& g = a.g;
  constexpr FixedConstsF K{};
  const int fl = a.flags;
  double gr = 0.0;
  if constexpr (SOFT) {
    // S = (1 - p) c + p c_opp per lane (smooth.py:118-155).  A sigmoid
    // sphere adds dJ/dr += mu . (c_opp - c) dp/dr, skipped where dp/dr <
    // alpha 2^-40 as in adjoint_cell
    // porosity field, or the sigmoid sphere's precomputed p and dp/dr
    const V2 p(__ldg(reinterpret_cast<const float2*>(a.porosity + idx)));
    if (fl & SF_SOLID_SPHERE) {
      const float2 dd = __ldg(reinterpret_cast<const float2*>(a.dpdr + idx));
      const float d0 = dd.x, d1 = dd.y;
      const float thr = a.sph.alpha * 9.094947017729282e-13f;
      const bool n0 = d0 > thr, n1 = d1 > thr;
      if (n0 || n1) {
        // mu . (c_opp - c) = sum_i c_i (mu_opp(i) - mu_i), summed as C emits c_i
        V2 gp(0.0f);
        auto acc = [&](int i, V2 c) { gp = gp + c * (mu[opp(i)] - mu[i]); };
        collide_cell<V2>(f, V2(a.tau), MRT, (fl & SF_SMAG) != 0, V2(a.c18cs2), K, acc);
        if (n0) gr += double(gp.x()) * double(d0);
        if (n1) gr += double(gp.y()) * double(d1);
      }
    }
    const V2 omp = V2(1.0f) - p;
    V2 m2[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) m2[i] = omp * mu[i] + p * mu[opp(i)];
#pragma unroll
    for (int i = 0; i < Q; ++i) mu[i] = m2[i];
  } else if (fl & SF_SOLID_HARD) {
    // B^T of the hard bounce-back: S_i = c_opp(i) on solid cells
    const bool s0 = (t0 & TAG_SOLID) != 0, s1 = (t1 & TAG_SOLID) != 0;
    if (s0 || s1) {
      V2 m2[Q];
#pragma unroll
      for (int i = 0; i < Q; ++i)
        m2[i] = V2(s0 ? mu[opp(i)].x() : mu[i].x(), s1 ? mu[opp(i)].y() : mu[i].y());
#pragma unroll
      for (int i = 0; i < Q; ++i) mu[i] = m2[i];
    }
  }
  // lambda_k = C^T mu
  CellScalars<V2> cs;
  cell_scalars<V2>(f, cs);
  collide_vjp_s<V2>(cs, f, mu, V2(a.tau), MRT, (fl & SF_SMAG) != 0, V2(a.c18cs2), K,
                    static_cast<V2*>(nullptr));
  // (x faces are listed pairs: no Zou-He transpose here)
#pragma unroll
  for (int i = 0; i < Q; ++i) *reinterpret_cast<float2*>(adj_out<ARITH>(P, i) + idx) = mu[i].v;
  return gr;
}


// k_adjoint_pair is one launch in two parts.  Blocks [0, nlist): the boundary pairs
// (pair_special, listed in spec_pairs), one thread per cell on the per-cell
// adjoint of k_adjoint, dJ/dr partials after the per-cell slots.  Blocks
// [nlist, ...): the interior pairs on packed values.  The list blocks come
// first so their longer per-thread latency overlaps the interior blocks.
template <class St, bool MRT>
__device__ __forceinline__ void adjoint_pair_list_part(const AdjPairArgs<St>& P, int nlist_block) {
  const AdjArgs<float>& A = P.A;
  const Grid& g = A.s.g;
  const int t = nlist_block * blockDim.x + threadIdx.x;
  double gr = 0.0;
  if (t < 2 * A.s.spec_count)
    gr = adjoint_cell<St, MRT>(A, (__ldg(A.s.spec_pairs + (t >> 1)) << 1) + (t & 1));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) gr += __shfl_down_sync(0xffffffffu, gr, o);
  // slots after the nblocks * 8 per-cell ones; one per warp (at most n / 32
  // list warps, since at most every pair is listed)
  if ((threadIdx.x & 31) == 0)
    A.gr_partials[size_t((g.n + 255) / 256) * 8 + size_t(nlist_block) * (blockDim.x >> 5) +
                  (threadIdx.x >> 5)] += gr;
}

// One interior pair of interior block `iblock`: mu_k gathered from
// nu_{k+1}, f_k pulled from S_{k-1}, then adj_pair_finish.  Returns the
// pair's dJ/dr contribution.
template <class St, bool MRT, bool SOFT, bool ARITH = false>
__device__ __forceinline__ double adjoint_pair_interior(const AdjPairArgs<St>& P, int iblock) {
  using Pr = Pair<St>;
  const AdjArgs<float>& A = P.A;
  const StepArgs<float>& a = A.s;
  const Grid& g = a.g;
  const int pidx = iblock * blockDim.x + threadIdx.x;
  if (pidx >= (g.n >> 1)) return 0.0;
  const int idx = pidx << 1;
  int x, y, z;
  decode(g, idx, x, y, z);
  const uint32_t t0 = a.tag ? __ldg(a.tag + idx) : 0u;
  const uint32_t t1 = a.tag ? __ldg(a.tag + idx + 1) : 0u;
  if (pair_special(g, a.near, sizeof(St) == 2, x, y, z, t0, t1)) return 0.0;
  const int cls = sizeof(St) == 2 ? near_class(g, a.near, x, y, z, 2) : 0;
  V2 mu[Q], f[Q];
  const int nyz = g.ny * g.nz;
  // mu_k(y) = nu_{k+1}(y + e_j): y wrap shared, z wrap per lane (x faces are
  // in the list launch)
  {
    const int iyp = idx - (y == g.ny - 1 ? nyz : 0);   // e_y = +1 reads y + 1
    const int iym = idx + (y == 0 ? nyz : 0);          // e_y = -1 reads y - 1
    const int zw1 = z + 2 == g.nz ? -g.nz : 0;         // lane 1, e_z = +1 reads z + 2
    const int zw0 = z == 0 ? g.nz : 0;                 // lane 0, e_z = -1 reads z - 1
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      const int b = ey(j) == 1 ? iyp : (ey(j) == -1 ? iym : idx);
      const float* p = adj_push<ARITH>(P, j) + b;
      if (ez(j) == 0) mu[j] = V2(ldg_s(reinterpret_cast<const float2*>(p)));
      else if (ez(j) == 1) mu[j] = V2(ldg_s(p), ldg_s(p + 1 + zw1));
      else mu[j] = V2(ldg_s(p + zw0), ldg_s(p + 1));
    }
  }
  // f_k
  if (A.first) {
    const float* f0 = static_cast<const float*>(a.src);
    const size_t N = size_t(g.n);
#pragma unroll
    for (int i = 0; i < Q; ++i)
      f[i] = V2(__ldg(reinterpret_cast<const float2*>(f0 + i * N + idx)));
  } else {
    const int iym = idx + (y == 0 ? nyz : 0);          // e_y = +1 pulls y - 1
    const int iyp = idx - (y == g.ny - 1 ? nyz : 0);   // e_y = -1 pulls y + 1
    const int zw0 = z == 0 ? g.nz : 0;                 // lane 0, e_z = +1 pulls z - 1
    const int zw1 = z + 2 == g.nz ? -g.nz : 0;         // lane 1, e_z = -1 pulls z + 2
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      const int b = ey(i) == 1 ? iym : (ey(i) == -1 ? iyp : idx);
      const St* p = adj_pull<ARITH>(P, i) + b;
      const V2 so(P.soff2[cls][i]);
      if (ez(i) == 0) f[i] = Pr::ld2(p, so);
      else if (ez(i) == 1) f[i] = Pr::ld2s(p + zw0, p + 1, so);
      else f[i] = Pr::ld2s(p, p + 1 + zw1, so);
    }
  }
  return adj_pair_finish<St, MRT, SOFT, ARITH>(P, idx, x, y, z, t0, t1, mu, f);
}


// Interior block `iblock`; a sigmoid sphere's dJ/dr partials go to the
// per-cell slots gr_partials[iblock * 8 + warp] (256 cells per block, as the
// blocks of k_adjoint).
template <class St, bool MRT, bool SOFT, bool ARITH = false>
__device__ __forceinline__ void adjoint_pair_interior_part(const AdjPairArgs<St>& P, int iblock) {
  double gr = adjoint_pair_interior<St, MRT, SOFT, ARITH>(P, iblock);
  if (SOFT && (P.A.s.flags & SF_SOLID_SPHERE)) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gr += __shfl_down_sync(0xffffffffu, gr, o);
    if ((threadIdx.x & 31) == 0)
      P.A.gr_partials[size_t(iblock) * 8 + (threadIdx.x >> 5)] += gr;
  }
}

template <class St, bool MRT, bool SOFT>
__global__ void __launch_bounds__(kAdjPairBlock, LBM_ADJ_PAIR_MINB)
    k_adjoint_pair(const AdjPairArgs<St> P, int nlist) {
  if (int(blockIdx.x) < nlist)
    adjoint_pair_list_part<St, MRT>(P, blockIdx.x);
  else
    adjoint_pair_interior_part<St, MRT, SOFT>(P, blockIdx.x - nlist);
}

// nu_N = Z^T lambda_N with lambda_N = dJ/df_N from the momentum exchange:
// lambda_N[opp j](x) = dJ/dFx * e_jx on every link (x, j).
template <class Re>
__device__ __forceinline__ void adjoint_seed_cell(const StepArgs<Re>& a,
                                                  const double* __restrict__ dj_dfx,
                                                  Re* __restrict__ nu, int idx) {
  const Grid& g = a.g;
  if (idx >= g.n) return;
  const size_t N = size_t(g.n);
  Re l[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) l[i] = Re(0);
  const uint32_t tag = a.tag ? a.tag[idx] : 0u;
  const uint32_t ri = tag & TAG_INDEX;
  if (ri) {
    const uint32_t lm = a.rec[ri - 1].linkmask;
    const Re gfx = Re(*dj_dfx);
#pragma unroll
    for (int j = 1; j < Q; ++j)
      if (ex(j) != 0 && ((lm >> j) & 1u)) l[opp(j)] += Re(ex(j)) * gfx;
    const int z = idx % g.nz, t = idx / g.nz, y = t % g.ny, x = t / g.ny;
    if (x == g.nx - 1 && !(a.flags & SF_NO_OUTLET)) zou_he_outlet_T<Re>(l, a.rho_out);
    if (x == 0 && !(a.flags & SF_NO_INLET)) {
      Re ux = a.u_in[0], uy = a.u_in[1], uz = a.u_in[2];
      if (a.flags & SF_INLET_FACE) {
        const int fi = y * g.nz + z, fn = g.ny * g.nz;
        ux = a.u_face[fi];
        uy = a.u_face[fn + fi];
        uz = a.u_face[2 * fn + fi];
      }
      zou_he_inlet_T<Re>(l, ux, uy, uz);
    }
  }
#pragma unroll
  for (int i = 0; i < Q; ++i) nu[i * N + idx] = l[i];
}

template <class Re>
__global__ void k_adjoint_seed(StepArgs<Re> a, const double* __restrict__ dj_dfx,
                               Re* __restrict__ nu) {
  adjoint_seed_cell<Re>(a, dj_dfx, nu, blockIdx.x * blockDim.x + threadIdx.x);
}

// nu_N = Z^T g for a given cotangent g on the final post-boundary f_N (the
// reference's state after N steps, state.py:129-171): the Zou-He
// transposes on the inlet / outlet faces, g itself elsewhere.
template <class Re>
__global__ void k_adjoint_seed_dense(StepArgs<Re> a, const Re* __restrict__ gin,
                                     Re* __restrict__ nu) {
  const Grid& g = a.g;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  const size_t N = size_t(g.n);
  Re l[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) l[i] = gin[i * N + idx];
  const int z = idx % g.nz, t = idx / g.nz, y = t % g.ny, x = t / g.ny;
  if (x == g.nx - 1 && !(a.flags & SF_NO_OUTLET)) zou_he_outlet_T<Re>(l, a.rho_out);
  if (x == 0 && !(a.flags & SF_NO_INLET)) {
    Re ux = a.u_in[0], uy = a.u_in[1], uz = a.u_in[2];
    if (a.flags & SF_INLET_FACE) {
      const int fi = y * g.nz + z, fn = g.ny * g.nz;
      ux = a.u_face[fi];
      uy = a.u_face[fn + fi];
      uz = a.u_face[2 * fn + fi];
    }
    zou_he_inlet_T<Re>(l, ux, uy, uz);
  }
#pragma unroll
  for (int i = 0; i < Q; ++i) nu[i * N + idx] = l[i];
}

// dJ/dFx = sign(Fx) / (0.5 rho U^2 A + 1e-10) from the finalized force record
// out = (Fx, Fy, Fz, Cd).
__global__ void k_dj_dfx(const double* __restrict__ fcd, double dyn_area, double* __restrict__ g) {
  const double fx = fcd[0];
  const double s = fx > 0.0 ? 1.0 : (fx < 0.0 ? -1.0 : 0.0);
  *g = s / (dyn_area + 1e-10);
}

// per-block partials -> scalar (fixed order)
__global__ void k_reduce_sum(const double* __restrict__ part, int n, double* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// per-link dJ/dq -> dense [19][n] (zero where there is no link)
template <class Re>
__global__ void k_scatter_gq(Grid g, const uint32_t* __restrict__ tag,
                             const LinkRec* __restrict__ rec, const double* __restrict__ gq,
                             Re* __restrict__ out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  const size_t N = size_t(g.n);
  const uint32_t ri = tag[idx] & TAG_INDEX;
  uint32_t lm = ri ? rec[ri - 1].linkmask : 0u;
#pragma unroll
  for (int j = 0; j < Q; ++j)
    out[j * N + idx] = ((lm >> j) & 1u) ? Re(gq[size_t(ri - 1) * Q + j]) : Re(0);
}

static inline int nblk(int n) { return (n + 255) / 256; }

template <class St>
cudaError_t launch_adjoint(const AdjArgs<typename Storage<St>::Re>& A, bool mrt,
                           cudaStream_t st) {
  // FP32 arithmetic (FP32 / FP16 / BF16 storage), nz even: k_adjoint_pair,
  // one launch of list blocks + interior blocks (166 us per 256x128x128 step
  // against 280 / 265 us for k_adjoint); SOFT for a porosity blend
  if constexpr (sizeof(typename Storage<St>::Re) == 4) {
    const Grid& g = A.s.g;
    if ((g.nz % 2) == 0 && A.s.spec_pairs) {
      AdjPairArgs<St> P;
      P.A = A;
      const long long N = g.n, nyz = (long long)g.ny * g.nz;
      for (int i = 0; i < Q; ++i) {
        const long long off = ex(i) * nyz + ey(i) * g.nz + ez(i);
        P.pull[i] = static_cast<const St*>(A.s.src) + i * N - off;
        P.push[i] = A.nu_in + i * N + off;
        P.out[i] = A.nu_out + i * N;
        P.soff2[0][i] = make_float2(A.s.soff[i], A.s.soff[i]);
        P.soff2[1][i] = make_float2(A.s.soff_near[i], A.s.soff_near[i]);
      }
      const int nb = (g.n / 2 + kAdjPairBlock - 1) / kAdjPairBlock;
      const int nlist = (2 * A.s.spec_count + kAdjPairBlock - 1) / kAdjPairBlock;
      const bool soft = (A.s.flags & (SF_SOLID_SPHERE | SF_SOLID_FIELD)) != 0;
      if (mrt && soft)
        k_adjoint_pair<St, true, true><<<nlist + nb, kAdjPairBlock, 0, st>>>(P, nlist);
      else if (mrt)
        k_adjoint_pair<St, true, false><<<nlist + nb, kAdjPairBlock, 0, st>>>(P, nlist);
      else if (soft)
        k_adjoint_pair<St, false, true><<<nlist + nb, kAdjPairBlock, 0, st>>>(P, nlist);
      else
        k_adjoint_pair<St, false, false><<<nlist + nb, kAdjPairBlock, 0, st>>>(P, nlist);
      return cudaGetLastError();
    }
  }
  if (mrt)
    k_adjoint<St, true><<<nblk(A.s.g.n), 256, 0, st>>>(A);
  else
    k_adjoint<St, false><<<nblk(A.s.g.n), 256, 0, st>>>(A);
  return cudaGetLastError();
}

template <class Re>
cudaError_t launch_adjoint_seed(const StepArgs<Re>& a, const double* dj, Re* nu, cudaStream_t st) {
  k_adjoint_seed<Re><<<nblk(a.g.n), 256, 0, st>>>(a, dj, nu);
  return cudaGetLastError();
}

template <class Re>
cudaError_t launch_adjoint_seed_dense(const StepArgs<Re>& a, const Re* g, Re* nu,
                                      cudaStream_t st) {
  k_adjoint_seed_dense<Re><<<nblk(a.g.n), 256, 0, st>>>(a, g, nu);
  return cudaGetLastError();
}

cudaError_t launch_dj_dfx(const double* fcd, double dyn_area, double* g, cudaStream_t st) {
  k_dj_dfx<<<1, 1, 0, st>>>(fcd, dyn_area, g);
  return cudaGetLastError();
}

cudaError_t launch_reduce_sum(const double* part, int n, double* out, cudaStream_t st) {
  k_reduce_sum<<<1, 256, 0, st>>>(part, n, out);
  return cudaGetLastError();
}

template <class Re>
cudaError_t launch_scatter_gq(const Grid& g, const uint32_t* tag, const LinkRec* rec,
                              const double* gq, Re* out, cudaStream_t st) {
  k_scatter_gq<Re><<<nblk(g.n), 256, 0, st>>>(g, tag, rec, gq, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Batched forms: one launch covers every instance of a batch.
// ---------------------------------------------------------------------------
#ifndef LBM_ADJ_BATCH_MINB
#define LBM_ADJ_BATCH_MINB 2
#endif

template <class St, bool MRT>
__global__ void __launch_bounds__(256, LBM_ADJ_BATCH_MINB)
    k_adjoint_batch(const AdjArgs<float>* __restrict__ args, const BatchInst* __restrict__ inst,
                    const int2* __restrict__ map, int sprev_slot, int sk_slot, int nu_in_slot,
                    int nu_out_slot, int first, int last) {
  __shared__ AdjArgs<float> A;
  const int2 m = map[blockIdx.x];
  copy_to_shared(&A, args + m.x);
  __syncthreads();
  const BatchInst& b = inst[m.x];
  if (threadIdx.x == 0) {
    A.s.src = batch_slot(b, sprev_slot);
    A.S_k = batch_slot(b, sk_slot);
    A.nu_in = static_cast<const float*>(batch_slot(b, nu_in_slot));
    A.nu_out = static_cast<float*>(batch_slot(b, nu_out_slot));
    A.first = first;
    A.last = last;
    A.dj_dfx = b.out + 4;
    A.gr_partials = b.gr_part;
    A.gq = b.gq;
  }
  __syncthreads();
  const int end = m.y + kBatchChunk < b.nblk ? m.y + kBatchChunk : b.nblk;
  for (int sb = m.y; sb < end; ++sb) adjoint_body<St, MRT>(A, sb);
}

// Batched k_adjoint_pair (FP32 storage, nz even): map[b] = (instance, first
// sub-block), the sub-blocks of an instance being its list blocks then its
// interior blocks, kPairBatchChunk per block; entries with instance -1 pad the
// map to the grid the launch (and a captured graph) was sized for.  SOFT:
// the instances with a porosity blend.
#ifndef LBM_ADJ_PAIR_BATCH_MINB
#define LBM_ADJ_PAIR_BATCH_MINB 4
#endif
// LBM_BATCH_PTR_ARITH 1: the batched pair adjoint forms its per-direction
// pointers from the instance's state pointers (adj_pull<true>), 0: it
// builds the tables in shared memory.
#ifndef LBM_BATCH_PTR_ARITH
#define LBM_BATCH_PTR_ARITH 1
#endif

template <bool MRT, bool SOFT>
__global__ void __launch_bounds__(kAdjPairBlock, LBM_ADJ_PAIR_BATCH_MINB)
    k_adjoint_pair_batch(const AdjArgs<float>* __restrict__ args,
                         const BatchInst* __restrict__ inst, const int2* __restrict__ map,
                         int sprev_slot, int sk_slot, int nu_in_slot, int nu_out_slot, int first,
                         int last) {
  __shared__ AdjPairArgs<float> P;
  const int2 m = map[blockIdx.x];
  if (m.x < 0) return;
  copy_to_shared(&P.A, args + m.x);
  __syncthreads();
  const BatchInst& b = inst[m.x];
  const float* src = static_cast<const float*>(batch_slot(b, sprev_slot));
  const float* nu_in = static_cast<const float*>(batch_slot(b, nu_in_slot));
  float* nu_out = static_cast<float*>(batch_slot(b, nu_out_slot));
  if (threadIdx.x == 0) {
    AdjArgs<float>& A = P.A;
    A.s.src = src;
    A.S_k = batch_slot(b, sk_slot);
    A.nu_in = nu_in;
    A.nu_out = nu_out;
    A.first = first;
    A.last = last;
    A.dj_dfx = b.out + 4;
    A.gr_partials = b.gr_part;
    A.gq = b.gq;
  } else if (!LBM_BATCH_PTR_ARITH && threadIdx.x <= Q) {
    // the per-direction tables, one direction per thread
    const int i = threadIdx.x - 1;
    const Grid& g = P.A.s.g;
    const long long N = g.n, nyz = (long long)g.ny * g.nz;
    const long long off = ex(i) * nyz + ey(i) * g.nz + ez(i);
    P.pull[i] = src + i * N - off;
    P.push[i] = nu_in + i * N + off;
    P.out[i] = nu_out + i * N;
    P.soff2[0][i] = make_float2(0.0f, 0.0f);
    P.soff2[1][i] = make_float2(0.0f, 0.0f);
  }
  __syncthreads();
  const int nlist = (2 * P.A.s.spec_count + kAdjPairBlock - 1) / kAdjPairBlock;
  const int nint = (P.A.s.g.n / 2 + kAdjPairBlock - 1) / kAdjPairBlock;
  const int end = m.y + kPairBatchChunk < nlist + nint ? m.y + kPairBatchChunk : nlist + nint;
  for (int sb = m.y; sb < end; ++sb) {
    if (sb < nlist)
      adjoint_pair_list_part<float, MRT>(P, sb);
    else
      adjoint_pair_interior_part<float, MRT, SOFT, LBM_BATCH_PTR_ARITH != 0>(P, sb - nlist);
  }
}

__global__ void __launch_bounds__(256)
    k_adjoint_seed_batch(const StepArgs<float>* __restrict__ args,
                         const BatchInst* __restrict__ inst, const int2* __restrict__ map,
                         int nu_slot) {
  __shared__ StepArgs<float> sa;
  const int2 m = map[blockIdx.x];
  copy_to_shared(&sa, args + m.x);
  __syncthreads();
  const BatchInst& b = inst[m.x];
  float* nu = static_cast<float*>(batch_slot(b, nu_slot));
  const int end = m.y + kBatchChunk < b.nblk ? m.y + kBatchChunk : b.nblk;
  for (int sb = m.y; sb < end; ++sb)
    adjoint_seed_cell<float>(sa, b.out + 4, nu, sb * blockDim.x + threadIdx.x);
}

// Per instance (one block each): clear the dJ/dr partials and the per-link dJ/dq.
__global__ void __launch_bounds__(256) k_zero_grad_batch(const BatchInst* __restrict__ inst) {
  const BatchInst& b = inst[blockIdx.x];
  for (int i = threadIdx.x; i < b.ngr; i += blockDim.x) b.gr_part[i] = 0.0;
  for (int i = threadIdx.x; i < b.ngq; i += blockDim.x) b.gq[i] = 0.0;
}

// Per instance (one block each): dCd/dr = fixed-order sum of the partials.
__global__ void __launch_bounds__(256) k_reduce_gr_batch(const BatchInst* __restrict__ inst) {
  __shared__ double sh[256];
  const BatchInst& b = inst[blockIdx.x];
  double v = 0.0;
  for (int i = threadIdx.x; i < b.ngr; i += blockDim.x) v += b.gr_part[i];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) b.out[5] = sh[0];
}

// One Adam step on each instance's radius (optax.adam, examples/11:182-194):
// loss = Cd (minimize_cd_loss) or (Cd - target)^2 (target_cd_loss,
// optim/losses.py:34-99); m, v bias-corrected; r clipped to [r_min, r_max]
// afterwards.  opt[i] = (r, m, v, t).
__global__ void k_adam_batch(const BatchInst* __restrict__ inst, int count, AdamP p,
                             double* __restrict__ opt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const BatchInst& b = inst[i];
  const double cd = b.out[3], dcd = b.out[5];
  const double loss = p.target ? (cd - p.target_cd) * (cd - p.target_cd) : cd;
  const double g = p.target ? 2.0 * (cd - p.target_cd) * dcd : dcd;
  b.out[6] = loss;
  b.out[7] = g;
  double* o = opt + 4 * i;
  const double t = o[3] + 1.0;
  const double m = p.b1 * o[1] + (1.0 - p.b1) * g;
  const double v = p.b2 * o[2] + (1.0 - p.b2) * g * g;
  const double mh = m / (1.0 - pow(p.b1, t));
  const double vh = v / (1.0 - pow(p.b2, t));
  double r = o[0] - p.lr * mh / (sqrt(vh) + p.eps);
  r = fmin(fmax(r, p.r_min), p.r_max);
  o[0] = r;
  o[1] = m;
  o[2] = v;
  o[3] = t;
}

template <class St>
cudaError_t launch_adjoint_batch(const AdjArgs<float>* args, const BatchInst* inst,
                                 const int2* map, int nblocks, int block, bool mrt,
                                 int sprev_slot, int sk_slot, int nu_in_slot, int nu_out_slot,
                                 int first, int last, cudaStream_t st) {
  if (mrt)
    k_adjoint_batch<St, true><<<nblocks, block, 0, st>>>(args, inst, map, sprev_slot, sk_slot,
                                                        nu_in_slot, nu_out_slot, first, last);
  else
    k_adjoint_batch<St, false><<<nblocks, block, 0, st>>>(args, inst, map, sprev_slot, sk_slot,
                                                         nu_in_slot, nu_out_slot, first, last);
  return cudaGetLastError();
}

cudaError_t launch_adjoint_pair_batch(const AdjArgs<float>* args, const BatchInst* inst,
                                      const int2* map, int nblocks, bool mrt, bool soft,
                                      int sprev_slot, int sk_slot, int nu_in_slot,
                                      int nu_out_slot, int first, int last, cudaStream_t st) {
  if (mrt && soft)
    k_adjoint_pair_batch<true, true><<<nblocks, kAdjPairBlock, 0, st>>>(
        args, inst, map, sprev_slot, sk_slot, nu_in_slot, nu_out_slot, first, last);
  else if (mrt)
    k_adjoint_pair_batch<true, false><<<nblocks, kAdjPairBlock, 0, st>>>(
        args, inst, map, sprev_slot, sk_slot, nu_in_slot, nu_out_slot, first, last);
  else if (soft)
    k_adjoint_pair_batch<false, true><<<nblocks, kAdjPairBlock, 0, st>>>(
        args, inst, map, sprev_slot, sk_slot, nu_in_slot, nu_out_slot, first, last);
  else
    k_adjoint_pair_batch<false, false><<<nblocks, kAdjPairBlock, 0, st>>>(
        args, inst, map, sprev_slot, sk_slot, nu_in_slot, nu_out_slot, first, last);
  return cudaGetLastError();
}

cudaError_t launch_adjoint_seed_batch(const StepArgs<float>* args, const BatchInst* inst,
                                      const int2* map, int nblocks, int block, int nu_slot,
                                      cudaStream_t st) {
  k_adjoint_seed_batch<<<nblocks, block, 0, st>>>(args, inst, map, nu_slot);
  return cudaGetLastError();
}

cudaError_t launch_zero_grad_batch(const BatchInst* inst, int count, cudaStream_t st) {
  k_zero_grad_batch<<<count, 256, 0, st>>>(inst);
  return cudaGetLastError();
}

cudaError_t launch_reduce_gr_batch(const BatchInst* inst, int count, cudaStream_t st) {
  k_reduce_gr_batch<<<count, 256, 0, st>>>(inst);
  return cudaGetLastError();
}

cudaError_t launch_adam_batch(const BatchInst* inst, int count, const AdamP& p, double* opt,
                              cudaStream_t st) {
  k_adam_batch<<<(count + 127) / 128, 128, 0, st>>>(inst, count, p, opt);
  return cudaGetLastError();
}

template cudaError_t launch_adjoint_batch<float>(const AdjArgs<float>*, const BatchInst*,
                                                 const int2*, int, int, bool, int, int, int, int,
                                                 int, int, cudaStream_t);

template cudaError_t launch_adjoint<float>(const AdjArgs<float>&, bool, cudaStream_t);
template cudaError_t launch_adjoint<double>(const AdjArgs<double>&, bool, cudaStream_t);
template cudaError_t launch_adjoint<__half>(const AdjArgs<float>&, bool, cudaStream_t);
template cudaError_t launch_adjoint<__nv_bfloat16>(const AdjArgs<float>&, bool, cudaStream_t);
template cudaError_t launch_adjoint_seed<float>(const StepArgs<float>&, const double*, float*,
                                                cudaStream_t);
template cudaError_t launch_adjoint_seed<double>(const StepArgs<double>&, const double*, double*,
                                                 cudaStream_t);
template cudaError_t launch_adjoint_seed_dense<float>(const StepArgs<float>&, const float*,
                                                      float*, cudaStream_t);
template cudaError_t launch_adjoint_seed_dense<double>(const StepArgs<double>&, const double*,
                                                       double*, cudaStream_t);
template cudaError_t launch_scatter_gq<float>(const Grid&, const uint32_t*, const LinkRec*,
                                              const double*, float*, cudaStream_t);
template cudaError_t launch_scatter_gq<double>(const Grid&, const uint32_t*, const LinkRec*,
                                               const double*, double*, cudaStream_t);

}  // namespace lbm
