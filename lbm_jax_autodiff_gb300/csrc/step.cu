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
#include "sim.cuh"

namespace lbm {

template <class St, bool MRT>
__global__ void __launch_bounds__(256, sizeof(St) == 8 ? 2 : 4) k_step(const StepArgs<typename Storage<St>::Re> a) {
  using Re = typename Storage<St>::Re;
  using S = Storage<St>;
  const Grid& g = a.g;
  const int n = g.n;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
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
      pull_post_bc<St>(a, static_cast<const St*>(a.src), idx, x, y, z, tag, f);
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
            const double tot = double(S::ld(src + j * N + idx, a.K.w[j])) + double(f[opp(j)]);
            fx += ex(j) * tot;
            fy += ey(j) * tot;
            fz += ez(j) * tot;
          }
        }
      }
    }

    if (fl & SF_STREAM_ONLY) {
      Re* fo = static_cast<Re*>(a.dst);
#pragma unroll
      for (int i = 0; i < Q; ++i) fo[i * N + idx] = f[i];
    } else {
      if ((fl & SF_GUARD_PRE) && unstable_rj<Re>(rho, jx, jy, jz)) {
#pragma unroll
        for (int i = 0; i < Q; ++i) f[i] = a.guard_reset[i];
        rho = density<Re>(f);
        momentum<Re>(f, jx, jy, jz);
        ++resets;
      }
      Re c[Q];
      collide_cell_rj<Re>(f, rho, jx, jy, jz, a.tau, MRT, (fl & SF_SMAG) != 0, a.c18cs2, a.K, c);

      St* dst = static_cast<St*>(a.dst);
      if ((fl & SF_SOLID_HARD) && (tag & TAG_SOLID)) {
#pragma unroll
        for (int i = 0; i < Q; ++i) S::st(dst + i * N + idx, c[opp(i)], a.K.w[i]);
      } else if (fl & (SF_SOLID_SPHERE | SF_SOLID_FIELD)) {
        const Re p = (fl & SF_SOLID_SPHERE) ? sphere_porosity<Re>(a.sph, x, y, z, nullptr)
                                            : a.porosity[idx];
        const Re omp = Re(1) - p;
#pragma unroll
        for (int i = 0; i < Q; ++i) S::st(dst + i * N + idx, omp * c[i] + p * c[opp(i)], a.K.w[i]);
      } else {
#pragma unroll
        for (int i = 0; i < Q; ++i) S::st(dst + i * N + idx, c[i], a.K.w[i]);
      }
    }
  }

  if (fl & SF_FORCE) block_sum3_store(fx, fy, fz, a.force_partials);
  if ((fl & (SF_GUARD_PRE | SF_GUARD_POST)) && a.guard_count) {
    const unsigned tot = __reduce_add_sync(0xffffffffu, resets);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd(a.guard_count, (unsigned long long)tot);
  }
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

template <class St>
cudaError_t launch_step(const StepArgs<typename Storage<St>::Re>& a, bool mrt,
                        cudaStream_t stream) {
  const int bs = 256;
  const int nb = (a.g.n + bs - 1) / bs;
  if (mrt)
    k_step<St, true><<<nb, bs, 0, stream>>>(a);
  else
    k_step<St, false><<<nb, bs, 0, stream>>>(a);
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

template cudaError_t launch_step<float>(const StepArgs<float>&, bool, cudaStream_t);
template cudaError_t launch_step<double>(const StepArgs<double>&, bool, cudaStream_t);
template cudaError_t launch_step<__half>(const StepArgs<float>&, bool, cudaStream_t);
template cudaError_t launch_step<__nv_bfloat16>(const StepArgs<float>&, bool, cudaStream_t);

}  // namespace lbm
