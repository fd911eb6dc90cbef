// Fused forward step on ONE population buffer (in-place "AA" streaming).
//
// The A/B step (step.cu) reads S_{k-1} from one buffer and writes S_k to a
// second.  Here one buffer A holds the state, alternating between two layouts
// so that every cell reads and writes the same 19 locations within a launch:
//   layout L ("local"):        S_i(x) at A[opp(i)][x]
//   layout P ("pre-streamed"): S_i(x) at A[i][x + e_i]   (y, z periodic)
// A launch on layout L pulls f_i(x) = S_i(x - e_i) from A[opp(i)][x - e_i] and
// writes S_k in layout P to A[i][x + e_i]; a launch on layout P reads
// f_i(x) = A[i][x] and writes S_k in layout L to A[opp(i)][x].  Location
// (j, z) is read and written only by cell z - e_j in the first and by cell z
// in the second, so the launches are race-free for the plain pull.
//
// The reads beyond the plain pull -- the Bouzidi terms (S_io(x), S_i(x) and
// the second fluid cell's S_io(x + e_i), streaming.py:148-183), the fallback
// of out-of-range x sources (S_i(x), streaming.py:109-142) and the momentum
// exchange (S_j(x) on links, forces.py:95-118) -- would race with
// neighbours' writes, so the cells that need them keep their whole S vector
// in a side buffer: the boundary-record cells (slot = record index) and the
// x-face cells (slots after the records).  A launch reads the side buffer of
// the previous step and writes the next one (two side buffers alternate).
// The arithmetic is that of step.cu's k_step (pull_post_bc + step_body), so
// both give the same states.  FP32 / FP64 storage, periodic y/z.
#include "sim.cuh"

namespace lbm {

template <class Re> struct AAArgs {
  Re* A;               // the population buffer (storage = compute type)
  const Re* sb_in;     // side buffer of the previous step [slots][19]
  Re* sb_out;          // side buffer of this step
  int nrec;            // boundary records: slots [0, nrec); x faces after them
  // per-direction bases of the interior accesses (before the y / z wrap):
  // layout-L launch: rd[i] + idx = A[opp(i)][x - e_i], wr[i] + idx =
  // A[i][x + e_i]; layout-P launch: rd[i] = A[i], wr[i] = A[opp(i)]
  const Re* rd[Q];
  Re* wr[Q];
};

// LBM_AA_TABLES 1: interior accesses through the per-direction bases of
// AAArgs; 0: indices formed from the buffer pointer in the kernel.
#ifndef LBM_AA_TABLES
#define LBM_AA_TABLES 1
#endif

// LBM_AA_LDHINT 1: interior loads carry a 256-byte L2 prefetch hint (plain
// coherent loads: the buffer is written in the same launch).  Measured at
// 256x128x128 FP32: 140.0 us per step with the hint and the pointer tables,
// 141.3 us with the tables alone, 145.3 us with neither.
#ifndef LBM_AA_LDHINT
#define LBM_AA_LDHINT 1
#endif
__device__ __forceinline__ float aa_ld(const float* p) {
#if LBM_AA_LDHINT
  float v;
  asm volatile("ld.global.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
#else
  return *p;
#endif
}
__device__ __forceinline__ double aa_ld(const double* p) {
#if LBM_AA_LDHINT
  double v;
  asm volatile("ld.global.L2::256B.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
#else
  return *p;
#endif
}

// Side-buffer slot of a cell: its record, else its x-face slot, else -1.
__device__ __forceinline__ int sb_slot(const Grid& g, int nrec, uint32_t tag, int x, int y,
                                       int z) {
  const uint32_t ri = tag & TAG_INDEX;
  if (ri) return int(ri) - 1;
  if (x == 0) return nrec + y * g.nz + z;
  if (x == g.nx - 1) return nrec + g.ny * g.nz + y * g.nz + z;
  return -1;
}

// LAYOUT_L: the launch reads layout L (and writes layout P).
template <class Re, bool MRT, bool LAYOUT_L>
__global__ void __launch_bounds__(256, sizeof(Re) == 8 ? 2 : 4)
    k_step_aa(const StepArgs<Re> a, const AAArgs<Re> aa) {
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
    const uint32_t ri = tag & TAG_INDEX;
    const size_t N = size_t(n);
    const int slot = sb_slot(g, aa.nrec, tag, x, y, z);
    const Re* own = slot >= 0 ? aa.sb_in + size_t(slot) * Q : nullptr;
    const int nyz = g.ny * g.nz;
    // index offsets of y - 1, y + 1, z - 1, z + 1 (periodic), once per cell;
    // nbr(d) = neighbour x + d for d in {-1, 0, 1} per axis
    const int oym = y == 0 ? (g.ny - 1) * g.nz : -g.nz;
    const int oyp = y == g.ny - 1 ? -(g.ny - 1) * g.nz : g.nz;
    const int ozm = z == 0 ? g.nz - 1 : -1;
    const int ozp = z == g.nz - 1 ? 1 - g.nz : 1;
    auto nbr = [&](int dx, int dy, int dz) {
      return idx + dx * nyz + (dy < 0 ? oym : (dy > 0 ? oyp : 0)) +
             (dz < 0 ? ozm : (dz > 0 ? ozp : 0));
    };
    // wrap corrections of a y / z step d (the table bases hold the plain
    // offsets)
    auto wy = [&](int d) { return d < 0 ? (y == 0 ? nyz : 0) : (d > 0 ? (y == g.ny - 1 ? -nyz : 0) : 0); };
    auto wz = [&](int d) { return d < 0 ? (z == 0 ? g.nz : 0) : (d > 0 ? (z == g.nz - 1 ? -g.nz : 0) : 0); };
    // interior x: every pull source and push target lies in the grid
    const bool xin = x > 0 && x < g.nx - 1;
    Re f[Q];

    if (fl & SF_COLLIDE_ONLY) {
      const Re* f0 = static_cast<const Re*>(a.src);
#pragma unroll
      for (int i = 0; i < Q; ++i) f[i] = __ldg(f0 + i * N + idx);
    } else {
      // pull (streaming.py:109-142): x never periodic, out-of-range x sources
      // keep the cell's own S_i(x) (side buffer of the x faces)
      if (xin && LBM_AA_TABLES) {
#pragma unroll
        for (int i = 0; i < Q; ++i)
          f[i] = aa_ld(LAYOUT_L ? aa.rd[i] + idx + wy(-ey(i)) + wz(-ez(i)) : aa.rd[i] + idx);
      } else if (xin) {
#pragma unroll
        for (int i = 0; i < Q; ++i)
          f[i] = LAYOUT_L ? aa.A[opp(i) * N + nbr(-ex(i), -ey(i), -ez(i))] : aa.A[i * N + idx];
      } else {
#pragma unroll
        for (int i = 0; i < Q; ++i) {
          const int sx = x - ex(i);
          if (sx < 0 || sx >= g.nx) {
            f[i] = own[i];
          } else if (LAYOUT_L) {
            f[i] = aa.A[opp(i) * N + nbr(-ex(i), -ey(i), -ez(i))];
          } else {
            f[i] = aa.A[i * N + idx];
          }
        }
      }
      // Bouzidi on the cell's wall links (streaming.py:148-183)
      if (ri) {
        const LinkRec& r = a.rec[ri - 1];
        const uint32_t lm = r.linkmask;
#pragma unroll
        for (int i = 1; i < Q; ++i) {
          const int io = opp(i);
          if (lm & (1u << io)) {
            const Re qv = Re(r.q[io]);
            const Re s_opp = own[io];
            if (qv >= Re(0.5)) {
              const Re s_i = own[i];
              const Re inv2q = Re(1) / (Re(2) * fmin(qv, Re(1)));
              f[i] = inv2q * s_opp + (Re(1) - inv2q) * s_i;
            } else {
              const int nb = ahead_wrap(g, x, y, z, ex(i), ey(i), ez(i));
              const int nbx = nb / nyz, nbr_ = nb - nbx * nyz;
              const int nby = nbr_ / g.nz, nbz = nbr_ - nby * g.nz;
              const int ns = sb_slot(g, aa.nrec, __ldg(a.tag + nb), nbx, nby, nbz);
              // the second fluid cell of a q < 0.5 link is a record
              const Re s_nb = ns >= 0 ? aa.sb_in[size_t(ns) * Q + io] : s_opp;
              const Re twoq = Re(2) * fmax(qv, Re(0));
              f[i] = twoq * s_opp + (Re(1) - twoq) * s_nb;
            }
          }
        }
      }
      if (x == 0 && !(fl & SF_NO_INLET)) {
        Re ux = a.u_in[0], uy = a.u_in[1], uz = a.u_in[2];
        if (fl & SF_INLET_FACE) {
          const int fi = y * g.nz + z, fn = g.ny * g.nz;
          ux = a.u_face[fi];
          uy = a.u_face[fn + fi];
          uz = a.u_face[2 * fn + fi];
        }
        zou_he_inlet<Re>(f, ux, uy, uz);
      }
      if (x == g.nx - 1 && !(fl & SF_NO_OUTLET)) zou_he_outlet<Re>(f, a.rho_out);
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
      if ((fl & SF_FORCE) && ri) {
        const uint32_t lm = a.rec[ri - 1].linkmask;
#pragma unroll
        for (int j = 1; j < Q; ++j) {
          if (lm & (1u << j)) {
            const double tot = double(own[j]) + double(f[opp(j)]);
            fx += ex(j) * tot;
            fy += ey(j) * tot;
            fz += ez(j) * tot;
          }
        }
      }
    }

    if (fl & SF_STREAM_ONLY) {
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
      // S_i(x) after the hard bounce-back or porosity blend (state.py:146-149,
      // smooth.py:151-155)
      Re s[Q];
      if ((fl & SF_SOLID_HARD) && (tag & TAG_SOLID)) {
#pragma unroll
        for (int i = 0; i < Q; ++i) s[i] = c[opp(i)];
      } else if (fl & (SF_SOLID_SPHERE | SF_SOLID_FIELD)) {
        const Re p = a.porosity[idx];
        const Re omp = Re(1) - p;
#pragma unroll
        for (int i = 0; i < Q; ++i) s[i] = omp * c[i] + p * c[opp(i)];
      } else {
#pragma unroll
        for (int i = 0; i < Q; ++i) s[i] = c[i];
      }
      if (!LAYOUT_L || (fl & SF_COLLIDE_ONLY)) {
#pragma unroll
        for (int i = 0; i < Q; ++i) aa.wr[i][idx] = s[i];     // layout L: A[opp(i)][x]
      } else if (xin && LBM_AA_TABLES) {
        // layout P: S_i(x) at A[i][x + e_i]
#pragma unroll
        for (int i = 0; i < Q; ++i) aa.wr[i][idx + wy(ey(i)) + wz(ez(i))] = s[i];
      } else if (xin) {
#pragma unroll
        for (int i = 0; i < Q; ++i) aa.A[i * N + nbr(ex(i), ey(i), ez(i))] = s[i];
      } else {
        // values leaving through an x face are not stored (the face cells
        // keep theirs in the side buffer)
#pragma unroll
        for (int i = 0; i < Q; ++i) {
          const int tx = x + ex(i);
          if (tx >= 0 && tx < g.nx) aa.A[i * N + nbr(ex(i), ey(i), ez(i))] = s[i];
        }
      }
      if (slot >= 0) {
        Re* so = aa.sb_out + size_t(slot) * Q;
#pragma unroll
        for (int i = 0; i < Q; ++i) so[i] = s[i];
      }
    }
  }

  if (fl & SF_FORCE) block_sum3_store_at(fx, fy, fz, a.force_partials, blockIdx.x);
  if ((fl & (SF_GUARD_PRE | SF_GUARD_POST)) && a.guard_count) {
    const unsigned tot = __reduce_add_sync(0xffffffffu, resets);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd(a.guard_count, (unsigned long long)tot);
  }
}

// layout_l: the buffer holds layout L (a COLLIDE_ONLY launch ignores it and
// writes layout L).
template <class Re>
cudaError_t launch_step_aa(const StepArgs<Re>& a, Re* A, const Re* sb_in, Re* sb_out, int nrec,
                           bool layout_l, bool mrt, cudaStream_t st) {
  AAArgs<Re> aa;
  aa.A = A;
  aa.sb_in = sb_in;
  aa.sb_out = sb_out;
  aa.nrec = nrec;
  const int nb = (a.g.n + 255) / 256;
  const bool l = layout_l && !(a.flags & SF_COLLIDE_ONLY);
  const Grid& g = a.g;
  const long long N = g.n, nyz = (long long)g.ny * g.nz;
  for (int i = 0; i < Q; ++i) {
    const long long off = ex(i) * nyz + ey(i) * g.nz + ez(i);
    aa.rd[i] = l ? A + opp(i) * N - off : A + i * N;
    aa.wr[i] = l ? A + i * N + off : A + opp(i) * N;
  }
  if (mrt && l) k_step_aa<Re, true, true><<<nb, 256, 0, st>>>(a, aa);
  else if (mrt) k_step_aa<Re, true, false><<<nb, 256, 0, st>>>(a, aa);
  else if (l) k_step_aa<Re, false, true><<<nb, 256, 0, st>>>(a, aa);
  else k_step_aa<Re, false, false><<<nb, 256, 0, st>>>(a, aa);
  return cudaGetLastError();
}

template cudaError_t launch_step_aa<float>(const StepArgs<float>&, float*, const float*, float*,
                                           int, bool, bool, cudaStream_t);
template cudaError_t launch_step_aa<double>(const StepArgs<double>&, double*, const double*,
                                            double*, int, bool, bool, cudaStream_t);

}  // namespace lbm
