// Per-op drop-in kernels: one launch per jax_lbm.core function, same
// semantics and layout, plus the matching vector-Jacobian products.
//
//   compute_density / compute_velocity / equilibrium   core/equilibrium.py:22-151
//   bgk / mrt / smagorinsky_tau                         core/collision.py:46-270
//   soft_bounce_back                                    geometry/smooth.py:118-155
//   stream (dense q)                                    core/streaming.py:40-185
//   zou_he_inlet / zou_he_outlet                        core/boundary.py:35-200
//   momentum_exchange / drag_coefficient / projected_area  core/forces.py:37-276
//
// These are the bisection / drop-in path: each call reads and writes whole
// arrays.  The fused solver (step.cu, adjoint.cu) is the fast path.
#include "../../include/lbm_gb300.h"
#include "capi_util.cuh"
#include "sim.cuh"

namespace lbm {

cudaError_t launch_force_sum(const double* part, int nblocks, double* out3, cudaStream_t st);

namespace {

struct OpDims {
  int nx, ny, nz, n;
};

__device__ __forceinline__ void decode3(const OpDims& d, int idx, int& x, int& y, int& z) {
  z = idx % d.nz;
  const int t = idx / d.nz;
  y = t % d.ny;
  x = t / d.ny;
}

inline int nblk(long long n) { return int((n + 255) / 256); }

template <class Re>
Consts<Re> op_consts(int flags) {
  Consts<Re> K;
  const double w[Q] = {1.0 / 3.0,  1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                       1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                       1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                       1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
  const double r[Q] = {0.0, 1.19, 1.4, 0.0, 1.2, 0.0, 1.2, 0.0, 1.2, 0.0,
                       1.4, 0.0,  1.4, 0.0, 0.0, 0.0, 1.98, 1.98, 1.98};
  const bool exact = (flags & LBM_OP_EXACT_CONSTANTS) != 0;
  for (int i = 0; i < Q; ++i) {
    K.w[i] = exact ? Re(w[i]) : Re(double(float(w[i])));
    K.rate[i] = exact ? Re(r[i]) : Re(double(float(r[i])));
  }
  return K;
}

// ---------------------------------------------------------------- forward ---

template <class Re>
__global__ void k_density(int n, const Re* __restrict__ f, Re* __restrict__ rho) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  Re v[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) v[i] = f[size_t(i) * n + c];
  rho[c] = density<Re>(v);
}

template <class Re>
__global__ void k_velocity(int n, const Re* __restrict__ f, const Re* __restrict__ rho,
                           Re* __restrict__ u) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  Re v[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) v[i] = f[size_t(i) * n + c];
  Re jx, jy, jz;
  momentum<Re>(v, jx, jy, jz);
  const Re r = rho[c];
  u[c] = jx / r;
  u[size_t(n) + c] = jy / r;
  u[2 * size_t(n) + c] = jz / r;
}

template <class Re>
__global__ void k_equilibrium(int n, const Re* __restrict__ rho, const Re* __restrict__ u,
                              Consts<Re> K, Re* __restrict__ feq) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  Re o[Q];
  equilibrium<Re>(rho[c], u[c], u[size_t(n) + c], u[2 * size_t(n) + c], K.w, o);
#pragma unroll
  for (int i = 0; i < Q; ++i) feq[size_t(i) * n + c] = o[i];
}

template <class Re>
__global__ void k_collide(int n, const Re* __restrict__ f, const Re* __restrict__ tau_f, Re tau,
                          int mrt, Consts<Re> K, Re* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  Re v[Q], o[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) v[i] = f[size_t(i) * n + c];
  const Re t = tau_f ? tau_f[c] : tau;
  collide_cell<Re>(v, t, mrt != 0, false, Re(0), K, o);
#pragma unroll
  for (int i = 0; i < Q; ++i) out[size_t(i) * n + c] = o[i];
}

template <class Re>
__global__ void k_smag_tau(int n, const Re* __restrict__ f, Re tau, Re c18, Consts<Re> K,
                           Re* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  Re v[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) v[i] = f[size_t(i) * n + c];
  CellScalars<Re> cs;
  cell_scalars<Re>(v, cs);
  Re s[6];
  neq_stress<Re>(cs.p, K.w, cs.rho, cs.ux, cs.uy, cs.uz, s);
  const Re ir = Re(1) / cs.rho;
  out[c] = smag_tau<Re>(tau, c18, smag_pi<Re>(s), inv_rho_eps<Re>(cs.rho, ir));
}

template <class Re>
__global__ void k_soft_bounce(int n, const Re* __restrict__ f, const Re* __restrict__ p,
                              Re* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const Re pc = p[c];
  Re v[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) v[i] = f[size_t(i) * n + c];
#pragma unroll
  for (int i = 0; i < Q; ++i) out[size_t(i) * n + c] = (Re(1) - pc) * v[i] + pc * v[opp(i)];
}

// jnp.roll-wrapped neighbour x + d (all axes)
__device__ __forceinline__ int wrap3(const OpDims& d, int x, int y, int z, int dx, int dy,
                                     int dz) {
  return (wrapi(x + dx, d.nx) * d.ny + wrapi(y + dy, d.ny)) * d.nz + wrapi(z + dz, d.nz);
}

// pull source (streaming.py:109-142): -1 when the cell keeps its own value
__device__ __forceinline__ int pull_or_self(const OpDims& d, int periodic, int x, int y, int z,
                                            int i) {
  int sx = x - ex(i), sy = y - ey(i), sz = z - ez(i);
  if (sx < 0 || sx >= d.nx) return -1;
  if (periodic) {
    sy = wrapi(sy, d.ny);
    sz = wrapi(sz, d.nz);
  } else if (sy < 0 || sy >= d.ny || sz < 0 || sz >= d.nz) {
    return -1;
  }
  return (sx * d.ny + sy) * d.nz + sz;
}

template <class Re>
__global__ void k_stream(OpDims d, int periodic, const Re* __restrict__ f,
                         const Re* __restrict__ q, Re* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.n) return;
  int x, y, z;
  decode3(d, c, x, y, z);
  const size_t N = size_t(d.n);
  out[c] = f[c];
#pragma unroll
  for (int i = 1; i < Q; ++i) {
    const int io = opp(i);
    const Re qo = q[io * N + c];
    Re v;
    if (qo >= Re(0)) {
      const Re s_io = f[io * N + c];
      if (qo >= Re(0.5)) {
        const Re a = Re(1) / (Re(2) * fmin(qo, Re(1)));
        v = a * s_io + (Re(1) - a) * f[i * N + c];
      } else {
        const Re b = Re(2) * fmax(qo, Re(0));
        v = b * s_io + (Re(1) - b) * f[io * N + wrap3(d, x, y, z, ex(i), ey(i), ez(i))];
      }
    } else {
      const int s = pull_or_self(d, periodic, x, y, z, i);
      v = f[i * N + (s < 0 ? c : s)];
    }
    out[i * N + c] = v;
  }
}

// copy f and apply the inlet / outlet on the face cells
template <class Re>
__global__ void k_zou_he(OpDims d, int inlet, const Re* __restrict__ f, const Re* __restrict__ uf,
                         Re u0, Re u1, Re u2, int has_rho_t, Re rho_t, Re rho_out,
                         Re* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.n) return;
  const size_t N = size_t(d.n);
  const int x = c / (d.ny * d.nz);
  Re v[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) v[i] = f[i * N + c];
  if (inlet && x == 0) {
    Re ux = u0, uy = u1, uz = u2;
    if (uf) {
      const int fi = c % (d.ny * d.nz), fn = d.ny * d.nz;
      ux = uf[fi];
      uy = uf[fn + fi];
      uz = uf[2 * fn + fi];
    }
    if (has_rho_t) {
      const Re c3 = Re(1.0 / 3.0) * rho_t, c6 = Re(1.0 / 6.0) * rho_t;
      v[1] = v[2] + c3 * ux;
      v[7] = v[10] + c6 * (ux + uy);
      v[9] = v[8] + c6 * (ux - uy);
      v[11] = v[14] + c6 * (ux + uz);
      v[13] = v[12] + c6 * (ux - uz);
    } else {
      zou_he_inlet<Re>(v, ux, uy, uz);
    }
  }
  if (!inlet && x == d.nx - 1) zou_he_outlet<Re>(v, rho_out);
#pragma unroll
  for (int i = 0; i < Q; ++i) out[i * N + c] = v[i];
}

template <class Re>
__global__ void k_momentum_partials(int n, const Re* __restrict__ fp, const Re* __restrict__ fs,
                                    const Re* __restrict__ q, double* __restrict__ part) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double ax = 0, ay = 0, az = 0;
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

__global__ void k_drag(const double* __restrict__ force, double u, double area, double rho,
                       double* __restrict__ cd) {
  const double dyn = 0.5 * rho * u * u;
  *cd = fabs(force[0]) / (dyn * area + 1e-10);
}

__global__ void k_area_flags(OpDims d, int axis, const int32_t* __restrict__ solid,
                             int* __restrict__ col) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.n || solid[c] != 1) return;
  int x, y, z;
  decode3(d, c, x, y, z);
  int k;
  if (axis == 0) k = y * d.nz + z;
  else if (axis == 1) k = x * d.nz + z;
  else k = x * d.ny + y;
  col[k] = 1;
}

__global__ void k_count(int m, const int* __restrict__ col, double* __restrict__ out) {
  __shared__ long long sh[256];
  long long s = 0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) s += col[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = double(sh[0]);
}

// ------------------------------------------------------------------- VJPs ---

template <class Re>
__global__ void k_density_vjp(int n, const Re* __restrict__ g_rho, Re* __restrict__ g_f) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const Re g = g_rho[c];
#pragma unroll
  for (int i = 0; i < Q; ++i) g_f[size_t(i) * n + c] = g;
}

// u_a = j_a / rho with rho an input: g_f_i = sum_a g_a e_ia / rho,
// g_rho = -sum_a g_a u_a / rho
template <class Re>
__global__ void k_velocity_vjp(int n, const Re* __restrict__ f, const Re* __restrict__ rho,
                               const Re* __restrict__ g_u, Re* __restrict__ g_f,
                               Re* __restrict__ g_rho) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  Re v[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) v[i] = f[size_t(i) * n + c];
  Re jx, jy, jz;
  momentum<Re>(v, jx, jy, jz);
  const Re r = rho[c], ir = Re(1) / r;
  const Re gx = g_u[c] * ir, gy = g_u[size_t(n) + c] * ir, gz = g_u[2 * size_t(n) + c] * ir;
#pragma unroll
  for (int i = 0; i < Q; ++i)
    g_f[size_t(i) * n + c] = Re(ex(i)) * gx + Re(ey(i)) * gy + Re(ez(i)) * gz;
  if (g_rho) g_rho[c] = -(gx * jx + gy * jy + gz * jz) * ir;
}

template <class Re>
__global__ void k_equilibrium_vjp(int n, const Re* __restrict__ rho, const Re* __restrict__ u,
                                  const Re* __restrict__ g, Consts<Re> K, Re* __restrict__ g_rho,
                                  Re* __restrict__ g_u) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  Re v[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) v[i] = g[size_t(i) * n + c];
  Re gr, gx, gy, gz;
  equilibrium_vjp<Re>(v, rho[c], u[c], u[size_t(n) + c], u[2 * size_t(n) + c], K.w, gr, gx, gy,
                      gz);
  g_rho[c] = gr;
  g_u[c] = gx;
  g_u[size_t(n) + c] = gy;
  g_u[2 * size_t(n) + c] = gz;
}

template <class Re>
__global__ void k_collide_vjp(int n, const Re* __restrict__ f, const Re* __restrict__ tau_f,
                              Re tau, int mrt, Consts<Re> K, const Re* __restrict__ g,
                              Re* __restrict__ g_f, Re* __restrict__ g_tau) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  Re v[Q], l[Q], o[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    v[i] = f[size_t(i) * n + c];
    l[i] = g[size_t(i) * n + c];
  }
  Re gt = Re(0);
  collide_vjp<Re>(v, l, tau_f ? tau_f[c] : tau, mrt != 0, false, Re(0), K, o,
                  g_tau ? &gt : nullptr);
#pragma unroll
  for (int i = 0; i < Q; ++i) g_f[size_t(i) * n + c] = o[i];
  if (g_tau) g_tau[c] = gt;
}

// tau_eff(f, tau): cotangent g on tau_eff -> g_f, g_tau
template <class Re>
__global__ void k_smag_tau_vjp(int n, const Re* __restrict__ f, Re tau, Re c18, Consts<Re> K,
                               const Re* __restrict__ g, Re* __restrict__ g_f,
                               Re* __restrict__ g_tau) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  Re v[Q], gf[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    v[i] = f[size_t(i) * n + c];
    gf[i] = Re(0);
  }
  CellScalars<Re> cs;
  cell_scalars<Re>(v, cs);
  const Re rho = cs.rho, ux = cs.ux, uy = cs.uy, uz = cs.uz;
  Re sst[6];
  neq_stress<Re>(cs.p, K.w, rho, ux, uy, uz, sst);
  const Re pi = smag_pi<Re>(sst);
  const Re inv_rr = inv_rho_eps<Re>(rho, Re(1) / rho);
  const Re R = sqrt(tau * tau + c18 * pi * inv_rr);
  const Re gte = g[c];
  const Re gX = (R > Re(0)) ? Re(0.5) * gte / (Re(2) * R) : Re(0);
  if (g_tau) g_tau[c] = Re(0.5) * gte + gX * Re(2) * tau;
  const Re g_pi = gX * c18 * inv_rr;
  const Re g_rho_direct = -gX * c18 * pi * inv_rr * inv_rr;
  if (pi > Re(0)) {
    const Re ip = g_pi / pi;
    Re gs[6] = {ip * sst[0], ip * sst[1], ip * sst[2], Re(2) * ip * sst[3], Re(2) * ip * sst[4],
                Re(2) * ip * sst[5]};
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      const int x = ex(i), y = ey(i), z = ez(i);
      Re t = Re(0);
      if (x != 0) t += gs[0];
      if (y != 0) t += gs[1];
      if (z != 0) t += gs[2];
      if (x * y != 0) t += Re(x * y) * gs[3];
      if (x * z != 0) t += Re(x * z) * gs[4];
      if (y * z != 0) t += Re(y * z) * gs[5];
      gf[i] += t;
    }
    Re er, exx, eyy, ezz;
    eq_second_vjp<Re>(K.w, rho, ux, uy, uz, gs, er, exx, eyy, ezz);
    macro_vjp_add<Re>(-er, -exx, -eyy, -ezz, rho, ux, uy, uz, gf);
  }
#pragma unroll
  for (int i = 0; i < Q; ++i) g_f[size_t(i) * n + c] = gf[i] + g_rho_direct;
}

template <class Re>
__global__ void k_soft_bounce_vjp(int n, const Re* __restrict__ f, const Re* __restrict__ p,
                                  const Re* __restrict__ g, Re* __restrict__ g_f,
                                  Re* __restrict__ g_p) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const Re pc = p[c];
  Re gv[Q];
  Re gp = Re(0);
#pragma unroll
  for (int i = 0; i < Q; ++i) gv[i] = g[size_t(i) * n + c];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    g_f[size_t(i) * n + c] = (Re(1) - pc) * gv[i] + pc * gv[opp(i)];
    gp += gv[i] * (f[size_t(opp(i)) * n + c] - f[size_t(i) * n + c]);
  }
  if (g_p) g_p[c] = gp;
}

// Transposed stream with a dense q (gather form), and dJ/dq per link.
template <class Re>
__global__ void k_stream_vjp(OpDims d, int periodic, const Re* __restrict__ f,
                             const Re* __restrict__ q, const Re* __restrict__ g,
                             Re* __restrict__ g_f, Re* __restrict__ g_q) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.n) return;
  int x, y, z;
  decode3(d, c, x, y, z);
  const size_t N = size_t(d.n);
  Re mu[Q];
  mu[0] = g[c];
#pragma unroll
  for (int j = 1; j < Q; ++j) {
    Re v = Re(0);
    // (a) output (x, j) at the pull neighbour x = c + e_j reads f_j(c) when normal
    const int nb = pull_or_self(d, periodic, x, y, z, opp(j));
    if (nb >= 0 && q[opp(j) * N + nb] < Re(0)) v += g[j * N + nb];
    // (b) output (c, j) falls back to f_j(c)
    if (pull_or_self(d, periodic, x, y, z, j) < 0 && q[opp(j) * N + c] < Re(0)) v += g[j * N + c];
    // (e) second-fluid term of a q < 0.5 link of the neighbour c + e_j (wrapped)
    const int w = wrap3(d, x, y, z, ex(j), ey(j), ez(j));
    const Re qw = q[j * N + w];
    if (qw >= Re(0) && qw < Re(0.5)) v += (Re(1) - Re(2) * fmax(qw, Re(0))) * g[opp(j) * N + w];
    mu[j] = v;
  }
  // own wall outputs i (q[opp i](c) >= 0)
#pragma unroll
  for (int i = 1; i < Q; ++i) {
    const int io = opp(i);
    const Re qo = q[io * N + c];
    Re gq = Re(0);
    if (qo >= Re(0)) {
      const Re gi = g[i * N + c];
      const Re s_io = f[io * N + c];
      if (qo >= Re(0.5)) {
        const Re qc = fmin(qo, Re(1));
        const Re a = Re(1) / (Re(2) * qc);
        mu[io] += a * gi;
        mu[i] += (Re(1) - a) * gi;
        gq = gi * clip_weight<Re>(qo, Re(0.5), Re(1)) * (-(s_io - f[i * N + c]) / (Re(2) * qc * qc));
      } else {
        const Re b = Re(2) * fmax(qo, Re(0));
        mu[io] += b * gi;
        const Re s_nb = f[io * N + wrap3(d, x, y, z, ex(i), ey(i), ez(i))];
        gq = gi * clip_weight<Re>(qo, Re(0), Re(0.5)) * Re(2) * (s_io - s_nb);
      }
    }
    if (g_q) g_q[io * N + c] = gq;
  }
  if (g_q) g_q[c] = Re(0);
#pragma unroll
  for (int j = 0; j < Q; ++j) g_f[j * N + c] = mu[j];
}

template <class Re>
__global__ void k_zou_he_vjp(OpDims d, int inlet, const Re* __restrict__ f,
                             const Re* __restrict__ uf, Re u0, Re u1, Re u2, int has_rho_t,
                             Re rho_t, Re rho_out, const Re* __restrict__ g, Re* __restrict__ g_f,
                             Re* __restrict__ g_uface, Re* __restrict__ g_rho_face) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.n) return;
  const size_t N = size_t(d.n);
  const int fn = d.ny * d.nz;
  const int x = c / fn, fi = c % fn;
  Re l[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) l[i] = g[i * N + c];
  if (inlet && x == 0) {
    Re ux = u0, uy = u1, uz = u2;
    if (uf) {
      ux = uf[fi];
      uy = uf[fn + fi];
      uz = uf[2 * fn + fi];
    }
    Re v[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) v[i] = f[i * N + c];
    const Re c3 = Re(1.0 / 3.0), c6 = Re(1.0 / 6.0);
    const Re k0 = v[0] + v[3] + v[4] + v[5] + v[6] + v[15] + v[16] + v[17] + v[18];
    const Re kn = v[2] + v[8] + v[10] + v[12] + v[14];
    const Re rho = has_rho_t ? rho_t : (k0 + Re(2) * kn) / (Re(1) - ux);
    // cotangents of the prescribed velocity
    const Re grho = c3 * ux * l[1] + c6 * (ux + uy) * l[7] + c6 * (ux - uy) * l[9] +
                    c6 * (ux + uz) * l[11] + c6 * (ux - uz) * l[13];
    if (g_uface) {
      Re gux = rho * (c3 * l[1] + c6 * (l[7] + l[9] + l[11] + l[13]));
      if (!has_rho_t) gux += grho * rho / (Re(1) - ux);     // d rho / d ux
      g_uface[fi] = gux;
      g_uface[fn + fi] = rho * c6 * (l[7] - l[9]);
      g_uface[2 * fn + fi] = rho * c6 * (l[11] - l[13]);
    }
    Re o[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) o[j] = l[j];
    o[1] = o[7] = o[9] = o[11] = o[13] = Re(0);
    o[2] += l[1];
    o[10] += l[7];
    o[8] += l[9];
    o[14] += l[11];
    o[12] += l[13];
    if (!has_rho_t) {
      const Re dd = grho / (Re(1) - ux);
      o[0] += dd; o[3] += dd; o[4] += dd; o[5] += dd; o[6] += dd;
      o[15] += dd; o[16] += dd; o[17] += dd; o[18] += dd;
      o[2] += Re(2) * dd; o[8] += Re(2) * dd; o[10] += Re(2) * dd; o[12] += Re(2) * dd;
      o[14] += Re(2) * dd;
    }
#pragma unroll
    for (int j = 0; j < Q; ++j) l[j] = o[j];
  }
  if (!inlet && x == d.nx - 1) {
    const Re c3 = Re(1.0 / 3.0), c6 = Re(1.0 / 6.0);
    // f2 = f1 - c3 (K - rho_out) etc. with K = k0 + 2 kpos: d/d rho_out = c3 / c6
    if (g_rho_face) g_rho_face[fi] = c3 * l[2] + c6 * (l[10] + l[8] + l[14] + l[12]);
    const Re gu = -rho_out * (c3 * l[2] + c6 * (l[10] + l[8] + l[14] + l[12]));
    const Re dd = gu / rho_out;
    Re o[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) o[j] = l[j];
    o[2] = o[10] = o[8] = o[14] = o[12] = Re(0);
    o[1] += l[2];
    o[7] += l[10];
    o[9] += l[8];
    o[11] += l[14];
    o[13] += l[12];
    o[0] += dd; o[3] += dd; o[4] += dd; o[5] += dd; o[6] += dd;
    o[15] += dd; o[16] += dd; o[17] += dd; o[18] += dd;
    o[1] += Re(2) * dd; o[7] += Re(2) * dd; o[9] += Re(2) * dd; o[11] += Re(2) * dd;
    o[13] += Re(2) * dd;
#pragma unroll
    for (int j = 0; j < Q; ++j) l[j] = o[j];
  }
#pragma unroll
  for (int j = 0; j < Q; ++j) g_f[j * N + c] = l[j];
}

// F is linear in (f_post, f_streamed): g_f_post[i] = [q_i >= 0] e_i.gF,
// g_f_streamed[opp i] = the same.
template <class Re>
__global__ void k_momentum_vjp(int n, const Re* __restrict__ q, const double* __restrict__ gF,
                               Re* __restrict__ g_fp, Re* __restrict__ g_fs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const size_t N = size_t(n);
  const double gx = gF[0], gy = gF[1], gz = gF[2];
  g_fp[c] = Re(0);
  g_fs[c] = Re(0);
#pragma unroll
  for (int i = 1; i < Q; ++i) {
    const Re v = q[i * N + c] >= Re(0) ? Re(ex(i) * gx + ey(i) * gy + ez(i) * gz) : Re(0);
    if (g_fp) g_fp[i * N + c] = v;
    const Re w = q[opp(i) * N + c] >= Re(0)
                     ? Re(ex(opp(i)) * gx + ey(opp(i)) * gy + ez(opp(i)) * gz) : Re(0);
    if (g_fs) g_fs[i * N + c] = w;
  }
}

template <class Re>
int check_dims(int nx, int ny, int nz) {
  if (nx < 1 || ny < 1 || nz < 1) return set_error(LBM_ERR_ARG, "dimensions must be >= 1");
  if ((long long)nx * ny * nz * Q >= (1LL << 31))
    return set_error(LBM_ERR_UNSUPPORTED, "19*cells must be < 2^31");
  return LBM_OK;
}

int check_dtype(int dtype) {
  if (dtype != LBM_F32 && dtype != LBM_F64)
    return set_error(LBM_ERR_UNSUPPORTED, "per-op kernels take LBM_F32 or LBM_F64");
  return LBM_OK;
}

#define LBM_NEED(p, name) \
  do { if (!(p)) return set_error(LBM_ERR_ARG, "null pointer: " name); } while (0)

// dispatch helper: body is instantiated for float and double
#define LBM_DISPATCH(dtype, BODY)            \
  do {                                       \
    if ((dtype) == LBM_F64) {                \
      using Re = double;                     \
      BODY;                                  \
    } else {                                 \
      using Re = float;                      \
      BODY;                                  \
    }                                        \
  } while (0)

}  // namespace
}  // namespace lbm

using namespace lbm;

extern "C" {

int lbm_compute_density(int dtype, const void* f, void* rho, int nx, int ny, int nz,
                        void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(rho, "rho");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_density<Re><<<nblk(n), 256, 0, st>>>(n, (const Re*)f, (Re*)rho)));
  return cuda_check(cudaGetLastError(), "compute_density");
}

int lbm_compute_velocity(int dtype, const void* f, const void* rho, void* u, int nx, int ny,
                         int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(rho, "rho");
  LBM_NEED(u, "u");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_velocity<Re><<<nblk(n), 256, 0, st>>>(n, (const Re*)f, (const Re*)rho,
                                                                 (Re*)u)));
  return cuda_check(cudaGetLastError(), "compute_velocity");
}

int lbm_equilibrium(int dtype, const void* rho, const void* u, void* feq, int nx, int ny, int nz,
                    int flags, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(rho, "rho");
  LBM_NEED(u, "u");
  LBM_NEED(feq, "feq");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_equilibrium<Re><<<nblk(n), 256, 0, st>>>(
                          n, (const Re*)rho, (const Re*)u, op_consts<Re>(flags), (Re*)feq)));
  return cuda_check(cudaGetLastError(), "equilibrium");
}

static int collide_op(int dtype, const void* f, const void* tau_field, double tau, void* out,
                      int nx, int ny, int nz, int flags, int mrt, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(out, "out");
  if (!tau_field && !(tau > 0.0)) return set_error(LBM_ERR_ARG, "tau must be > 0");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_collide<Re><<<nblk(n), 256, 0, st>>>(
                          n, (const Re*)f, (const Re*)tau_field, Re(tau), mrt,
                          op_consts<Re>(flags), (Re*)out)));
  return cuda_check(cudaGetLastError(), mrt ? "mrt" : "bgk");
}

int lbm_bgk(int dtype, const void* f, const void* tau_field, double tau, void* out, int nx,
            int ny, int nz, int flags, void* stream) {
  return collide_op(dtype, f, tau_field, tau, out, nx, ny, nz, flags, 0, stream);
}

int lbm_mrt(int dtype, const void* f, const void* tau_field, double tau, void* out, int nx,
            int ny, int nz, int flags, void* stream) {
  return collide_op(dtype, f, tau_field, tau, out, nx, ny, nz, flags, 1, stream);
}

int lbm_smagorinsky_tau(int dtype, const void* f, double tau, double cs, void* tau_eff, int nx,
                        int ny, int nz, int flags, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(tau_eff, "tau_eff");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_smag_tau<Re><<<nblk(n), 256, 0, st>>>(
                          n, (const Re*)f, Re(tau), Re(18.0 * (cs * cs)), op_consts<Re>(flags),
                          (Re*)tau_eff)));
  return cuda_check(cudaGetLastError(), "smagorinsky_tau");
}

int lbm_soft_bounce_back(int dtype, const void* f, const void* porosity, void* out, int nx,
                         int ny, int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(porosity, "porosity");
  LBM_NEED(out, "out");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_soft_bounce<Re><<<nblk(n), 256, 0, st>>>(n, (const Re*)f,
                                                                    (const Re*)porosity,
                                                                    (Re*)out)));
  return cuda_check(cudaGetLastError(), "soft_bounce_back");
}

int lbm_stream(int dtype, const void* f, const void* q, int periodic_yz, void* out, int nx, int ny,
               int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(q, "q");
  LBM_NEED(out, "out");
  const OpDims d{nx, ny, nz, nx * ny * nz};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_stream<Re><<<nblk(d.n), 256, 0, st>>>(d, periodic_yz ? 1 : 0,
                                                                 (const Re*)f, (const Re*)q,
                                                                 (Re*)out)));
  return cuda_check(cudaGetLastError(), "stream");
}

int lbm_zou_he_inlet(int dtype, const void* f, const void* u_face, const double* velocity,
                     int has_rho_target, double rho_target, void* out, int nx, int ny, int nz,
                     void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(out, "out");
  if (!u_face && !velocity) return set_error(LBM_ERR_ARG, "zou_he_inlet: no velocity");
  const OpDims d{nx, ny, nz, nx * ny * nz};
  const double v0 = velocity ? velocity[0] : 0.0, v1 = velocity ? velocity[1] : 0.0,
               v2 = velocity ? velocity[2] : 0.0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_zou_he<Re><<<nblk(d.n), 256, 0, st>>>(
                          d, 1, (const Re*)f, (const Re*)u_face, Re(v0), Re(v1), Re(v2),
                          has_rho_target, Re(rho_target), Re(1), (Re*)out)));
  return cuda_check(cudaGetLastError(), "zou_he_inlet");
}

int lbm_zou_he_outlet(int dtype, const void* f, double rho_out, void* out, int nx, int ny, int nz,
                      void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(out, "out");
  const OpDims d{nx, ny, nz, nx * ny * nz};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_zou_he<Re><<<nblk(d.n), 256, 0, st>>>(
                          d, 0, (const Re*)f, nullptr, Re(0), Re(0), Re(0), 0, Re(0),
                          Re(rho_out), (Re*)out)));
  return cuda_check(cudaGetLastError(), "zou_he_outlet");
}

int lbm_momentum_exchange(int dtype, const void* f_post, const void* f_streamed, const void* q,
                          double* force, int nx, int ny, int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f_post, "f_post");
  LBM_NEED(f_streamed, "f_streamed");
  LBM_NEED(q, "q");
  LBM_NEED(force, "force");
  LBM_TRY(check_align(force, 8, "force"));
  const int n = nx * ny * nz;
  const int nb = nblk(n);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* part = nullptr;
  LBM_TRY(cuda_check(cudaMallocAsync((void**)&part, size_t(nb) * 3 * sizeof(double), st),
                     "cudaMallocAsync"));
  LBM_DISPATCH(dtype, (k_momentum_partials<Re><<<nb, 256, 0, st>>>(n, (const Re*)f_post,
                                                                     (const Re*)f_streamed,
                                                                     (const Re*)q, part)));
  int rc = cuda_check(cudaGetLastError(), "momentum_exchange");
  if (rc == LBM_OK) rc = cuda_check(launch_force_sum(part, nb, force, st), "force reduce");
  cudaFreeAsync(part, st);
  return rc;
}

int lbm_drag_coefficient(const double* force, double inlet_velocity, double area, double rho,
                         double* cd, void* stream) {
  LBM_NEED(force, "force");
  LBM_NEED(cd, "cd");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_drag<<<1, 1, 0, st>>>(force, inlet_velocity, area, rho, cd);
  return cuda_check(cudaGetLastError(), "drag_coefficient");
}

int lbm_projected_area(const int32_t* solid, int axis, double* area, int nx, int ny, int nz,
                       void* stream) {
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(solid, "solid");
  LBM_NEED(area, "area");
  if (axis < 0 || axis > 2) return set_error(LBM_ERR_ARG, "axis must be 0, 1 or 2");
  const OpDims d{nx, ny, nz, nx * ny * nz};
  const int m = axis == 0 ? ny * nz : (axis == 1 ? nx * nz : nx * ny);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int* col = nullptr;
  LBM_TRY(cuda_check(cudaMallocAsync((void**)&col, size_t(m) * sizeof(int), st), "cudaMallocAsync"));
  int rc = cuda_check(cudaMemsetAsync(col, 0, size_t(m) * sizeof(int), st), "memset");
  if (rc == LBM_OK) {
    k_area_flags<<<nblk(d.n), 256, 0, st>>>(d, axis, solid, col);
    k_count<<<1, 256, 0, st>>>(m, col, area);
    rc = cuda_check(cudaGetLastError(), "projected_area");
  }
  cudaFreeAsync(col, st);
  return rc;
}

// ---- VJPs ------------------------------------------------------------------

int lbm_compute_density_vjp(int dtype, const void* g_rho, void* g_f, int nx, int ny, int nz,
                            void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(g_rho, "g_rho");
  LBM_NEED(g_f, "g_f");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_density_vjp<Re><<<nblk(n), 256, 0, st>>>(n, (const Re*)g_rho,
                                                                    (Re*)g_f)));
  return cuda_check(cudaGetLastError(), "compute_density_vjp");
}

int lbm_compute_velocity_vjp(int dtype, const void* f, const void* rho, const void* g_u,
                             void* g_f, void* g_rho, int nx, int ny, int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(rho, "rho");
  LBM_NEED(g_u, "g_u");
  LBM_NEED(g_f, "g_f");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_velocity_vjp<Re><<<nblk(n), 256, 0, st>>>(
                          n, (const Re*)f, (const Re*)rho, (const Re*)g_u, (Re*)g_f,
                          (Re*)g_rho)));
  return cuda_check(cudaGetLastError(), "compute_velocity_vjp");
}

int lbm_equilibrium_vjp(int dtype, const void* rho, const void* u, const void* g_feq, void* g_rho,
                        void* g_u, int nx, int ny, int nz, int flags, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(rho, "rho");
  LBM_NEED(u, "u");
  LBM_NEED(g_feq, "g_feq");
  LBM_NEED(g_rho, "g_rho");
  LBM_NEED(g_u, "g_u");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_equilibrium_vjp<Re><<<nblk(n), 256, 0, st>>>(
                          n, (const Re*)rho, (const Re*)u, (const Re*)g_feq, op_consts<Re>(flags),
                          (Re*)g_rho, (Re*)g_u)));
  return cuda_check(cudaGetLastError(), "equilibrium_vjp");
}

static int collide_vjp_op(int dtype, const void* f, const void* tau_field, double tau,
                          const void* g_out, void* g_f, void* g_tau, int nx, int ny, int nz,
                          int flags, int mrt, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(g_out, "g_out");
  LBM_NEED(g_f, "g_f");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_collide_vjp<Re><<<nblk(n), 256, 0, st>>>(
                          n, (const Re*)f, (const Re*)tau_field, Re(tau), mrt,
                          op_consts<Re>(flags), (const Re*)g_out, (Re*)g_f, (Re*)g_tau)));
  return cuda_check(cudaGetLastError(), mrt ? "mrt_vjp" : "bgk_vjp");
}

int lbm_bgk_vjp(int dtype, const void* f, const void* tau_field, double tau, const void* g_out,
                void* g_f, void* g_tau, int nx, int ny, int nz, int flags, void* stream) {
  return collide_vjp_op(dtype, f, tau_field, tau, g_out, g_f, g_tau, nx, ny, nz, flags, 0, stream);
}

int lbm_mrt_vjp(int dtype, const void* f, const void* tau_field, double tau, const void* g_out,
                void* g_f, void* g_tau, int nx, int ny, int nz, int flags, void* stream) {
  return collide_vjp_op(dtype, f, tau_field, tau, g_out, g_f, g_tau, nx, ny, nz, flags, 1, stream);
}

int lbm_smagorinsky_tau_vjp(int dtype, const void* f, double tau, double cs,
                            const void* g_tau_eff, void* g_f, void* g_tau, int nx, int ny, int nz,
                            int flags, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(g_tau_eff, "g_tau_eff");
  LBM_NEED(g_f, "g_f");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_smag_tau_vjp<Re><<<nblk(n), 256, 0, st>>>(
                          n, (const Re*)f, Re(tau), Re(18.0 * (cs * cs)), op_consts<Re>(flags),
                          (const Re*)g_tau_eff, (Re*)g_f, (Re*)g_tau)));
  return cuda_check(cudaGetLastError(), "smagorinsky_tau_vjp");
}

int lbm_soft_bounce_back_vjp(int dtype, const void* f, const void* porosity, const void* g_out,
                             void* g_f, void* g_porosity, int nx, int ny, int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(porosity, "porosity");
  LBM_NEED(g_out, "g_out");
  LBM_NEED(g_f, "g_f");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_soft_bounce_vjp<Re><<<nblk(n), 256, 0, st>>>(
                          n, (const Re*)f, (const Re*)porosity, (const Re*)g_out, (Re*)g_f,
                          (Re*)g_porosity)));
  return cuda_check(cudaGetLastError(), "soft_bounce_back_vjp");
}

int lbm_stream_vjp(int dtype, const void* f, const void* q, int periodic_yz, const void* g_out,
                   void* g_f, void* g_q, int nx, int ny, int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(q, "q");
  LBM_NEED(g_out, "g_out");
  LBM_NEED(g_f, "g_f");
  const OpDims d{nx, ny, nz, nx * ny * nz};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_stream_vjp<Re><<<nblk(d.n), 256, 0, st>>>(
                          d, periodic_yz ? 1 : 0, (const Re*)f, (const Re*)q, (const Re*)g_out,
                          (Re*)g_f, (Re*)g_q)));
  return cuda_check(cudaGetLastError(), "stream_vjp");
}

int lbm_zou_he_inlet_vjp(int dtype, const void* f, const void* u_face, const double* velocity,
                         int has_rho_target, double rho_target, const void* g_out, void* g_f,
                         void* g_u_face, int nx, int ny, int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(g_out, "g_out");
  LBM_NEED(g_f, "g_f");
  if (!u_face && !velocity) return set_error(LBM_ERR_ARG, "zou_he_inlet_vjp: no velocity");
  const OpDims d{nx, ny, nz, nx * ny * nz};
  const double v0 = velocity ? velocity[0] : 0.0, v1 = velocity ? velocity[1] : 0.0,
               v2 = velocity ? velocity[2] : 0.0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_zou_he_vjp<Re><<<nblk(d.n), 256, 0, st>>>(
                          d, 1, (const Re*)f, (const Re*)u_face, Re(v0), Re(v1), Re(v2),
                          has_rho_target, Re(rho_target), Re(1), (const Re*)g_out, (Re*)g_f,
                          (Re*)g_u_face, nullptr)));
  return cuda_check(cudaGetLastError(), "zou_he_inlet_vjp");
}

int lbm_zou_he_outlet_vjp(int dtype, const void* f, double rho_out, const void* g_out, void* g_f,
                          void* g_rho_out_face, int nx, int ny, int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(f, "f");
  LBM_NEED(g_out, "g_out");
  LBM_NEED(g_f, "g_f");
  const OpDims d{nx, ny, nz, nx * ny * nz};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_zou_he_vjp<Re><<<nblk(d.n), 256, 0, st>>>(
                          d, 0, (const Re*)f, nullptr, Re(0), Re(0), Re(0), 0, Re(0),
                          Re(rho_out), (const Re*)g_out, (Re*)g_f, nullptr,
                          (Re*)g_rho_out_face)));
  return cuda_check(cudaGetLastError(), "zou_he_outlet_vjp");
}

int lbm_momentum_exchange_vjp(int dtype, const void* q, const double* g_force, void* g_f_post,
                              void* g_f_streamed, int nx, int ny, int nz, void* stream) {
  LBM_TRY(check_dtype(dtype));
  LBM_TRY(check_dims<float>(nx, ny, nz));
  LBM_NEED(q, "q");
  LBM_NEED(g_force, "g_force");
  if (!g_f_post || !g_f_streamed)
    return set_error(LBM_ERR_ARG, "momentum_exchange_vjp: both outputs are required");
  const int n = nx * ny * nz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_DISPATCH(dtype, (k_momentum_vjp<Re><<<nblk(n), 256, 0, st>>>(
                          n, (const Re*)q, g_force, (Re*)g_f_post, (Re*)g_f_streamed)));
  return cuda_check(cudaGetLastError(), "momentum_exchange_vjp");
}

}  // extern "C"
