// D3Q19 lattice, population storage and per-cell collision math for sm_103a.
//
// Everything here is per-cell register arithmetic shared by the fused step
// kernels, the adjoint kernels and the per-op drop-in kernels.
//
// Reference semantics (jax_lbm):
//   velocities / opposite / cs^2         core/lattice.py:29-82
//   MRT moment basis, norms, rates       core/lattice.py:88-391
//   equilibrium                          core/equilibrium.py:90-151
//   bgk, mrt, smagorinsky_tau            core/collision.py:46-270
// The hand-derived vector-Jacobian products (``*_vjp``) are the transposes of
// those maps; they replace what jax.grad derives through the same code.
#pragma once

#include <cmath>
#include <cstring>
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace lbm {

constexpr int Q = 19;

__host__ __device__ constexpr int ex(int i) {
  constexpr int t[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
  return t[i];
}
__host__ __device__ constexpr int ey(int i) {
  constexpr int t[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
  return t[i];
}
__host__ __device__ constexpr int ez(int i) {
  constexpr int t[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
  return t[i];
}
__host__ __device__ constexpr int opp(int i) {
  constexpr int t[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
  return t[i];
}

// Moment matrix row k evaluated at velocity i (d'Humieres 2002 basis, rows in
// the order rho, e, eps, jx, qx, jy, qy, jz, qz, 3pxx, 3pixx, pww, piww, pxy,
// pyz, pxz, mx, my, mz).
__host__ __device__ constexpr int mrow(int k, int i) {
  const int x = ex(i), y = ey(i), z = ez(i);
  const int e2 = x * x + y * y + z * z;
  switch (k) {
    case 0: return 1;
    case 1: return 19 * e2 - 30;
    case 2: return (21 * e2 * e2 - 53 * e2 + 24) / 2;
    case 3: return x;
    case 4: return (5 * e2 - 9) * x;
    case 5: return y;
    case 6: return (5 * e2 - 9) * y;
    case 7: return z;
    case 8: return (5 * e2 - 9) * z;
    case 9: return 3 * x * x - e2;
    case 10: return (3 * e2 - 5) * (3 * x * x - e2);
    case 11: return y * y - z * z;
    case 12: return (3 * e2 - 5) * (y * y - z * z);
    case 13: return x * y;
    case 14: return y * z;
    case 15: return x * z;
    case 16: return (y * y - z * z) * x;
    case 17: return (z * z - x * x) * y;
    default: return (x * x - y * y) * z;
  }
}
__host__ __device__ constexpr int mnorm(int k) {
  int s = 0;
  for (int i = 0; i < Q; ++i) s += mrow(k, i) * mrow(k, i);
  return s;
}
__host__ __device__ constexpr bool is_stress(int k) {
  return k == 9 || k == 11 || k == 13 || k == 14 || k == 15;
}
__host__ __device__ constexpr bool is_conserved(int k) {
  return k == 0 || k == 3 || k == 5 || k == 7;
}

// ---------------------------------------------------------------------------
// Population storage.  FP32/FP64 store f itself; FP16/BF16 store the deviation
// f_i - w from a per-direction offset w that the caller passes (the solver
// uses the free-stream equilibrium); arithmetic stays FP32.
// ---------------------------------------------------------------------------
// Read-only global loads of the population sweeps with a 256-byte L2
// prefetch (ld.global.nc.L2::256B): the sweeps stream through HBM, and
// fetching the whole 256-byte span an access falls in measured about 1 %
// faster per FP32 step than plain ld.global.nc.
#ifndef LBM_L2_PREFETCH
#define LBM_L2_PREFETCH 1
#endif
__device__ __forceinline__ float ldg_s(const float* p) {
#if LBM_L2_PREFETCH
  float v;
  asm("ld.global.nc.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
#else
  return __ldg(p);
#endif
}
__device__ __forceinline__ float2 ldg_s(const float2* p) {
#if LBM_L2_PREFETCH
  float2 v;
  asm("ld.global.nc.L2::256B.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
#else
  return __ldg(p);
#endif
}
__device__ __forceinline__ unsigned short ldg_s16(const void* p) {
#if LBM_L2_PREFETCH
  unsigned short v;
  asm("ld.global.nc.L2::256B.b16 %0, [%1];" : "=h"(v) : "l"(p));
  return v;
#else
  return __ldg(static_cast<const unsigned short*>(p));
#endif
}
__device__ __forceinline__ unsigned ldg_s32(const void* p) {
#if LBM_L2_PREFETCH
  unsigned v;
  asm("ld.global.nc.L2::256B.b32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
#else
  return __ldg(static_cast<const unsigned*>(p));
#endif
}
__device__ __forceinline__ __half ldg_s(const __half* p) { return __ushort_as_half(ldg_s16(p)); }
__device__ __forceinline__ __nv_bfloat16 ldg_s(const __nv_bfloat16* p) {
  return __ushort_as_bfloat16(ldg_s16(p));
}
__device__ __forceinline__ __half2 ldg_s(const __half2* p) {
  const unsigned u = ldg_s32(p);
  __half2 h;
  memcpy(&h, &u, 4);
  return h;
}
__device__ __forceinline__ __nv_bfloat162 ldg_s(const __nv_bfloat162* p) {
  const unsigned u = ldg_s32(p);
  __nv_bfloat162 h;
  memcpy(&h, &u, 4);
  return h;
}

template <class St> struct Storage;
template <> struct Storage<float> {
  using Re = float;
  static __device__ __forceinline__ float ld(const float* p, float) { return ldg_s(p); }
  static __device__ __forceinline__ void st(float* p, float v, float) { *p = v; }
};
template <> struct Storage<double> {
  using Re = double;
  static __device__ __forceinline__ double ld(const double* p, double) { return __ldg(p); }
  static __device__ __forceinline__ void st(double* p, double v, double) { *p = v; }
};
template <> struct Storage<__half> {
  using Re = float;
  static __device__ __forceinline__ float ld(const __half* p, float w) {
    return w + __half2float(ldg_s(p));
  }
  static __device__ __forceinline__ void st(__half* p, float v, float w) {
    *p = __float2half_rn(v - w);
  }
};
template <> struct Storage<__nv_bfloat16> {
  using Re = float;
  static __device__ __forceinline__ float ld(const __nv_bfloat16* p, float w) {
    return w + __bfloat162float(ldg_s(p));
  }
  static __device__ __forceinline__ void st(__nv_bfloat16* p, float v, float w) {
    *p = __float2bfloat16_rn(v - w);
  }
};

// Lattice constants handed to kernels by value (constant bank).  ``w`` and
// ``rate`` are either the reference's float32-rounded values or the exact
// rationals, chosen on the host.
template <class Re> struct Consts {
  Re w[Q];
  Re rate[Q];   // fixed MRT rates; stress slots are overwritten by omega
};

// Compile-time lattice constants for FP32 arithmetic.  Rounded to float, the
// exact weights 1/3, 1/18, 1/36 and the reference's float32 weights
// (lattice.py:53-60) are the same numbers, and so are the MRT rates
// (lattice.py:106-126); a kernel computing in FP32 can therefore take them
// as immediates instead of reading them from the parameter bank.
struct FixedWeightsF {
  __host__ __device__ constexpr float operator[](int i) const {
    return i == 0 ? float(1.0 / 3.0) : (i < 7 ? float(1.0 / 18.0) : float(1.0 / 36.0));
  }
};
struct FixedRatesF {
  __host__ __device__ constexpr float operator[](int k) const {
    return k == 1 ? float(1.19)
         : (k == 2 || k == 10 || k == 12) ? float(1.4)
         : (k == 4 || k == 6 || k == 8) ? float(1.2)
         : (k >= 16) ? float(1.98) : 0.0f;
  }
};
struct FixedConstsF {
  FixedWeightsF w;
  FixedRatesF rate;
};

// Scalar type of an arithmetic type (a packed two-lane type names its lane
// type) and whether that scalar is 32-bit.
template <class Re> struct ScalarOf { using type = Re; };
template <class Re> struct IsSingle {
  static constexpr bool value = sizeof(typename ScalarOf<Re>::type) == 4;
};

// Reciprocal and square root of the collision arithmetic in FP32 device
// code.  LBM_FAST_MATH 0 (the default): the correctly rounded operations;
// 1: the hardware approximations rcp.approx.ftz.f32 and sqrt.approx.ftz.f32;
// 2: rcp.approx.f32 refined by one Newton step and sqrt.approx.f32.  Measured
// at 256x128x128 (MRT + Smagorinsky sphere), 1 and 2 take the 16-bit step
// from 92 / 94 us to 88-90 us and the FP32 step from 112.6 to 109-110 us,
// but move the FP32 dCd/dr from 3.5e-7 to 1.6e-5 of FP64 over 2000 steps
// (the FP16 one from 6.4e-4 to 0.9-1.9e-3), past the accuracy bars, so
// they stay off.  FP64 and host code always round correctly.
#ifndef LBM_FAST_MATH
#define LBM_FAST_MATH 0
#endif
__host__ __device__ __forceinline__ float lbm_sqrt(float x) {
#if defined(__CUDA_ARCH__) && LBM_FAST_MATH == 1
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#elif defined(__CUDA_ARCH__) && LBM_FAST_MATH == 2
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return sqrtf(x);
#endif
}
__host__ __device__ __forceinline__ double lbm_sqrt(double x) { return sqrt(x); }
__host__ __device__ __forceinline__ float lbm_rcp(float x) {
#if defined(__CUDA_ARCH__) && LBM_FAST_MATH == 1
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#elif defined(__CUDA_ARCH__) && LBM_FAST_MATH == 2
  float r;
  asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  // Newton step r += r (1 - x r)
  return fmaf(r, fmaf(-x, r, 1.0f), r);
#else
  return 1.0f / x;
#endif
}
__host__ __device__ __forceinline__ double lbm_rcp(double x) { return 1.0 / x; }

// Output sink of the collision routines: an array (out[i] = v) or a callable
// out(i, v) that consumes each post-collision population as it is produced
// (a kernel that stores them straight away holds no output array).
template <class Re>
__host__ __device__ __forceinline__ void emit(Re* out, int i, Re v) {
  out[i] = v;
}
template <class F, class Re>
__host__ __device__ __forceinline__ auto emit(F& out, int i, Re v) -> decltype(out(i, v), void()) {
  out(i, v);
}

// b > 0 ? a / b : 0, and "is any lane > 0" (a packed type overloads both).
template <class Re>
__host__ __device__ __forceinline__ Re div_if_pos(Re a, Re b) {
#if LBM_FAST_MATH
  return b > Re(0) ? Re(a * lbm_rcp(b)) : Re(0);
#else
  return b > Re(0) ? Re(a / b) : Re(0);
#endif
}
template <class Re>
__host__ __device__ __forceinline__ bool any_pos(Re v) {
  return v > Re(0);
}

// Derivative weight of clip(x, lo, hi) = min(max(x, lo), hi) under jax's
// convention: 1 strictly inside, 1/2 at a tie with a bound, 0 outside.
template <class Re>
__host__ __device__ __forceinline__ Re clip_weight(Re x, Re lo, Re hi) {
  if (x > lo && x < hi) return Re(1);
  if (x == lo || x == hi) return Re(0.5);
  return Re(0);
}

// ---------------------------------------------------------------------------
// Macroscopic moments.
// ---------------------------------------------------------------------------
template <class Re>
__host__ __device__ __forceinline__ Re density(const Re f[Q]) {
  Re r = f[0];
#pragma unroll
  for (int i = 1; i < Q; ++i) r += f[i];
  return r;
}

template <class Re>
__host__ __device__ __forceinline__ void momentum(const Re f[Q], Re& jx, Re& jy, Re& jz) {
  jx = (f[1] - f[2]) + (f[7] - f[8]) + (f[9] - f[10]) + (f[11] - f[12]) + (f[13] - f[14]);
  jy = (f[3] - f[4]) + (f[7] + f[8]) - (f[9] + f[10]) + (f[15] - f[16]) + (f[17] - f[18]);
  jz = (f[5] - f[6]) + (f[11] + f[12]) - (f[13] + f[14]) + (f[15] + f[16]) - (f[17] + f[18]);
}

// e_i . u for direction i (compile-time i).
template <class Re>
__host__ __device__ __forceinline__ Re edotu(int i, Re ux, Re uy, Re uz) {
  Re s = Re(0);
  if (ex(i) == 1) s += ux;
  if (ex(i) == -1) s -= ux;
  if (ey(i) == 1) s += uy;
  if (ey(i) == -1) s -= uy;
  if (ez(i) == 1) s += uz;
  if (ez(i) == -1) s -= uz;
  return s;
}

// f_eq_i = w_i rho (1 + 3 eu + 4.5 eu^2 - 1.5 u^2)   (equilibrium.py:144-149)
template <class Re, class W>
__host__ __device__ __forceinline__ void equilibrium(Re rho, Re ux, Re uy, Re uz, const W& w,
                                            Re feq[Q]) {
  const Re usq = ux * ux + uy * uy + uz * uz;
  const Re base = Re(1) - Re(1.5) * usq;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const Re eu = edotu<Re>(i, ux, uy, uz);
    feq[i] = Re(w[i]) * rho * (base + eu * (Re(3) + Re(4.5) * eu));
  }
}

// Cotangent v on f_eq(rho, u) -> (g_rho, g_u) at fixed (rho, u).
template <class Re, class W>
__host__ __device__ __forceinline__ void equilibrium_vjp(const Re v[Q], Re rho, Re ux, Re uy, Re uz,
                                                const W& w, Re& grho, Re& gx, Re& gy,
                                                Re& gz) {
  const Re usq = ux * ux + uy * uy + uz * uz;
  const Re base = Re(1) - Re(1.5) * usq;
  Re sp = 0, sw = 0, ax = 0, ay = 0, az = 0;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const Re eu = edotu<Re>(i, ux, uy, uz);
    const Re vw = v[i] * Re(w[i]);
    sp += vw * (base + eu * (Re(3) + Re(4.5) * eu));
    sw += vw;
    const Re t = vw * (Re(1) + Re(3) * eu);
    if (ex(i) == 1) ax += t;
    if (ex(i) == -1) ax -= t;
    if (ey(i) == 1) ay += t;
    if (ey(i) == -1) ay -= t;
    if (ez(i) == 1) az += t;
    if (ez(i) == -1) az -= t;
  }
  grho = sp;
  gx = Re(3) * rho * (ax - ux * sw);
  gy = Re(3) * rho * (ay - uy * sw);
  gz = Re(3) * rho * (az - uz * sw);
}

// Chain (g_rho, g_u) through rho = sum f, u = j / rho onto g_f (accumulates).
template <class Re>
__host__ __device__ __forceinline__ void macro_vjp_add(Re grho, Re gx, Re gy, Re gz, Re rho, Re ux,
                                              Re uy, Re uz, Re gf[Q]) {
  const Re ir = lbm_rcp(rho);
  const Re hx = gx * ir, hy = gy * ir, hz = gz * ir;
  const Re c0 = grho - (hx * ux + hy * uy + hz * uz);
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    Re s = c0;
    if (ex(i) == 1) s += hx;
    if (ex(i) == -1) s -= hx;
    if (ey(i) == 1) s += hy;
    if (ey(i) == -1) s -= hy;
    if (ez(i) == 1) s += hz;
    if (ez(i) == -1) s -= hz;
    gf[i] += s;
  }
}

// ---------------------------------------------------------------------------
// MRT transforms.  m = M f with shared partial sums; the back transform applies
// f_i -= sum_k M[k][i] d_k for the 15 non-conserved moments.
// ---------------------------------------------------------------------------
template <class Re>
__host__ __device__ __forceinline__ void mrt_moments(const Re f[Q], Re m[Q]) {
  const Re a1 = f[1] + f[2], d1 = f[1] - f[2];
  const Re a3 = f[3] + f[4], d3 = f[3] - f[4];
  const Re a5 = f[5] + f[6], d5 = f[5] - f[6];
  const Re pxy = f[7] + f[10], qxy = f[8] + f[9];
  const Re pxz = f[11] + f[14], qxz = f[12] + f[13];
  const Re pyz = f[15] + f[18], qyz = f[16] + f[17];
  const Re sxy = pxy + qxy, sxz = pxz + qxz, syz = pyz + qyz;
  const Re u1 = f[7] - f[10], u2 = f[9] - f[8];
  const Re v1 = f[11] - f[14], v2 = f[13] - f[12];
  const Re w1 = f[15] - f[18], w2 = f[17] - f[16];
  const Re jx_xy = u1 + u2, jy_xy = u1 - u2;
  const Re jx_xz = v1 + v2, jz_xz = v1 - v2;
  const Re jy_yz = w1 + w2, jz_yz = w1 - w2;
  const Re sf = a1 + a3 + a5;
  const Re se = sxy + sxz + syz;
  m[0] = f[0] + sf + se;
  m[1] = Re(-30) * f[0] - Re(11) * sf + Re(8) * se;
  m[2] = Re(12) * f[0] - Re(4) * sf + se;
  m[3] = d1 + jx_xy + jx_xz;
  m[4] = Re(-4) * d1 + jx_xy + jx_xz;
  m[5] = d3 + jy_xy + jy_yz;
  m[6] = Re(-4) * d3 + jy_xy + jy_yz;
  m[7] = d5 + jz_xz + jz_yz;
  m[8] = Re(-4) * d5 + jz_xz + jz_yz;
  const Re t9 = sxy + sxz - Re(2) * syz;
  m[9] = Re(2) * a1 - a3 - a5 + t9;
  m[10] = Re(-4) * a1 + Re(2) * (a3 + a5) + t9;
  const Re t11 = sxy - sxz;
  m[11] = a3 - a5 + t11;
  m[12] = Re(-2) * (a3 - a5) + t11;
  m[13] = pxy - qxy;
  m[14] = pyz - qyz;
  m[15] = pxz - qxz;
  m[16] = jx_xy - jx_xz;
  m[17] = jy_yz - jy_xy;
  m[18] = jz_xz - jz_yz;
}

// out_i = in_i - sum_{k non-conserved} M[k][i] d_k (out may alias in)
template <class Re, class Out>
__host__ __device__ __forceinline__ void mrt_back(const Re d[Q], const Re in[Q], Out out) {
  const Re cf = Re(-11) * d[1] - Re(4) * d[2];
  const Re ce = Re(8) * d[1] + d[2];
  const Re fx = Re(2) * d[9] - Re(4) * d[10];
  const Re fy = -d[9] + Re(2) * d[10] + d[11] - Re(2) * d[12];
  const Re fz = -d[9] + Re(2) * d[10] - d[11] + Re(2) * d[12];
  const Re exy = ce + d[9] + d[10] + d[11] + d[12];
  const Re exz = ce + d[9] + d[10] - d[11] - d[12];
  const Re eyz = ce - Re(2) * (d[9] + d[10]);
  emit(out, 0, in[0] - (Re(-30) * d[1] + Re(12) * d[2]));
  emit(out, 1, in[1] - (cf + fx - Re(4) * d[4]));
  emit(out, 2, in[2] - (cf + fx + Re(4) * d[4]));
  emit(out, 3, in[3] - (cf + fy - Re(4) * d[6]));
  emit(out, 4, in[4] - (cf + fy + Re(4) * d[6]));
  emit(out, 5, in[5] - (cf + fz - Re(4) * d[8]));
  emit(out, 6, in[6] - (cf + fz + Re(4) * d[8]));
  // xy edges: rows 4, 6, 13, 16, 17
  const Re a46p = d[4] + d[6], a46m = d[4] - d[6];
  const Re b1617p = d[16] + d[17], b1617m = d[16] - d[17];
  emit(out, 7, in[7] - (exy + a46p + d[13] + b1617m));
  emit(out, 8, in[8] - (exy - a46m - d[13] - b1617p));
  emit(out, 9, in[9] - (exy + a46m - d[13] + b1617p));
  emit(out, 10, in[10] - (exy - a46p + d[13] - b1617m));
  // xz edges: rows 4, 8, 15, 16, 18
  const Re a48p = d[4] + d[8], a48m = d[4] - d[8];
  const Re b1618p = d[16] + d[18], b1618m = d[16] - d[18];
  emit(out, 11, in[11] - (exz + a48p + d[15] - b1618m));
  emit(out, 12, in[12] - (exz - a48m - d[15] + b1618p));
  emit(out, 13, in[13] - (exz + a48m - d[15] - b1618p));
  emit(out, 14, in[14] - (exz - a48p + d[15] + b1618m));
  // yz edges: rows 6, 8, 14, 17, 18
  const Re a68p = d[6] + d[8], a68m = d[6] - d[8];
  const Re b1718p = d[17] + d[18], b1718m = d[17] - d[18];
  emit(out, 15, in[15] - (eyz + a68p + d[14] + b1718m));
  emit(out, 16, in[16] - (eyz - a68m - d[14] - b1718p));
  emit(out, 17, in[17] - (eyz + a68m - d[14] + b1718p));
  emit(out, 18, in[18] - (eyz - a68p + d[14] - b1718m));
}

// Equilibrium moments (lattice.py:342-391) for the non-conserved rows.
template <class Re>
__host__ __device__ __forceinline__ void mrt_meq(Re rho, Re ux, Re uy, Re uz, Re meq[Q]) {
  const Re u2 = ux * ux + uy * uy + uz * uz;
  const Re pxx = Re(2) * ux * ux - uy * uy - uz * uz;
  const Re pww = uy * uy - uz * uz;
  meq[0] = rho;
  meq[1] = rho * (Re(-11) + Re(19) * u2);
  meq[2] = rho * (Re(3) - Re(5.5) * u2);
  meq[3] = rho * ux;
  meq[4] = Re(-2.0 / 3.0) * rho * ux;
  meq[5] = rho * uy;
  meq[6] = Re(-2.0 / 3.0) * rho * uy;
  meq[7] = rho * uz;
  meq[8] = Re(-2.0 / 3.0) * rho * uz;
  meq[9] = rho * pxx;
  meq[10] = Re(-0.5) * rho * pxx;
  meq[11] = rho * pww;
  meq[12] = Re(-0.5) * rho * pww;
  meq[13] = rho * ux * uy;
  meq[14] = rho * uy * uz;
  meq[15] = rho * ux * uz;
  meq[16] = Re(0);
  meq[17] = Re(0);
  meq[18] = Re(0);
}

// ---------------------------------------------------------------------------
// Smagorinsky: tau_eff = (tau + sqrt(tau^2 + c Pi / (rho + 1e-10))) / 2 with
// c = 18 Cs^2 and Pi the Frobenius norm of the non-equilibrium stress
// Pi_ab = sum_i e_ia e_ib (f_i - feq_i) (collision.py:187-270).  The
// equilibrium part is evaluated in closed form, sum_i e_ia e_ib feq_i =
// rho/3 delta_ab + rho u_a u_b, from the raw second moments of f.
// ---------------------------------------------------------------------------
template <class Re>
__host__ __device__ __forceinline__ void raw_second_moments(const Re f[Q], Re p[6]) {
  const Re a1 = f[1] + f[2], a3 = f[3] + f[4], a5 = f[5] + f[6];
  const Re sxy = (f[7] + f[10]) + (f[8] + f[9]);
  const Re sxz = (f[11] + f[14]) + (f[12] + f[13]);
  const Re syz = (f[15] + f[18]) + (f[16] + f[17]);
  p[0] = a1 + sxy + sxz;                       // sum ex^2 f
  p[1] = a3 + sxy + syz;                       // sum ey^2 f
  p[2] = a5 + sxz + syz;                       // sum ez^2 f
  p[3] = (f[7] + f[10]) - (f[8] + f[9]);       // sum ex ey f
  p[4] = (f[11] + f[14]) - (f[12] + f[13]);    // sum ex ez f
  p[5] = (f[15] + f[18]) - (f[16] + f[17]);    // sum ey ez f
}

// Second moments of f_eq in closed form, exact for any symmetric weight set:
// sum_i e_ia e_ib feq_i = rho [W2 (1 - 1.5 u^2) + 4.5 (W2 u_a^2 + W22 (u^2 - u_a^2))] (a = b)
//                       = 9 W22 rho u_a u_b                                    (a != b)
// with W2 = sum_i w_i e_ix^2 = 2 w_face + 8 w_edge and W22 = sum_i w_i e_ix^2 e_iy^2
// = 4 w_edge (1/3 and 1/9 for the rational weights; the float32-rounded
// weights of lattice.py:53-60 shift them by ~1e-8, which this form keeps).
template <class Re, class W>
__host__ __device__ __forceinline__ void eq_second(const W& w, Re rho, Re ux, Re uy, Re uz,
                                                   Re e[6]) {
  using Sc = typename ScalarOf<Re>::type;
  const Re W2 = Re(Sc(2) * Sc(w[1]) + Sc(8) * Sc(w[7])), W22 = Re(Sc(4) * Sc(w[7]));
  const Re xx = ux * ux, yy = uy * uy, zz = uz * uz;
  const Re base = W2 * (Re(1) - Re(1.5) * (xx + yy + zz));
  e[0] = rho * (base + Re(4.5) * (W2 * xx + W22 * (yy + zz)));
  e[1] = rho * (base + Re(4.5) * (W2 * yy + W22 * (xx + zz)));
  e[2] = rho * (base + Re(4.5) * (W2 * zz + W22 * (xx + yy)));
  const Re c9 = Re(9) * W22 * rho;
  e[3] = c9 * ux * uy;
  e[4] = c9 * ux * uz;
  e[5] = c9 * uy * uz;
}

// Cotangent ge on eq_second -> (g_rho, g_u).
template <class Re, class W>
__host__ __device__ __forceinline__ void eq_second_vjp(const W& w, Re rho, Re ux, Re uy,
                                                       Re uz, const Re ge[6], Re& gr, Re& gx,
                                                       Re& gy, Re& gz) {
  using Sc = typename ScalarOf<Re>::type;
  const Re W2 = Re(Sc(2) * Sc(w[1]) + Sc(8) * Sc(w[7])), W22 = Re(Sc(4) * Sc(w[7]));
  const Re xx = ux * ux, yy = uy * uy, zz = uz * uz;
  const Re base = W2 * (Re(1) - Re(1.5) * (xx + yy + zz));
  const Re c9 = Re(9) * W22;
  gr = ge[0] * (base + Re(4.5) * (W2 * xx + W22 * (yy + zz))) +
       ge[1] * (base + Re(4.5) * (W2 * yy + W22 * (xx + zz))) +
       ge[2] * (base + Re(4.5) * (W2 * zz + W22 * (xx + yy))) +
       c9 * (ge[3] * ux * uy + ge[4] * ux * uz + ge[5] * uy * uz);
  const Re own = Re(6) * W2, oth = Re(9) * W22 - Re(3) * W2;
  gx = rho * (ux * (own * ge[0] + oth * (ge[1] + ge[2])) + c9 * (ge[3] * uy + ge[4] * uz));
  gy = rho * (uy * (own * ge[1] + oth * (ge[0] + ge[2])) + c9 * (ge[3] * ux + ge[5] * uz));
  gz = rho * (uz * (own * ge[2] + oth * (ge[0] + ge[1])) + c9 * (ge[4] * ux + ge[5] * uy));
}

// Non-equilibrium stress Pi_ab = sum_i e_ia e_ib f_i - sum_i e_ia e_ib feq_i.
template <class Re, class W>
__host__ __device__ __forceinline__ void neq_stress(const Re p[6], const W& w, Re rho, Re ux,
                                                    Re uy, Re uz, Re s[6]) {
  Re e[6];
  eq_second<Re>(w, rho, ux, uy, uz, e);
#pragma unroll
  for (int k = 0; k < 6; ++k) s[k] = p[k] - e[k];
}

template <class Re>
__host__ __device__ __forceinline__ Re smag_pi(const Re s[6]) {
  return lbm_sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2] +
                  Re(2) * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]));
}

// 1 / (rho + 1e-10): in float the epsilon is below half an ulp of any
// physical density, so the reciprocal of rho is reused.
template <class Re>
__host__ __device__ __forceinline__ Re inv_rho_eps(Re rho, Re inv_rho) {
  if (IsSingle<Re>::value) return inv_rho;
  return Re(1) / (rho + Re(1e-10));
}

template <class Re>
__host__ __device__ __forceinline__ Re smag_tau(Re tau, Re c18cs2, Re pi, Re inv_rr) {
  return Re(0.5) * (tau + lbm_sqrt(tau * tau + c18cs2 * pi * inv_rr));
}

// ---------------------------------------------------------------------------
// Collision forward.  ``omega`` = 1 / tau_eff.  BGK: f - omega (f - f_eq).
// MRT: f - M^-1 S (M f - m_eq), with S = rates and omega in the stress slots.
// ---------------------------------------------------------------------------
template <class Re, class W, class Out>
__host__ __device__ __forceinline__ void bgk_collide(const Re f[Q], Re rho, Re ux, Re uy, Re uz,
                                            Re omega, const W& w, Out out) {
  Re feq[Q];
  equilibrium<Re>(rho, ux, uy, uz, w, feq);
#pragma unroll
  for (int i = 0; i < Q; ++i) emit(out, i, Re(f[i] - omega * (f[i] - feq[i])));
}

template <class Re, class RT, class Out>
__host__ __device__ __forceinline__ void mrt_relax_back(const Re f[Q], const Re m[Q], Re rho,
                                                        Re ux, Re uy, Re uz, Re omega,
                                                        const RT& rate, Out out) {
  using Sc = typename ScalarOf<Re>::type;
  Re meq[Q], d[Q];
  mrt_meq<Re>(rho, ux, uy, uz, meq);
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    const Sc inv_norm = Sc(1.0 / double(mnorm(k)));
    // rows 16-18 have a zero equilibrium moment
    const Re dm = k >= 16 ? m[k] : m[k] - meq[k];
    if (is_conserved(k)) d[k] = Re(0);
    else if (is_stress(k)) d[k] = (omega * Re(inv_norm)) * dm;
    else d[k] = Re(Sc(rate[k]) * inv_norm) * dm;
  }
  mrt_back<Re>(d, f, out);
}

template <class Re, class RT, class Out>
__host__ __device__ __forceinline__ void mrt_collide(const Re f[Q], Re rho, Re ux, Re uy, Re uz,
                                            Re omega, const RT& rate, Out out) {
  Re m[Q];
  mrt_moments<Re>(f, m);
  mrt_relax_back<Re>(f, m, rho, ux, uy, uz, omega, rate, out);
}

// Full collide of one cell given its density and momentum: optional
// Smagorinsky tau, then BGK/MRT.  Returns omega actually used.
template <class Re, class KT, class Out>
__host__ __device__ __forceinline__ Re collide_cell_rj(const Re f[Q], Re rho, Re jx, Re jy, Re jz,
                                                       Re tau, bool mrt, bool smag, Re c18cs2,
                                                       const KT& K, Out out) {
  const Re ir = lbm_rcp(rho);
  const Re ux = jx * ir, uy = jy * ir, uz = jz * ir;
  Re omega;
  if (mrt) {
    Re m[Q];
    mrt_moments<Re>(f, m);
    if (smag) {
      // raw second moments from the MRT partial sums: sum ex^2 f = (m0 + ... )
      Re p[6], s[6];
      raw_second_moments<Re>(f, p);
      neq_stress<Re>(p, K.w, rho, ux, uy, uz, s);
      omega = lbm_rcp(smag_tau<Re>(tau, c18cs2, smag_pi<Re>(s), inv_rho_eps<Re>(rho, ir)));
    } else {
      omega = lbm_rcp(tau);
    }
    mrt_relax_back<Re>(f, m, rho, ux, uy, uz, omega, K.rate, out);
  } else {
    if (smag) {
      Re p[6], s[6];
      raw_second_moments<Re>(f, p);
      neq_stress<Re>(p, K.w, rho, ux, uy, uz, s);
      omega = lbm_rcp(smag_tau<Re>(tau, c18cs2, smag_pi<Re>(s), inv_rho_eps<Re>(rho, ir)));
    } else {
      omega = lbm_rcp(tau);
    }
    bgk_collide<Re>(f, rho, ux, uy, uz, omega, K.w, out);
  }
  return omega;
}

template <class Re, class KT, class Out>
__host__ __device__ __forceinline__ Re collide_cell(const Re f[Q], Re tau, bool mrt, bool smag,
                                                    Re c18cs2, const KT& K, Out out) {
  Re jx, jy, jz;
  momentum<Re>(f, jx, jy, jz);
  return collide_cell_rj<Re>(f, density<Re>(f), jx, jy, jz, tau, mrt, smag, c18cs2, K, out);
}

// g_i += c0 + e_i . h (+ sum_ab e_ia e_ib q_ab when Quad, q = xx, yy, zz, xy,
// xz, yz with the off-diagonal terms already doubled).  Opposite directions
// share the even part and take the odd part with opposite signs.
template <class Re, bool Quad>
__host__ __device__ __forceinline__ void cell_terms_add(Re g[Q], Re c0, Re hx, Re hy, Re hz,
                                                        const Re q[6]) {
  g[0] += c0;
  const Re ax = Quad ? Re(c0 + q[0]) : c0;
  const Re ay = Quad ? Re(c0 + q[1]) : c0;
  const Re az = Quad ? Re(c0 + q[2]) : c0;
  g[1] += ax + hx;
  g[2] += ax - hx;
  g[3] += ay + hy;
  g[4] += ay - hy;
  g[5] += az + hz;
  g[6] += az - hz;
  // xy edges: 7 (1,1,0), 10 (-1,-1,0), 9 (1,-1,0), 8 (-1,1,0)
  {
    const Re b = Quad ? Re(ax + q[1]) : c0;
    const Re p = Quad ? Re(b + q[3]) : c0, m = Quad ? Re(b - q[3]) : c0;
    const Re s = hx + hy, d = hx - hy;
    g[7] += p + s;
    g[10] += p - s;
    g[9] += m + d;
    g[8] += m - d;
  }
  // xz edges: 11 (1,0,1), 14 (-1,0,-1), 13 (1,0,-1), 12 (-1,0,1)
  {
    const Re b = Quad ? Re(ax + q[2]) : c0;
    const Re p = Quad ? Re(b + q[4]) : c0, m = Quad ? Re(b - q[4]) : c0;
    const Re s = hx + hz, d = hx - hz;
    g[11] += p + s;
    g[14] += p - s;
    g[13] += m + d;
    g[12] += m - d;
  }
  // yz edges: 15 (0,1,1), 18 (0,-1,-1), 17 (0,1,-1), 16 (0,-1,1)
  {
    const Re b = Quad ? Re(ay + q[2]) : c0;
    const Re p = Quad ? Re(b + q[5]) : c0, m = Quad ? Re(b - q[5]) : c0;
    const Re s = hy + hz, d = hy - hz;
    g[15] += p + s;
    g[18] += p - s;
    g[17] += m + d;
    g[16] += m - d;
  }
}

// ---------------------------------------------------------------------------
// Collision VJP.  The pre-collision populations enter only through a few
// per-cell scalars (rho, u and the raw second moments, which also give the
// MRT stress moments m9, m11, m13, m14, m15), so the VJP works on those and
// on the cotangent in place, keeping register pressure low.
//
// Smagorinsky: d Pi / d s is undefined at Pi = 0 (jax.grad yields NaN there);
// this implementation uses the subgradient 0.
// ---------------------------------------------------------------------------
template <class Re> struct CellScalars {
  Re rho, ux, uy, uz;
  Re p[6];   // sum e_a e_b f : xx, yy, zz, xy, xz, yz
};

template <class Re>
__host__ __device__ __forceinline__ void cell_scalars(const Re f[Q], CellScalars<Re>& c) {
  c.rho = density<Re>(f);
  Re jx, jy, jz;
  momentum<Re>(f, jx, jy, jz);
  const Re ir = lbm_rcp(c.rho);
  c.ux = jx * ir;
  c.uy = jy * ir;
  c.uz = jz * ir;
  raw_second_moments<Re>(f, c.p);
}

// g (in: cotangent on the collide output, out: cotangent on f).  ``f`` is
// only read for BGK when the omega cotangent is needed (Smagorinsky or a
// requested g_tau): sum_i lam_i (f_i - feq_i).
template <class Re, class KT>
__host__ __device__ __forceinline__ void collide_vjp_s(const CellScalars<Re>& cs, const Re* f,
                                                       Re g[Q], Re tau, bool mrt, bool smag,
                                                       Re c18cs2, const KT& K,
                                                       Re* g_tau_out) {
  const Re rho = cs.rho, ux = cs.ux, uy = cs.uy, uz = cs.uz;
  const Re ir = lbm_rcp(rho);
  Re sst[6];
  Re tau_eff = tau, pi = Re(0), R = Re(0), inv_rr = Re(0);
  if (smag) {
    neq_stress<Re>(cs.p, K.w, rho, ux, uy, uz, sst);
    pi = smag_pi<Re>(sst);
    inv_rr = inv_rho_eps<Re>(rho, ir);
    R = lbm_sqrt(tau * tau + c18cs2 * pi * inv_rr);
    tau_eff = Re(0.5) * (tau + R);
  }
  const Re omega = lbm_rcp(tau_eff);
  const bool want_omega = smag || g_tau_out != nullptr;
  Re g_omega = Re(0);
  Re grho = 0, gx = 0, gy = 0, gz = 0;
  if (mrt) {
    Re d[Q];
    {
      Re ml[Q];
      mrt_moments<Re>(g, ml);
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        const Re pk = ml[k] * Re(1.0 / double(mnorm(k)));
        d[k] = is_conserved(k) ? Re(0) : (is_stress(k) ? omega : K.rate[k]) * pk;
        if (want_omega && is_stress(k)) {
          // stress moments of f from the raw second moments
          Re mk;
          if (k == 9) mk = Re(2) * cs.p[0] - cs.p[1] - cs.p[2];
          else if (k == 11) mk = cs.p[1] - cs.p[2];
          else if (k == 13) mk = cs.p[3];
          else if (k == 14) mk = cs.p[5];
          else mk = cs.p[4];
          Re meqk;
          if (k == 9) meqk = rho * (Re(2) * ux * ux - uy * uy - uz * uz);
          else if (k == 11) meqk = rho * (uy * uy - uz * uz);
          else if (k == 13) meqk = rho * ux * uy;
          else if (k == 14) meqk = rho * uy * uz;
          else meqk = rho * ux * uz;
          g_omega -= pk * (mk - meqk);
        }
      }
    }
    mrt_back<Re>(d, g, g);   // g <- lam - M^T d (elementwise in place)
    const Re a9 = d[9] - Re(0.5) * d[10];
    const Re a11 = d[11] - Re(0.5) * d[12];
    const Re u2 = ux * ux + uy * uy + uz * uz;
    const Re pxx = Re(2) * ux * ux - uy * uy - uz * uz;
    const Re pww = uy * uy - uz * uz;
    grho = d[1] * (Re(-11) + Re(19) * u2) + d[2] * (Re(3) - Re(5.5) * u2) +
           Re(-2.0 / 3.0) * (d[4] * ux + d[6] * uy + d[8] * uz) + a9 * pxx + a11 * pww +
           d[13] * ux * uy + d[14] * uy * uz + d[15] * ux * uz;
    const Re q12 = Re(38) * d[1] - Re(11) * d[2];
    gx = rho * (q12 * ux + Re(-2.0 / 3.0) * d[4] + Re(4) * a9 * ux + d[13] * uy + d[15] * uz);
    gy = rho * (q12 * uy + Re(-2.0 / 3.0) * d[6] - Re(2) * a9 * uy + Re(2) * a11 * uy +
                d[13] * ux + d[14] * uz);
    gz = rho * (q12 * uz + Re(-2.0 / 3.0) * d[8] - Re(2) * a9 * uz - Re(2) * a11 * uz +
                d[14] * uy + d[15] * ux);
  } else {
    equilibrium_vjp<Re>(g, rho, ux, uy, uz, K.w, grho, gx, gy, gz);
    grho *= omega;
    gx *= omega;
    gy *= omega;
    gz *= omega;
    if (want_omega) {
      Re feq[Q];
      equilibrium<Re>(rho, ux, uy, uz, K.w, feq);
#pragma unroll
      for (int i = 0; i < Q; ++i) g_omega -= g[i] * (f[i] - feq[i]);
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) g[i] *= (Re(1) - omega);
  }
  // omega = 1 / tau_eff
  const Re g_tau_eff = -g_omega * omega * omega;
  Re g_tau = g_tau_eff;
  Re gs[6];
  bool quad = false;
  if (smag) {
    // tau_eff = (tau + R)/2, R = sqrt(tau^2 + c pi inv_rr)
    const Re gR = Re(0.5) * g_tau_eff;
    const Re gX = div_if_pos(gR, Re(2) * R);
    g_tau = Re(0.5) * g_tau_eff + gX * Re(2) * tau;
    const Re g_pi = gX * c18cs2 * inv_rr;
    // d(inv_rr)/d rho, the same for every population
    grho += -gX * c18cs2 * pi * inv_rr * inv_rr;
    if (any_pos(pi)) {
      const Re ip = div_if_pos(g_pi, pi);
      gs[0] = ip * sst[0];
      gs[1] = ip * sst[1];
      gs[2] = ip * sst[2];
      gs[3] = Re(2) * ip * sst[3];
      gs[4] = Re(2) * ip * sst[4];
      gs[5] = Re(2) * ip * sst[5];
      // s = p(f) - eq(rho, u): the equilibrium part goes through rho and u,
      // the raw moments p add e_ia e_ib gs_ab per population (below)
      Re er, exx, eyy, ezz;
      eq_second_vjp<Re>(K.w, rho, ux, uy, uz, gs, er, exx, eyy, ezz);
      grho -= er;
      gx -= exx;
      gy -= eyy;
      gz -= ezz;
      quad = true;
    }
  }
  // rho = sum f, u = sum e f / rho: g_i += grho + (e_i - u) . g_u / rho
  const Re hx = gx * ir, hy = gy * ir, hz = gz * ir;
  const Re c0 = grho - (hx * ux + hy * uy + hz * uz);
  if (quad) cell_terms_add<Re, true>(g, c0, hx, hy, hz, gs);
  else cell_terms_add<Re, false>(g, c0, hx, hy, hz, gs);
  if (g_tau_out) *g_tau_out = g_tau;
}

// Convenience form: gf = (d collide / d f)^T lam.
template <class Re, class KT>
__host__ __device__ __forceinline__ void collide_vjp(const Re f[Q], const Re lam[Q], Re tau,
                                                     bool mrt, bool smag, Re c18cs2,
                                                     const KT& K, Re gf[Q],
                                                     Re* g_tau_out) {
  CellScalars<Re> cs;
  cell_scalars<Re>(f, cs);
#pragma unroll
  for (int i = 0; i < Q; ++i) gf[i] = lam[i];
  collide_vjp_s<Re>(cs, f, gf, tau, mrt, smag, c18cs2, K, g_tau_out);
}

}  // namespace lbm
