// Two FP32 lanes per thread on Blackwell's packed FP32x2 pipe.
//
// V2 holds the same quantity for two neighbouring cells; +, -, * map to the
// sm_100+ packed instructions (FADD2 / FMUL2 / FFMA2 via __fadd2_rn,
// __fmul2_rn, __ffma2_rn), so the per-cell collision math issues about half
// the FP instructions when a thread owns two cells.  A product is kept lazy
// (V2Prod) until it meets an addition, which then becomes one FFMA2.
#pragma once

#include "lbm_core.cuh"

namespace lbm {

struct V2 {
  float2 v;
  __device__ __forceinline__ V2() {}
  __device__ __forceinline__ V2(float2 a) : v(a) {}
  __device__ __forceinline__ V2(float a, float b) : v(make_float2(a, b)) {}
  __device__ __forceinline__ V2(double c) : v(make_float2(float(c), float(c))) {}
  __device__ __forceinline__ V2(float c) : v(make_float2(c, c)) {}
  __device__ __forceinline__ V2(int c) : v(make_float2(float(c), float(c))) {}
  __device__ __forceinline__ float x() const { return v.x; }
  __device__ __forceinline__ float y() const { return v.y; }
};

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

struct V2Prod {
  float2 a, b;
  __device__ __forceinline__ operator V2() const { return V2(__fmul2_rn(a, b)); }
};

__device__ __forceinline__ V2Prod operator*(V2 a, V2 b) { return V2Prod{a.v, b.v}; }
__device__ __forceinline__ V2Prod operator*(V2Prod p, V2 b) { return V2Prod{V2(p).v, b.v}; }
__device__ __forceinline__ V2Prod operator*(V2 a, V2Prod p) { return V2Prod{a.v, V2(p).v}; }
__device__ __forceinline__ V2Prod operator*(V2Prod p, V2Prod q) { return V2Prod{V2(p).v, V2(q).v}; }

__device__ __forceinline__ V2 operator+(V2 a, V2 b) { return V2(__fadd2_rn(a.v, b.v)); }
// a - b in one packed subtract (PTX sub.rn.f32x2, sm_100 and later)
__device__ __forceinline__ V2 operator-(V2 a, V2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;"
      : "=l"(r)
      : "l"(*reinterpret_cast<const unsigned long long*>(&a.v)),
        "l"(*reinterpret_cast<const unsigned long long*>(&b.v)));
  return V2(*reinterpret_cast<const float2*>(&r));
}
__device__ __forceinline__ V2 operator-(V2 a) { return V2(neg2(a.v)); }

__device__ __forceinline__ V2 operator+(V2Prod p, V2 c) { return V2(__ffma2_rn(p.a, p.b, c.v)); }
__device__ __forceinline__ V2 operator+(V2 c, V2Prod p) { return V2(__ffma2_rn(p.a, p.b, c.v)); }
__device__ __forceinline__ V2 operator-(V2 c, V2Prod p) { return V2(__ffma2_rn(neg2(p.a), p.b, c.v)); }
__device__ __forceinline__ V2 operator-(V2Prod p, V2 c) { return V2(__ffma2_rn(p.a, p.b, neg2(c.v))); }
__device__ __forceinline__ V2 operator+(V2Prod p, V2Prod q) { return V2(__ffma2_rn(q.a, q.b, V2(p).v)); }
__device__ __forceinline__ V2 operator-(V2Prod p, V2Prod q) {
  return V2(__ffma2_rn(neg2(q.a), q.b, V2(p).v));
}
__device__ __forceinline__ V2 operator-(V2Prod p) { return V2(__fmul2_rn(neg2(p.a), p.b)); }

__device__ __forceinline__ V2 operator/(V2 a, V2 b) { return V2(a.v.x / b.v.x, a.v.y / b.v.y); }
__device__ __forceinline__ V2 operator/(V2Prod a, V2 b) { return V2(a) / b; }

__device__ __forceinline__ V2& operator+=(V2& a, V2 b) { a = a + b; return a; }
__device__ __forceinline__ V2& operator+=(V2& a, V2Prod p) { a = a + p; return a; }
__device__ __forceinline__ V2& operator-=(V2& a, V2 b) { a = a - b; return a; }
__device__ __forceinline__ V2& operator-=(V2& a, V2Prod p) { a = a - p; return a; }
__device__ __forceinline__ V2& operator*=(V2& a, V2 b) { a = V2(a * b); return a; }

__device__ __forceinline__ V2 lbm_sqrt(V2 a) { return V2(lbm_sqrt(a.v.x), lbm_sqrt(a.v.y)); }
__device__ __forceinline__ V2 lbm_rcp(V2 a) { return V2(lbm_rcp(a.v.x), lbm_rcp(a.v.y)); }
__device__ __forceinline__ V2 div_if_pos(V2 a, V2 b) {
  return V2(div_if_pos(a.v.x, b.v.x), div_if_pos(a.v.y, b.v.y));
}
__device__ __forceinline__ bool any_pos(V2 v) { return v.v.x > 0.0f || v.v.y > 0.0f; }

template <> struct ScalarOf<V2> { using type = float; };

// Populations of two z-adjacent cells (z even, z + 1) in the storage type.
// ld2/st2 move the aligned pair at p (p even) as one 8-byte (FP32) or 4-byte
// (FP16/BF16) access; ld2s gathers two separate elements.  16-bit storage
// holds f minus a per-direction offset w (one value per lane), as Storage<>
// does.
template <class St> struct Pair;
template <> struct Pair<float> {
  static __device__ __forceinline__ V2 ld2(const float* p, V2) {
    return V2(ldg_s(reinterpret_cast<const float2*>(p)));
  }
  static __device__ __forceinline__ V2 ld2s(const float* p0, const float* p1, V2) {
    return V2(ldg_s(p0), ldg_s(p1));
  }
  static __device__ __forceinline__ void st2(float* p, V2 v, V2) {
    *reinterpret_cast<float2*>(p) = v.v;
  }
};
// float(h) + c for a 16-bit h in one mixed-precision add (sm_100+); the
// conversion is exact, so this rounds as convert-then-add does.  (Measured
// 98 us against 104 us per bf16 step at 256x128x128, 91.1 us against 92.1 us
// per fp16 step.)
__device__ __forceinline__ float add_f16(__half h, float c) {
  float d;
  asm("add.rn.f32.f16 %0, %1, %2;" : "=f"(d) : "h"(__half_as_ushort(h)), "f"(c));
  return d;
}
__device__ __forceinline__ float add_bf16(__nv_bfloat16 h, float c) {
  float d;
  asm("add.rn.f32.bf16 %0, %1, %2;" : "=f"(d) : "h"(__bfloat16_as_ushort(h)), "f"(c));
  return d;
}

template <> struct Pair<__half> {
  static __device__ __forceinline__ V2 ld2(const __half* p, V2 w) {
    const __half2 v = ldg_s(reinterpret_cast<const __half2*>(p));
    return V2(add_f16(__low2half(v), w.x()), add_f16(__high2half(v), w.y()));
  }
  static __device__ __forceinline__ V2 ld2s(const __half* p0, const __half* p1, V2 w) {
    return V2(add_f16(ldg_s(p0), w.x()), add_f16(ldg_s(p1), w.y()));
  }
  static __device__ __forceinline__ void st2(__half* p, V2 v, V2 w) {
    *reinterpret_cast<__half2*>(p) = __float22half2_rn((v - w).v);
  }
};
template <> struct Pair<__nv_bfloat16> {
  static __device__ __forceinline__ V2 ld2(const __nv_bfloat16* p, V2 w) {
    const __nv_bfloat162 v = ldg_s(reinterpret_cast<const __nv_bfloat162*>(p));
    return V2(add_bf16(__low2bfloat16(v), w.x()), add_bf16(__high2bfloat16(v), w.y()));
  }
  static __device__ __forceinline__ V2 ld2s(const __nv_bfloat16* p0, const __nv_bfloat16* p1,
                                            V2 w) {
    return V2(add_bf16(ldg_s(p0), w.x()), add_bf16(ldg_s(p1), w.y()));
  }
  static __device__ __forceinline__ void st2(__nv_bfloat16* p, V2 v, V2 w) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __float22bfloat162_rn((v - w).v);
  }
};

}  // namespace lbm
