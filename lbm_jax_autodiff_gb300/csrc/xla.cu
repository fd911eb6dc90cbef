// XLA custom-call targets (legacy api_version = 0 on CUDA):
//   void target(cudaStream_t stream, void** buffers, const char* opaque, size_t opaque_len)
// buffers = operands then results; `opaque` is an lbm_xla_desc.  These wrap
// the per-op entry points so jax.ffi can call the kernels from inside a
// jitted function (jax_lbm's operator API is its set of pure jnp functions,
// jax_lbm/__init__.py:23-60).  The legacy API has no status channel: a failed
// call prints lbm_last_error() to stderr and fills every result buffer with
// NaN (all-ones bytes), so a jitted program that reads them sees NaN instead
// of uninitialised memory.  A descriptor that cannot be parsed leaves the
// results unwritten (their sizes are unknown).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>

#include "../../include/lbm_gb300.h"

namespace {

// The descriptor is either the raw lbm_xla_desc bytes or, for hosts that pass
// backend_config as text, "lbm1 nx ny nz dtype flags periodic_yz tau_field
// u_face has_rho_target tau cs u0 u1 u2 rho" with the doubles in C99 hex
// ("%a", Python float.hex()) so they round-trip exactly.
bool read_desc(const char* opaque, size_t len, lbm_xla_desc& d) {
  std::memset(&d, 0, sizeof(d));
  if (opaque && len >= 5 && std::strncmp(opaque, "lbm1 ", 5) == 0) {
    char buf[512];
    const size_t n = len < sizeof(buf) - 1 ? len : sizeof(buf) - 1;
    std::memcpy(buf, opaque, n);
    buf[n] = 0;
    char* p = buf + 5;
    long iv[9];
    for (int k = 0; k < 9; ++k) iv[k] = std::strtol(p, &p, 10);
    double dv[6];
    for (int k = 0; k < 6; ++k) dv[k] = std::strtod(p, &p);
    d.nx = int32_t(iv[0]); d.ny = int32_t(iv[1]); d.nz = int32_t(iv[2]);
    d.dtype = int32_t(iv[3]); d.flags = int32_t(iv[4]); d.periodic_yz = int32_t(iv[5]);
    d.tau_field = int32_t(iv[6]); d.u_face = int32_t(iv[7]); d.has_rho_target = int32_t(iv[8]);
    d.tau = dv[0]; d.cs = dv[1]; d.u[0] = dv[2]; d.u[1] = dv[3]; d.u[2] = dv[4]; d.rho = dv[5];
    return true;
  }
  if (!opaque || len != sizeof(lbm_xla_desc)) {
    std::fprintf(stderr, "lbm_gb300: bad custom-call descriptor (%zu bytes, want %zu)\n", len,
                 sizeof(lbm_xla_desc));
    return false;
  }
  std::memcpy(&d, opaque, sizeof(d));
  return true;
}

// One result buffer of a target: device pointer and size in bytes.
struct Res {
  void* p;
  size_t bytes;
};

size_t elem(const lbm_xla_desc& d) { return d.dtype == LBM_F64 ? 8 : 4; }
size_t cells(const lbm_xla_desc& d) { return size_t(d.nx) * size_t(d.ny) * size_t(d.nz); }
size_t face(const lbm_xla_desc& d) { return size_t(d.ny) * size_t(d.nz); }

// On failure: message to stderr, every result buffer set to NaN on `stream`.
// The sizes come from the descriptor, so the fill runs only for dimensions
// the entry points accept (each >= 1, 19 * cells < 2^31) and element types
// they accept (LBM_F32 / LBM_F64): a call that failed on either writes nothing.
void report(const char* name, int rc, const lbm_xla_desc& d, void* stream,
            std::initializer_list<Res> results) {
  if (rc == LBM_OK) return;
  std::fprintf(stderr, "lbm_gb300: %s failed: %s\n", name, lbm_last_error());
  if (d.nx < 1 || d.ny < 1 || d.nz < 1 || 19 * cells(d) >= (size_t(1) << 31)) return;
  if (d.dtype != LBM_F32 && d.dtype != LBM_F64) return;
  for (const Res& r : results)
    if (r.p && r.bytes)
      cudaMemsetAsync(r.p, 0xFF, r.bytes, static_cast<cudaStream_t>(stream));
}

}  // namespace

extern "C" {

void lbm_xla_compute_density(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("compute_density", lbm_compute_density(d.dtype, b[0], b[1], d.nx, d.ny, d.nz, stream),
         d, stream, {{b[1], cells(d) * elem(d)}});
}

void lbm_xla_compute_velocity(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("compute_velocity",
         lbm_compute_velocity(d.dtype, b[0], b[1], b[2], d.nx, d.ny, d.nz, stream),
         d, stream, {{b[2], 3 * cells(d) * elem(d)}});
}

void lbm_xla_equilibrium(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("equilibrium", lbm_equilibrium(d.dtype, b[0], b[1], b[2], d.nx, d.ny, d.nz, d.flags,
                                        stream),
         d, stream, {{b[2], 19 * cells(d) * elem(d)}});
}

// operands: f [, tau_field when d.tau_field]; result: out
void lbm_xla_bgk(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  const void* tf = d.tau_field ? b[1] : nullptr;
  void* out = d.tau_field ? b[2] : b[1];
  report("bgk", lbm_bgk(d.dtype, b[0], tf, d.tau, out, d.nx, d.ny, d.nz, d.flags, stream),
         d, stream, {{out, 19 * cells(d) * elem(d)}});
}

void lbm_xla_mrt(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  const void* tf = d.tau_field ? b[1] : nullptr;
  void* out = d.tau_field ? b[2] : b[1];
  report("mrt", lbm_mrt(d.dtype, b[0], tf, d.tau, out, d.nx, d.ny, d.nz, d.flags, stream),
         d, stream, {{out, 19 * cells(d) * elem(d)}});
}

void lbm_xla_smagorinsky_tau(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("smagorinsky_tau", lbm_smagorinsky_tau(d.dtype, b[0], d.tau, d.cs, b[1], d.nx, d.ny,
                                                d.nz, d.flags, stream),
         d, stream, {{b[1], cells(d) * elem(d)}});
}

void lbm_xla_soft_bounce_back(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("soft_bounce_back",
         lbm_soft_bounce_back(d.dtype, b[0], b[1], b[2], d.nx, d.ny, d.nz, stream),
         d, stream, {{b[2], 19 * cells(d) * elem(d)}});
}

void lbm_xla_stream(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("stream", lbm_stream(d.dtype, b[0], b[1], d.periodic_yz, b[2], d.nx, d.ny, d.nz, stream),
         d, stream, {{b[2], 19 * cells(d) * elem(d)}});
}

// operands: f [, u_face when d.u_face]; result: out
void lbm_xla_zou_he_inlet(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  const void* uf = d.u_face ? b[1] : nullptr;
  void* out = d.u_face ? b[2] : b[1];
  report("zou_he_inlet", lbm_zou_he_inlet(d.dtype, b[0], uf, d.u, d.has_rho_target, d.rho,
                                          out, d.nx, d.ny, d.nz, stream),
         d, stream, {{out, 19 * cells(d) * elem(d)}});
}

void lbm_xla_zou_he_outlet(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("zou_he_outlet",
         lbm_zou_he_outlet(d.dtype, b[0], d.rho, b[1], d.nx, d.ny, d.nz, stream),
         d, stream, {{b[1], 19 * cells(d) * elem(d)}});
}

// operands: f_post, f_streamed, q; result: force f64[3]
void lbm_xla_momentum_exchange(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("momentum_exchange", lbm_momentum_exchange(d.dtype, b[0], b[1], b[2],
                                                    static_cast<double*>(b[3]), d.nx, d.ny,
                                                    d.nz, stream),
         d, stream, {{b[3], 3 * sizeof(double)}});
}

// ---- VJPs (operands: primal inputs, cotangent; results: input cotangents) ----

void lbm_xla_compute_density_vjp(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("compute_density_vjp",
         lbm_compute_density_vjp(d.dtype, b[0], b[1], d.nx, d.ny, d.nz, stream),
         d, stream, {{b[1], 19 * cells(d) * elem(d)}});
}

// operands: f, rho, g_u; results: g_f, g_rho
void lbm_xla_compute_velocity_vjp(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("compute_velocity_vjp", lbm_compute_velocity_vjp(d.dtype, b[0], b[1], b[2], b[3], b[4],
                                                          d.nx, d.ny, d.nz, stream),
         d, stream, {{b[3], 19 * cells(d) * elem(d)}, {b[4], cells(d) * elem(d)}});
}

// operands: rho, u, g_feq; results: g_rho, g_u
void lbm_xla_equilibrium_vjp(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("equilibrium_vjp", lbm_equilibrium_vjp(d.dtype, b[0], b[1], b[2], b[3], b[4], d.nx, d.ny,
                                                d.nz, d.flags, stream),
         d, stream, {{b[3], cells(d) * elem(d)}, {b[4], 3 * cells(d) * elem(d)}});
}

// operands: f [, tau_field], g; results: g_f, g_tau (per cell)
static void collide_vjp_xla(int mrt, void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  const int k = d.tau_field ? 1 : 0;
  const void* tf = d.tau_field ? b[1] : nullptr;
  auto fn = mrt ? lbm_mrt_vjp : lbm_bgk_vjp;
  report(mrt ? "mrt_vjp" : "bgk_vjp", fn(d.dtype, b[0], tf, d.tau, b[1 + k], b[2 + k], b[3 + k],
                                         d.nx, d.ny, d.nz, d.flags, stream),
         d, stream, {{b[2 + k], 19 * cells(d) * elem(d)}, {b[3 + k], cells(d) * elem(d)}});
}
void lbm_xla_bgk_vjp(void* s, void** b, const char* o, size_t l) { collide_vjp_xla(0, s, b, o, l); }
void lbm_xla_mrt_vjp(void* s, void** b, const char* o, size_t l) { collide_vjp_xla(1, s, b, o, l); }

// operands: f, g_tau_eff; results: g_f, g_tau (per cell)
void lbm_xla_smagorinsky_tau_vjp(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("smagorinsky_tau_vjp", lbm_smagorinsky_tau_vjp(d.dtype, b[0], d.tau, d.cs, b[1], b[2],
                                                        b[3], d.nx, d.ny, d.nz, d.flags, stream),
         d, stream, {{b[2], 19 * cells(d) * elem(d)}, {b[3], cells(d) * elem(d)}});
}

// operands: f, porosity, g; results: g_f, g_porosity
void lbm_xla_soft_bounce_back_vjp(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("soft_bounce_back_vjp", lbm_soft_bounce_back_vjp(d.dtype, b[0], b[1], b[2], b[3], b[4],
                                                          d.nx, d.ny, d.nz, stream),
         d, stream, {{b[3], 19 * cells(d) * elem(d)}, {b[4], cells(d) * elem(d)}});
}

// operands: f, q, g; results: g_f, g_q
void lbm_xla_stream_vjp(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("stream_vjp", lbm_stream_vjp(d.dtype, b[0], b[1], d.periodic_yz, b[2], b[3], b[4], d.nx,
                                      d.ny, d.nz, stream),
         d, stream, {{b[3], 19 * cells(d) * elem(d)}, {b[4], 19 * cells(d) * elem(d)}});
}

// operands: f [, u_face], g; results: g_f, g_u_face
void lbm_xla_zou_he_inlet_vjp(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  const int k = d.u_face ? 1 : 0;
  const void* uf = d.u_face ? b[1] : nullptr;
  report("zou_he_inlet_vjp", lbm_zou_he_inlet_vjp(d.dtype, b[0], uf, d.u, d.has_rho_target, d.rho,
                                                  b[1 + k], b[2 + k], b[3 + k], d.nx, d.ny, d.nz,
                                                  stream),
         d, stream, {{b[2 + k], 19 * cells(d) * elem(d)}, {b[3 + k], 3 * face(d) * elem(d)}});
}

// operands: f, g; results: g_f, g_rho_out_face
void lbm_xla_zou_he_outlet_vjp(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("zou_he_outlet_vjp", lbm_zou_he_outlet_vjp(d.dtype, b[0], d.rho, b[1], b[2], b[3], d.nx,
                                                    d.ny, d.nz, stream),
         d, stream, {{b[2], 19 * cells(d) * elem(d)}, {b[3], face(d) * elem(d)}});
}

// operands: q, g_force f64[3]; results: g_f_post, g_f_streamed
void lbm_xla_momentum_exchange_vjp(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_desc d;
  if (!read_desc(op, len, d)) return;
  report("momentum_exchange_vjp",
         lbm_momentum_exchange_vjp(d.dtype, b[0], static_cast<const double*>(b[1]), b[2], b[3],
                                   d.nx, d.ny, d.nz, stream),
         d, stream, {{b[2], 19 * cells(d) * elem(d)}, {b[3], 19 * cells(d) * elem(d)}});
}

}  // extern "C"
