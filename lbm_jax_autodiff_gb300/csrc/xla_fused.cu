// XLA custom-call targets of the fused solver (legacy api_version = 0):
//   void target(cudaStream_t stream, void** buffers, const char* opaque, size_t opaque_len)
// with `opaque` one lbm_xla_fused_desc (raw bytes).  They let a jitted JAX
// driver -- the reference's Cd study (examples/10:69-106) or its gradient
// driver (examples/11:139-176) -- reach the fused step and the hand-written
// adjoint instead of composing the per-op targets.
//
// The library keeps one solver handle per (device, lbm_params) for these
// targets, created on first use, so a jitted loop pays the allocation once.
// At most kMaxHandles are kept: a new parameter set beyond that destroys the
// least recently used handle that no call is using.  The sphere's geometry is
// rebuilt when its radius or description changes (the radius is an operand,
// read back to the host).  Keys and comparisons use the structs' fields, not
// their bytes, so padding a caller left uninitialised does not matter.
// Every target writes an int32 status (an lbm_status) as its last result;
// on failure its other results are filled with NaN (all-ones bytes) and the
// message goes to stderr.  Calls are serialised per handle by a mutex.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <map>
#include <mutex>
#include <string>

#include "../../include/lbm_gb300.h"

namespace {

struct Entry {
  lbm_sim* sim = nullptr;
  lbm_sphere sphere{};
  bool have_sphere = false;
  unsigned long long last_use = 0;
  int refs = 0;            // calls between handle_for and release (guarded by g_mu)
  std::mutex mu;
};

constexpr size_t kMaxHandles = 8;
std::mutex g_mu;
std::map<std::string, Entry*>* g_handles = nullptr;
unsigned long long g_clock = 0;

// Field-wise copies into zeroed structs: equal parameters give equal bytes.
lbm_params canonical(const lbm_params& p) {
  lbm_params c;
  std::memset(&c, 0, sizeof(c));
  c.nx = p.nx;
  c.ny = p.ny;
  c.nz = p.nz;
  c.storage = p.storage;
  c.collision = p.collision;
  c.tau = p.tau;
  c.use_smagorinsky = p.use_smagorinsky;
  c.smagorinsky_cs = p.smagorinsky_cs;
  c.periodic_yz = p.periodic_yz;
  c.guard = p.guard;
  for (int k = 0; k < 3; ++k) c.inlet_velocity[k] = p.inlet_velocity[k];
  c.rho_out = p.rho_out;
  c.u_ref = p.u_ref;
  c.area_min = p.area_min;
  c.exact_constants = p.exact_constants;
  return c;
}
lbm_sphere canonical(const lbm_sphere& s) {
  lbm_sphere c;
  std::memset(&c, 0, sizeof(c));
  for (int k = 0; k < 3; ++k) c.center[k] = s.center[k];
  c.radius = s.radius;
  c.sharpness = s.sharpness;
  c.kind = s.kind;
  c.q_mode = s.q_mode;
  c.porosity = s.porosity;
  c.disc_floor = s.disc_floor;
  c.denom_eps = s.denom_eps;
  return c;
}

__global__ void k_put_status(int32_t* status, int32_t v) { *status = v; }
__global__ void k_put2(double* a, double va, double* b, double vb) {
  *a = va;
  *b = vb;
}

bool read_fused(const char* opaque, size_t len, lbm_xla_fused_desc& d) {
  if (!opaque || len != sizeof(lbm_xla_fused_desc)) {
    std::fprintf(stderr, "lbm_gb300: bad fused custom-call descriptor (%zu bytes, want %zu)\n",
                 len, sizeof(lbm_xla_fused_desc));
    return false;
  }
  std::memcpy(&d, opaque, sizeof(d));
  return true;
}

// The handle of (current device, params), created on first use.  The entry
// is referenced until release(), so it cannot be evicted meanwhile; the
// caller serialises its calls on the entry's mutex.
int handle_for(const lbm_params& p_in, Entry** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LBM_ERR_CUDA;
  const lbm_params p = canonical(p_in);
  std::string key(reinterpret_cast<const char*>(&dev), sizeof(dev));
  key.append(reinterpret_cast<const char*>(&p), sizeof(p));
  Entry* e = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_handles) g_handles = new std::map<std::string, Entry*>();
    auto it = g_handles->find(key);
    if (it != g_handles->end()) {
      e = it->second;
    } else {
      // make room: destroy the least recently used handles no call references
      while (g_handles->size() >= kMaxHandles) {
        auto victim = g_handles->end();
        for (auto jt = g_handles->begin(); jt != g_handles->end(); ++jt)
          if (jt->second->refs == 0 &&
              (victim == g_handles->end() || jt->second->last_use < victim->second->last_use))
            victim = jt;
        if (victim == g_handles->end()) break;
        Entry* v = victim->second;
        g_handles->erase(victim);
        lbm_destroy(v->sim);
        delete v;
      }
      e = new Entry();
      const int rc = lbm_create(&p, &e->sim);
      if (rc != LBM_OK) {
        delete e;
        return rc;
      }
      (*g_handles)[key] = e;
    }
    e->last_use = ++g_clock;
    ++e->refs;
  }
  *out = e;
  return LBM_OK;
}

void release(Entry* e) {
  std::lock_guard<std::mutex> lock(g_mu);
  --e->refs;
}

// Geometry of the descriptor's sphere with the radius operand (device f64).
int set_sphere(Entry* e, const lbm_xla_fused_desc& d, const void* radius_dev, cudaStream_t st) {
  double r = 0.0;
  if (cudaMemcpyAsync(&r, radius_dev, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return LBM_ERR_CUDA;
  lbm_sphere s = canonical(d.sphere);
  s.radius = r;
  if (e->have_sphere && std::memcmp(&s, &e->sphere, sizeof(s)) == 0) return LBM_OK;
  const int rc = lbm_set_geometry_sphere(e->sim, &s, st);
  e->have_sphere = rc == LBM_OK;
  if (rc == LBM_OK) e->sphere = s;
  return rc;
}

size_t pop_bytes(const lbm_params& p) {
  return size_t(19) * size_t(p.nx) * size_t(p.ny) * size_t(p.nz) *
         (p.storage == LBM_F64 ? 8 : 4);
}

bool dims_ok(const lbm_params& p) {
  return p.nx >= 1 && p.ny >= 1 && p.nz >= 1 &&
         (long long)p.nx * p.ny * p.nz * 19 < (1LL << 31) && p.storage >= LBM_F32 &&
         p.storage <= LBM_BF16;
}

struct Res {
  void* p;
  size_t bytes;
};

void finish(const char* name, int rc, cudaStream_t st, int32_t* status,
            std::initializer_list<Res> results) {
  if (rc != LBM_OK) {
    std::fprintf(stderr, "lbm_gb300: %s failed: %s\n", name, lbm_last_error());
    for (const Res& r : results)
      if (r.p && r.bytes) cudaMemsetAsync(r.p, 0xFF, r.bytes, st);
  }
  k_put_status<<<1, 1, 0, st>>>(status, int32_t(rc));
}

}  // namespace

extern "C" {

// operands: f0 [19][n] (compute dtype), radius f64[1];
// results: f [19][n], samples f64[max(1, n_steps / sample_every)][4], status int32[1]
void lbm_xla_run(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_fused_desc d;
  if (!read_fused(op, len, d)) return;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int32_t* status = static_cast<int32_t*>(b[4]);
  const bool ok_dims = dims_ok(d.params);
  const size_t nsamp = d.sample_every > 0 && d.n_steps >= d.sample_every
                           ? size_t(d.n_steps / d.sample_every) : size_t(1);
  const size_t fbytes = ok_dims ? pop_bytes(d.params) : 0;
  Entry* e = nullptr;
  int rc = ok_dims ? handle_for(d.params, &e) : int(LBM_ERR_ARG);
  if (rc == LBM_OK) {
    {
      std::lock_guard<std::mutex> lock(e->mu);
      rc = set_sphere(e, d, b[1], st);
      if (rc == LBM_OK) rc = lbm_set_state(e->sim, b[0], st);
      if (rc == LBM_OK)
        rc = lbm_run(e->sim, d.n_steps, d.sample_every > 0 ? d.sample_every : 0,
                     d.sample_every > 0 ? static_cast<double*>(b[3]) : nullptr, st);
      if (rc == LBM_OK) rc = lbm_get_state(e->sim, b[2], st);
    }
    release(e);
  }
  if (rc == LBM_OK && d.sample_every <= 0) cudaMemsetAsync(b[3], 0, 4 * sizeof(double), st);
  finish("xla_run", rc, st, status, {{b[2], fbytes}, {b[3], nsamp * 4 * sizeof(double)}});
}

// operands: f0 [19][n] (compute dtype), radius f64[1];
// results: cd f64[1], dcd_dr f64[1], dcd_dq [19][n] (compute dtype), status int32[1]
void lbm_xla_cd_and_grad(void* stream, void** b, const char* op, size_t len) {
  lbm_xla_fused_desc d;
  if (!read_fused(op, len, d)) return;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int32_t* status = static_cast<int32_t*>(b[5]);
  const bool ok_dims = dims_ok(d.params);
  const size_t fbytes = ok_dims ? pop_bytes(d.params) : 0;
  Entry* e = nullptr;
  int rc = ok_dims ? handle_for(d.params, &e) : int(LBM_ERR_ARG);
  double cd = 0.0, g = 0.0;
  if (rc == LBM_OK) {
    {
      std::lock_guard<std::mutex> lock(e->mu);
      rc = set_sphere(e, d, b[1], st);
      if (rc == LBM_OK) rc = lbm_set_state(e->sim, b[0], st);
      if (rc == LBM_OK)
        rc = lbm_cd_and_grad(e->sim, d.n_steps, d.checkpoint_every, &cd, &g, b[4], nullptr, st);
    }
    release(e);
  }
  if (rc == LBM_OK)
    k_put2<<<1, 1, 0, st>>>(static_cast<double*>(b[2]), cd, static_cast<double*>(b[3]), g);
  finish("xla_cd_and_grad", rc, st, status,
         {{b[2], sizeof(double)}, {b[3], sizeof(double)}, {b[4], fbytes}});
}

}  // extern "C"
