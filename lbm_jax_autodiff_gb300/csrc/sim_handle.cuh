// Internal to the C-ABI translation units: the solver handle, the kernel
// launchers the handle code calls and the helpers that fill kernel argument
// blocks from a handle.
#pragma once

#include <cstdio>
#include <cstring>

#include "../../include/lbm_gb300.h"
#include "capi_util.cuh"
#include "sim.cuh"

namespace lbm {

template <class St>
cudaError_t launch_step(const StepArgs<typename Storage<St>::Re>& a, bool mrt,
                        cudaStream_t stream);
template <class Re>
cudaError_t launch_step_aa(const StepArgs<Re>& a, Re* A, const Re* sb_in, Re* sb_out, int nrec,
                           bool layout_l, bool mrt, cudaStream_t st);
cudaError_t launch_force_finalize(const double* part, int nblocks, double dyn_area, double* out,
                                  cudaStream_t stream);

struct SphereSpec {
  double c[3];
  double r;
  double alpha;
  int sigmoid_mask;
  int bouzidi;
  double disc_floor;
  double denom_eps;
};
template <class Re>
cudaError_t launch_sphere_fields(const Grid& g, const SphereSpec& s, uint8_t* solid, Re* q,
                                 Re* dqdr, cudaStream_t st);
template <class Re>
cudaError_t launch_sphere_porosity(const Grid& g, const SphereP<Re>& sp, Re* p, Re* dpdr,
                                   cudaStream_t st);
template <class Re>
cudaError_t launch_q_from_solid(const Grid& g, const uint8_t* solid, double dq, Re* q,
                                cudaStream_t st);
cudaError_t launch_solid_from_i32(int n, const int32_t* m, uint8_t* s, cudaStream_t st);
template <class Re>
cudaError_t launch_classify(const Grid& g, const uint8_t* solid, const Re* q, const Re* dqdr,
                            uint32_t* tag, LinkRec* rec, int cap, int* counter, int count_only,
                            cudaStream_t st);
cudaError_t launch_area_cols(const Grid& g, const uint8_t* solid, int* col, cudaStream_t st);
cudaError_t launch_solid_bbox(const Grid& g, const uint8_t* solid, int* bb, cudaStream_t st);
cudaError_t launch_pair_flags(const Grid& g, const uint32_t* tag, const int near[6], int use_class,
                              uint8_t* flags, cudaStream_t st);
template <class Re>
cudaError_t launch_box_fields(const Grid& g, const double lo[3], const double hi[3],
                              uint8_t* solid, Re* q, cudaStream_t st);
template <class Re>
cudaError_t launch_export_fields(const Grid& g, const SphereSpec& s, int with_porosity,
                                 const uint8_t* solid, int32_t* solid_out, Re* porosity,
                                 cudaStream_t st);

template <class Re> struct AdjArgs {
  StepArgs<Re> s;
  const void* S_k;
  const Re* nu_in;
  Re* nu_out;
  int first;
  int last;
  const double* dj_dfx;
  double* gr_partials;
  double* gq;
};
template <class St>
cudaError_t launch_adjoint(const AdjArgs<typename Storage<St>::Re>& A, bool mrt, cudaStream_t st);
template <class Re>
cudaError_t launch_adjoint_seed(const StepArgs<Re>& a, const double* dj, Re* nu, cudaStream_t st);
template <class Re>
cudaError_t launch_adjoint_seed_dense(const StepArgs<Re>& a, const Re* g, Re* nu,
                                      cudaStream_t st);
cudaError_t launch_dj_dfx(const double* fcd, double dyn_area, double* g, cudaStream_t st);
cudaError_t launch_reduce_sum(const double* part, int n, double* out, cudaStream_t st);
template <class Re>
cudaError_t launch_scatter_gq(const Grid& g, const uint32_t* tag, const LinkRec* rec,
                              const double* gq, Re* out, cudaStream_t st);

}  // namespace lbm

using namespace lbm;

struct lbm_sim {
  lbm_params p;
  Grid g;
  size_t n = 0;
  size_t st_bytes = 0;       // bytes per stored population value
  size_t re_bytes = 0;       // bytes per compute value
  void* S[2] = {nullptr, nullptr};
  int cur = 0;
  int state_is_S = 0;        // 0: f_k in fbuf; 1: S_{k-1} in S[cur]
  long long steps = 0;
  void* fbuf = nullptr;      // reference-layout f (compute dtype)
  long long fbuf_step = -1;  // fbuf holds the reference f after this many steps (-1: none)
  uint32_t* tag = nullptr;
  LinkRec* rec = nullptr;
  int nrec = 0;
  int nlinks = 0;
  double area = 0.0;
  int near[6] = {0, 0, 0, 0, 0, 0};   // rest-offset box of 16-bit storage (solid bbox + 2)
  int* spec_pairs = nullptr;          // pairs the pair kernels run per cell (pair_special)
  int nspec = 0;
  int have_geometry = 0;
  int porosity_mode = LBM_POROSITY_NONE;
  int sphere_porosity = 0;   // analytic sigmoid porosity in-kernel
  lbm_sphere sphere{};
  void* porosity = nullptr;  // porosity field (compute dtype)
  void* dpdr = nullptr;      // dp/dr field of a sigmoid sphere (compute dtype)
  void* u_face = nullptr;    // inlet profile (compute dtype)
  double* partials = nullptr;
  int nblocks = 0;
  unsigned long long* guard_count = nullptr;
  // adjoint workspace (grown on demand, kept between calls)
  void* states = nullptr;    // checkpoints + stash, storage dtype
  size_t states_cap = 0;     // in states
  void* nu[2] = {nullptr, nullptr};
  double* gq = nullptr;
  int gq_cap = 0;
  double* gr_partials = nullptr;
  double* scal = nullptr;    // [0..3] F, Cd ; [4] dJ/dFx ; [5] dJ/dr
  int plan_K = 0;            // last adjoint plan: segment length, recomputed steps, bytes
  int plan_recompute = 0;
  size_t plan_bytes = 0;
  size_t workspace_limit = 0;  // cap on the population workspace of the automatic plan (0: none)
  // in-place ("AA") streaming of lbm_run: one population buffer S[0] in
  // layout L or P, side buffers of the boundary cells' S (step_aa.cu)
  int aa = 0;
  int aa_layout_l = 0;       // S[0] holds layout L (else P)
  int aa_needs_state = 0;    // the geometry changed under an AA state
  void* sb[2] = {nullptr, nullptr};
  int sb_cur = 0;            // side buffer holding the current step's values
  size_t sb_slots = 0;
};

// Longest segment length K in [1, N] whose workspace, ceil(N/K) - 1 + K
// states, fits in `max_states` states.  The count falls as K falls from N to
// about sqrt(N) and rises below that, so the search stops there; when even
// the smallest workspace does not fit, LBM_ERR_NOMEM names the bytes it needs.
inline int plan_segment(int N, long long max_states, size_t state_bytes, int* K_out) {
  auto states = [&](long long K) { return (N + K - 1) / K - 1 + K; };
  long long K = N;
  while (K > 1 && states(K) > max_states && states(K - 1) <= states(K)) --K;
  if (states(K) > max_states) {
    char msg[200];
    snprintf(msg, sizeof(msg),
             "adjoint workspace: %d steps need at least %lld states (%.3g GB), %lld fit",
             N, states(K), double(states(K)) * double(state_bytes) / 1e9, max_states);
    return set_error(LBM_ERR_NOMEM, msg);
  }
  *K_out = int(K);
  return LBM_OK;
}

using namespace lbm;

inline bool is_fp64(const lbm_sim* s) { return s->p.storage == LBM_F64; }

template <class Re>
inline void fill_consts(const lbm_params& p, Consts<Re>& K) {
  const double w[Q] = {1.0 / 3.0,  1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                       1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                       1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                       1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
  // MRT_RELAXATION_RATES of lattice.py:106-126 (stress slots filled at run time)
  const double r[Q] = {0.0, 1.19, 1.4, 0.0, 1.2, 0.0, 1.2, 0.0, 1.2, 0.0,
                       1.4, 0.0,  1.4, 0.0, 0.0, 0.0, 1.98, 1.98, 1.98};
  for (int i = 0; i < Q; ++i) {
    K.w[i] = p.exact_constants ? Re(w[i]) : Re(double(float(w[i])));
    K.rate[i] = p.exact_constants ? Re(r[i]) : Re(double(float(r[i])));
  }
}

// Sigmoid-sphere parameters in the kernels' arithmetic type (world frame:
// x in [-4, 4], y and z in [-2, 2]); the precomputed porosity fields and the
// kernels' arguments use the same values.
template <class Re>
inline SphereP<Re> sphere_params(const lbm_sim* s) {
  SphereP<Re> p;
  p.c[0] = Re(s->sphere.center[0]);
  p.c[1] = Re(s->sphere.center[1]);
  p.c[2] = Re(s->sphere.center[2]);
  p.r = Re(s->sphere.radius);
  p.alpha = Re(s->sphere.sharpness);
  p.sx = Re(s->g.nx / 8.0);
  p.sy = Re(s->g.ny / 4.0);
  p.sz = Re(s->g.nz / 4.0);
  return p;
}

template <class Re>
inline void fill_args(const lbm_sim* s, StepArgs<Re>& a) {
  memset(&a, 0, sizeof(a));
  a.tag = s->tag;
  a.rec = s->rec;
  a.g = s->g;
  fill_consts<Re>(s->p, a.K);
  a.tau = Re(s->p.tau);
  a.c18cs2 = Re(18.0 * (s->p.smagorinsky_cs * s->p.smagorinsky_cs));
  int fl = 0;
  if (s->p.use_smagorinsky) fl |= SF_SMAG;
  if (s->porosity_mode == LBM_POROSITY_HARD) fl |= SF_SOLID_HARD;
  if (s->porosity_mode == LBM_POROSITY_SOFT) fl |= s->sphere_porosity ? SF_SOLID_SPHERE : SF_SOLID_FIELD;
  if (s->p.guard == LBM_GUARD_PRE) fl |= SF_GUARD_PRE;
  if (s->p.guard == LBM_GUARD_POST) fl |= SF_GUARD_POST;
  if (s->u_face) fl |= SF_INLET_FACE;
  a.flags = fl;
  for (int k = 0; k < 3; ++k) a.u_in[k] = Re(s->p.inlet_velocity[k]);
  a.u_face = static_cast<const Re*>(s->u_face);
  a.rho_out = Re(s->p.rho_out);
  a.sph = sphere_params<Re>(s);
  a.porosity = static_cast<const Re*>(s->porosity);
  a.dpdr = static_cast<const Re*>(s->dpdr);
  // 16-bit storage offsets: the rest equilibrium w inside the box around the
  // body, the free-stream equilibrium f_eq(1, (U, 0, 0)) elsewhere
  for (int i = 0; i < Q; ++i) {
    const double U = s->p.inlet_velocity[0];
    const double eu = ex(i) * U;
    a.soff[i] = Re(double(a.K.w[i]) * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * U * U));
    a.soff_near[i] = a.K.w[i];
  }
  for (int k = 0; k < 6; ++k) a.near[k] = s->near[k];
  a.spec_pairs = s->spec_pairs;
  a.spec_count = s->nspec;
  // guard reset targets: pre -> f_eq(1, (U,0,0)) (examples/10:160), post -> f_eq(1, 0) = w
  for (int i = 0; i < Q; ++i) {
    if (s->p.guard == LBM_GUARD_PRE) {
      const double U = s->p.inlet_velocity[0];
      const double eu = ex(i) * U;
      a.guard_reset[i] = Re(double(a.K.w[i]) * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * U * U));
    } else {
      a.guard_reset[i] = a.K.w[i];
    }
  }
  a.force_partials = s->partials;
  a.guard_count = s->guard_count;
}

inline double dyn_area(const lbm_sim* s) {
  const double U = s->p.u_ref;
  const double A = s->area > s->p.area_min ? s->area : s->p.area_min;
  return 0.5 * 1.0 * U * U * A;
}

// Launch one fused step of handle `s` from src to dst (defined in capi.cu).
int launch(const lbm_sim* s, const void* src, void* dst, int extra_flags, cudaStream_t st,
           void* f_emit = nullptr);
