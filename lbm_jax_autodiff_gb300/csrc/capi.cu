// C ABI of the fused solver handle (include/lbm_gb300.h).
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sim_handle.cuh"

int launch(const lbm_sim* s, const void* src, void* dst, int extra_flags, cudaStream_t st,
           void* f_emit) {
  cudaError_t e;
  const bool mrt = s->p.collision == LBM_MRT;
  if (is_fp64(s)) {
    StepArgs<double> a;
    fill_args<double>(s, a);
    a.src = src;
    a.dst = dst;
    a.flags |= extra_flags;
    a.f_emit = f_emit;
    e = launch_step<double>(a, mrt, st);
  } else {
    StepArgs<float> a;
    fill_args<float>(s, a);
    a.src = src;
    a.dst = dst;
    a.flags |= extra_flags;
    a.f_emit = f_emit;
    switch (s->p.storage) {
      case LBM_F32: e = launch_step<float>(a, mrt, st); break;
      case LBM_F16: e = launch_step<__half>(a, mrt, st); break;
      default: e = launch_step<__nv_bfloat16>(a, mrt, st); break;
    }
  }
  return cuda_check(e, "k_step launch");
}

namespace {

// Side buffers of the AA scheme: one S vector per boundary record and per
// x-face cell, two copies.
int ensure_aa(lbm_sim* s) {
  const size_t slots = size_t(s->nrec) + size_t(2) * s->g.ny * s->g.nz;
  if (s->sb_slots >= slots && s->sb[0] && s->sb[1]) return LBM_OK;
  for (int b = 0; b < 2; ++b) {
    cudaFree(s->sb[b]);
    s->sb[b] = nullptr;
  }
  s->sb_slots = 0;
  for (int b = 0; b < 2; ++b) LBM_TRY(dev_alloc(&s->sb[b], slots * Q * s->re_bytes));
  s->sb_slots = slots;
  return LBM_OK;
}

// The second population buffer of the A/B scheme (released in AA mode).
int ensure_ab(lbm_sim* s) {
  if (!s->S[1]) LBM_TRY(dev_alloc(&s->S[1], s->n * Q * s->st_bytes));
  return LBM_OK;
}

// One AA launch from the handle's state: SF_COLLIDE_ONLY from f_0 (fbuf),
// a step (the layout flips), or SF_STREAM_ONLY into f_out (state unchanged).
template <class Re>
int aa_launch_t(lbm_sim* s, int extra, void* f_out, cudaStream_t st) {
  StepArgs<Re> a;
  fill_args<Re>(s, a);
  a.flags |= extra;
  a.src = (extra & SF_COLLIDE_ONLY) ? s->fbuf : nullptr;
  a.dst = (extra & SF_STREAM_ONLY) ? f_out : nullptr;
  const bool mrt = s->p.collision == LBM_MRT;
  Re* A = static_cast<Re*>(s->S[0]);
  const Re* sb_in = static_cast<const Re*>(s->sb[s->sb_cur]);
  Re* sb_out = static_cast<Re*>(s->sb[1 - s->sb_cur]);
  LBM_TRY(cuda_check(launch_step_aa<Re>(a, A, sb_in, sb_out, s->nrec, s->aa_layout_l != 0, mrt, st),
                     "k_step_aa launch"));
  if (!(extra & SF_STREAM_ONLY)) {
    s->sb_cur = 1 - s->sb_cur;
    s->aa_layout_l = (extra & SF_COLLIDE_ONLY) ? 1 : 1 - s->aa_layout_l;
  }
  return LBM_OK;
}

int aa_launch(lbm_sim* s, int extra, void* f_out, cudaStream_t st) {
  LBM_TRY(ensure_aa(s));
  return is_fp64(s) ? aa_launch_t<double>(s, extra, f_out, st)
                    : aa_launch_t<float>(s, extra, f_out, st);
}

template <class Re>
int adjoint_launch_t(const lbm_sim* s, const void* S_prev, const void* S_k, const Re* nu_in,
                     Re* nu_out, int first, int last, cudaStream_t st) {
  AdjArgs<Re> A;
  memset(&A, 0, sizeof(A));
  fill_args<Re>(s, A.s);
  A.s.flags &= ~(SF_GUARD_PRE | SF_GUARD_POST);
  A.s.src = S_prev;
  A.S_k = S_k;
  A.nu_in = nu_in;
  A.nu_out = nu_out;
  A.first = first;
  A.last = last;
  A.dj_dfx = s->scal + 4;
  A.gr_partials = s->gr_partials;
  A.gq = s->gq;
  const bool mrt = s->p.collision == LBM_MRT;
  cudaError_t e;
  if constexpr (sizeof(Re) == 8) {
    e = launch_adjoint<double>(A, mrt, st);
  } else {
    switch (s->p.storage) {
      case LBM_F32: e = launch_adjoint<float>(A, mrt, st); break;
      case LBM_F16: e = launch_adjoint<__half>(A, mrt, st); break;
      default: e = launch_adjoint<__nv_bfloat16>(A, mrt, st); break;
    }
  }
  return cuda_check(e, "k_adjoint launch");
}

int adjoint_launch(const lbm_sim* s, const void* S_prev, const void* S_k, const void* nu_in,
                   void* nu_out, int first, int last, cudaStream_t st) {
  if (is_fp64(s))
    return adjoint_launch_t<double>(s, S_prev, S_k, static_cast<const double*>(nu_in),
                                    static_cast<double*>(nu_out), first, last, st);
  return adjoint_launch_t<float>(s, S_prev, S_k, static_cast<const float*>(nu_in),
                                 static_cast<float*>(nu_out), first, last, st);
}

int adjoint_seed(const lbm_sim* s, void* nu, cudaStream_t st) {
  cudaError_t e;
  if (is_fp64(s)) {
    StepArgs<double> a;
    fill_args<double>(s, a);
    e = launch_adjoint_seed<double>(a, s->scal + 4, static_cast<double*>(nu), st);
  } else {
    StepArgs<float> a;
    fill_args<float>(s, a);
    e = launch_adjoint_seed<float>(a, s->scal + 4, static_cast<float*>(nu), st);
  }
  return cuda_check(e, "adjoint seed");
}

// nu_N = Z^T g for a cotangent g on the final f_N (compute type).
int adjoint_seed_dense(const lbm_sim* s, const void* g, void* nu, cudaStream_t st) {
  cudaError_t e;
  if (is_fp64(s)) {
    StepArgs<double> a;
    fill_args<double>(s, a);
    e = launch_adjoint_seed_dense<double>(a, static_cast<const double*>(g),
                                          static_cast<double*>(nu), st);
  } else {
    StepArgs<float> a;
    fill_args<float>(s, a);
    e = launch_adjoint_seed_dense<float>(a, static_cast<const float*>(g),
                                         static_cast<float*>(nu), st);
  }
  return cuda_check(e, "adjoint dense seed");
}

void free_geometry(lbm_sim* s) {
  cudaFree(s->tag);
  cudaFree(s->rec);
  cudaFree(s->porosity);
  cudaFree(s->dpdr);
  cudaFree(s->spec_pairs);
  s->spec_pairs = nullptr;
  s->nspec = 0;
  s->tag = nullptr;
  s->rec = nullptr;
  s->porosity = s->dpdr = nullptr;
  s->nrec = 0;
  s->nlinks = 0;
  s->have_geometry = 0;
}

// The pairs (z even) that the packed pair kernels run on their per-cell path,
// in ascending order; flagged on the device with the kernels' own predicate.
// Only for even nz (the pair kernels' condition).
int build_pair_list(lbm_sim* s, cudaStream_t st) {
  cudaFree(s->spec_pairs);
  s->spec_pairs = nullptr;
  s->nspec = 0;
  if (s->g.nz % 2 != 0 || s->p.storage == LBM_F64) return LBM_OK;
  const int np = s->g.n / 2;
  const int use_class = (s->p.storage == LBM_F16 || s->p.storage == LBM_BF16) ? 1 : 0;
  uint8_t* flags = nullptr;
  LBM_TRY(dev_alloc((void**)&flags, size_t(np)));
  std::vector<uint8_t> h(np);
  int rc = cuda_check(launch_pair_flags(s->g, s->tag, s->near, use_class, flags, st), "pair flags");
  if (!rc) rc = cuda_check(cudaMemcpyAsync(h.data(), flags, size_t(np), cudaMemcpyDeviceToHost, st),
                           "flags D2H");
  if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "sync");
  cudaFree(flags);
  if (rc) return rc;
  std::vector<int> list;
  for (int p = 0; p < np; ++p)
    if (h[p]) list.push_back(p);
  int* d = nullptr;
  LBM_TRY(dev_alloc((void**)&d, (list.empty() ? 1 : list.size()) * sizeof(int)));
  if (!list.empty() &&
      (rc = cuda_check(cudaMemcpy(d, list.data(), list.size() * sizeof(int),
                                  cudaMemcpyHostToDevice), "list H2D"))) {
    cudaFree(d);
    return rc;
  }
  s->spec_pairs = d;
  s->nspec = int(list.size());
  return LBM_OK;
}

// Shared tail of the two geometry entry points: classify cells from the dense
// q (compute dtype), count links, projected area.
template <class Re>
int finish_geometry(lbm_sim* s, const uint8_t* solid, const Re* q, const Re* dqdr,
                    cudaStream_t st) {
  int* counter = nullptr;
  int* cols = nullptr;
  int* bb = nullptr;
  int hbb[6] = {0, -1, 0, -1, 0, -1};
  const int ncol = s->g.ny * s->g.nz;
  LBM_TRY(dev_alloc((void**)&counter, sizeof(int)));
  if (!s->tag) LBM_TRY(dev_alloc((void**)&s->tag, s->n * sizeof(uint32_t)));
  int rc = LBM_OK;
  do {
    if ((rc = cuda_check(cudaMemsetAsync(counter, 0, sizeof(int), st), "memset"))) break;
    if ((rc = cuda_check(launch_classify<Re>(s->g, solid, q, dqdr, s->tag, nullptr, 0, counter, 1, st),
                         "classify count")))
      break;
    int count = 0;
    if ((rc = cuda_check(cudaMemcpyAsync(&count, counter, sizeof(int), cudaMemcpyDeviceToHost, st),
                         "count D2H")))
      break;
    if ((rc = cuda_check(cudaStreamSynchronize(st), "sync"))) break;
    cudaFree(s->rec);
    s->rec = nullptr;
    if (count > 0 && (rc = dev_alloc((void**)&s->rec, size_t(count) * sizeof(LinkRec)))) break;
    if ((rc = cuda_check(cudaMemsetAsync(counter, 0, sizeof(int), st), "memset"))) break;
    if ((rc = cuda_check(launch_classify<Re>(s->g, solid, q, dqdr, s->tag, s->rec, count, counter, 0, st),
                         "classify fill")))
      break;
    s->nrec = count;
    // rest-offset box of 16-bit storage: the solid cells' bounding box grown
    // by 2 cells (clipped to the grid)
    if ((rc = dev_alloc((void**)&bb, 6 * sizeof(int)))) break;
    {
      const int init[6] = {INT_MAX, -1, INT_MAX, -1, INT_MAX, -1};
      if ((rc = cuda_check(cudaMemcpyAsync(bb, init, sizeof(init), cudaMemcpyHostToDevice, st),
                           "bbox H2D")))
        break;
      if ((rc = cuda_check(launch_solid_bbox(s->g, solid, bb, st), "bbox"))) break;
      if ((rc = cuda_check(cudaMemcpyAsync(hbb, bb, sizeof(hbb), cudaMemcpyDeviceToHost, st),
                           "bbox D2H")))
        break;
    }
    // link count and projected area
    if ((rc = dev_alloc((void**)&cols, ncol * sizeof(int)))) break;
    if ((rc = cuda_check(cudaMemsetAsync(cols, 0, ncol * sizeof(int), st), "memset"))) break;
    if ((rc = cuda_check(launch_area_cols(s->g, solid, cols, st), "area"))) break;
    std::vector<int> hc(ncol);
    if ((rc = cuda_check(cudaMemcpyAsync(hc.data(), cols, ncol * sizeof(int), cudaMemcpyDeviceToHost, st),
                         "area D2H")))
      break;
    std::vector<LinkRec> hr(count);
    if (count > 0 &&
        (rc = cuda_check(cudaMemcpyAsync(hr.data(), s->rec, count * sizeof(LinkRec),
                                         cudaMemcpyDeviceToHost, st),
                         "rec D2H")))
      break;
    if ((rc = cuda_check(cudaStreamSynchronize(st), "sync"))) break;
    long long a = 0;
    for (int v : hc) a += v;
    s->area = double(a);
    if (hbb[1] < 0) {
      for (int k = 0; k < 6; ++k) s->near[k] = 0;   // no solid: free-stream offset everywhere
    } else {
      const int dims[3] = {s->g.nx, s->g.ny, s->g.nz};
      for (int k = 0; k < 3; ++k) {
        int lo = hbb[2 * k] - 2, hi = hbb[2 * k + 1] + 3;
        if (k == 2) {   // even z bounds: both cells of a z-pair share the class
          lo &= ~1;
          hi += hi & 1;
        }
        s->near[2 * k] = lo < 0 ? 0 : lo;
        s->near[2 * k + 1] = hi > dims[k] ? dims[k] : hi;
      }
    }
    int nl = 0;
    for (const auto& r : hr) nl += __builtin_popcount(r.linkmask);
    s->nlinks = nl;
    if ((rc = build_pair_list(s, st))) break;
    s->have_geometry = 1;
    // the side buffers of an in-place state belong to the old records
    if (s->aa && s->state_is_S) s->aa_needs_state = 1;
  } while (0);
  cudaFree(counter);
  cudaFree(cols);
  cudaFree(bb);
  return rc;
}

template <class Re>
int set_sphere_impl(lbm_sim* s, const lbm_sphere* sp, cudaStream_t st) {
  uint8_t* solid = nullptr;
  Re* q = nullptr;
  Re* dq = nullptr;
  int rc = LBM_OK;
  do {
    if ((rc = dev_alloc((void**)&solid, s->n))) break;
    if ((rc = dev_alloc((void**)&q, s->n * Q * sizeof(Re)))) break;
    if ((rc = dev_alloc((void**)&dq, s->n * Q * sizeof(Re)))) break;
    SphereSpec spec;
    for (int k = 0; k < 3; ++k) spec.c[k] = sp->center[k];
    spec.r = sp->radius;
    spec.alpha = sp->sharpness;
    spec.sigmoid_mask = sp->kind == LBM_SPHERE_SIGMOID_MASK;
    spec.bouzidi = sp->q_mode == LBM_Q_BOUZIDI;
    spec.disc_floor = sp->disc_floor;
    spec.denom_eps = sp->denom_eps;
    if ((rc = cuda_check(launch_sphere_fields<Re>(s->g, spec, solid, q, dq, st), "sphere fields")))
      break;
    rc = finish_geometry<Re>(s, solid, q, dq, st);
  } while (0);
  cudaStreamSynchronize(st);
  cudaFree(solid);
  cudaFree(q);
  cudaFree(dq);
  return rc;
}

template <class Re>
int set_mask_impl(lbm_sim* s, const int32_t* solid_i32, const void* q_user, double default_q,
                  cudaStream_t st) {
  uint8_t* solid = nullptr;
  Re* q = nullptr;
  int rc = LBM_OK;
  do {
    if ((rc = dev_alloc((void**)&solid, s->n))) break;
    if ((rc = cuda_check(launch_solid_from_i32(int(s->n), solid_i32, solid, st), "solid"))) break;
    const Re* qq = static_cast<const Re*>(q_user);
    if (!qq) {
      if ((rc = dev_alloc((void**)&q, s->n * Q * sizeof(Re)))) break;
      if ((rc = cuda_check(launch_q_from_solid<Re>(s->g, solid, default_q, q, st), "q from solid")))
        break;
      qq = q;
    }
    rc = finish_geometry<Re>(s, solid, qq, nullptr, st);
  } while (0);
  cudaStreamSynchronize(st);
  cudaFree(solid);
  cudaFree(q);
  return rc;
}

}  // namespace

template <class Re>
static int sphere_fields_impl(int nx, int ny, int nz, const lbm_sphere* sp, int32_t* solid_out,
                              Re* q, Re* dqdr, Re* porosity, cudaStream_t st) {
  const Grid g = make_grid(nx, ny, nz, 1);
  SphereSpec spec;
  for (int k = 0; k < 3; ++k) spec.c[k] = sp->center[k];
  spec.r = sp->radius;
  spec.alpha = sp->sharpness;
  spec.sigmoid_mask = sp->kind == LBM_SPHERE_SIGMOID_MASK;
  spec.bouzidi = sp->q_mode == LBM_Q_BOUZIDI;
  spec.disc_floor = sp->disc_floor;
  spec.denom_eps = sp->denom_eps;
  uint8_t* solid = nullptr;
  Re* dq_tmp = nullptr;
  LBM_TRY(dev_alloc((void**)&solid, size_t(g.n)));
  int rc = LBM_OK;
  do {
    Re* dq = dqdr;
    if (!dq && (rc = dev_alloc((void**)&dq_tmp, size_t(g.n) * Q * sizeof(Re)))) break;
    if (!dq) dq = dq_tmp;
    if ((rc = cuda_check(launch_sphere_fields<Re>(g, spec, solid, q, dq, st), "sphere fields"))) break;
    rc = cuda_check(launch_export_fields<Re>(g, spec, sp->porosity == LBM_POROSITY_SOFT, solid,
                                             solid_out, porosity, st), "export");
  } while (0);
  cudaStreamSynchronize(st);
  cudaFree(solid);
  cudaFree(dq_tmp);
  return rc;
}

extern "C" {

int lbm_api_version(void) { return LBM_GB300_API_VERSION; }

int lbm_create(const lbm_params* p, lbm_sim** out) {
  if (!p || !out) return set_error(LBM_ERR_ARG, "lbm_create: null argument");
  *out = nullptr;
  if (p->nx < 3 || p->ny < 1 || p->nz < 1)
    return set_error(LBM_ERR_ARG, "lbm_create: need nx >= 3, ny >= 1, nz >= 1");
  const long long n = (long long)p->nx * p->ny * p->nz;
  if (n * Q >= (1LL << 31))
    return set_error(LBM_ERR_UNSUPPORTED, "lbm_create: 19*cells must be < 2^31");
  if (p->storage < LBM_F32 || p->storage > LBM_BF16)
    return set_error(LBM_ERR_ARG, "lbm_create: bad storage dtype");
  if (p->collision != LBM_BGK && p->collision != LBM_MRT)
    return set_error(LBM_ERR_ARG, "lbm_create: bad collision");
  if (p->guard < LBM_GUARD_OFF || p->guard > LBM_GUARD_POST)
    return set_error(LBM_ERR_ARG, "lbm_create: bad guard mode");
  if (!(p->tau > 0.5)) return set_error(LBM_ERR_ARG, "lbm_create: tau must be > 0.5");
  if (p->rho_out <= 0.0) return set_error(LBM_ERR_ARG, "lbm_create: rho_out must be > 0");
  lbm_sim* s = new (std::nothrow) lbm_sim();
  if (!s) return set_error(LBM_ERR_NOMEM, "lbm_create: host allocation failed");
  s->p = *p;
  s->g = make_grid(p->nx, p->ny, p->nz, p->periodic_yz);
  s->n = size_t(n);
  s->st_bytes = p->storage == LBM_F64 ? 8 : (p->storage == LBM_F32 ? 4 : 2);
  s->re_bytes = p->storage == LBM_F64 ? 8 : 4;
  s->nblocks = int((n + 255) / 256);
  int rc = LBM_OK;
  do {
    if ((rc = dev_alloc(&s->S[0], s->n * Q * s->st_bytes))) break;
    if ((rc = dev_alloc(&s->S[1], s->n * Q * s->st_bytes))) break;
    if ((rc = dev_alloc(&s->fbuf, s->n * Q * s->re_bytes))) break;
    if ((rc = dev_alloc((void**)&s->partials, size_t(s->nblocks) * 3 * sizeof(double)))) break;
    if ((rc = dev_alloc((void**)&s->guard_count, sizeof(unsigned long long)))) break;
    if ((rc = cuda_check(cudaMemset(s->guard_count, 0, sizeof(unsigned long long)), "memset"))) break;
    if ((rc = dev_alloc((void**)&s->tag, s->n * sizeof(uint32_t)))) break;
    if ((rc = cuda_check(cudaMemset(s->tag, 0, s->n * sizeof(uint32_t)), "memset"))) break;
  } while (0);
  if (rc) {
    lbm_destroy(s);
    return rc;
  }
  *out = s;
  return LBM_OK;
}

int lbm_destroy(lbm_sim* s) {
  if (!s) return LBM_OK;
  cudaFree(s->S[0]);
  cudaFree(s->S[1]);
  cudaFree(s->sb[0]);
  cudaFree(s->sb[1]);
  cudaFree(s->fbuf);
  cudaFree(s->partials);
  cudaFree(s->guard_count);
  cudaFree(s->u_face);
  cudaFree(s->states);
  cudaFree(s->nu[0]);
  cudaFree(s->nu[1]);
  cudaFree(s->gq);
  cudaFree(s->gr_partials);
  cudaFree(s->scal);
  free_geometry(s);
  delete s;
  return LBM_OK;
}

int lbm_set_geometry_sphere(lbm_sim* s, const lbm_sphere* sp, void* stream) {
  if (!s || !sp) return set_error(LBM_ERR_ARG, "lbm_set_geometry_sphere: null argument");
  if (!(sp->radius > 0.0)) return set_error(LBM_ERR_ARG, "lbm_set_geometry_sphere: radius <= 0");
  if (sp->porosity < LBM_POROSITY_NONE || sp->porosity > LBM_POROSITY_SOFT ||
      (sp->q_mode != LBM_Q_HALFWAY && sp->q_mode != LBM_Q_BOUZIDI) ||
      (sp->kind != LBM_SPHERE_DIST_MASK && sp->kind != LBM_SPHERE_SIGMOID_MASK))
    return set_error(LBM_ERR_ARG, "lbm_set_geometry_sphere: bad enum");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaFree(s->porosity);
  cudaFree(s->dpdr);
  s->porosity = s->dpdr = nullptr;
  s->sphere = *sp;
  s->porosity_mode = sp->porosity;
  s->sphere_porosity = sp->porosity == LBM_POROSITY_SOFT;
  LBM_TRY(is_fp64(s) ? set_sphere_impl<double>(s, sp, st) : set_sphere_impl<float>(s, sp, st));
  if (!s->sphere_porosity) return LBM_OK;
  // sigmoid sphere: porosity and dp/dr fields for the kernels
  LBM_TRY(dev_alloc(&s->porosity, s->n * s->re_bytes));
  LBM_TRY(dev_alloc(&s->dpdr, s->n * s->re_bytes));
  const cudaError_t e =
      is_fp64(s) ? launch_sphere_porosity<double>(s->g, sphere_params<double>(s),
                                                  static_cast<double*>(s->porosity),
                                                  static_cast<double*>(s->dpdr), st)
                 : launch_sphere_porosity<float>(s->g, sphere_params<float>(s),
                                                 static_cast<float*>(s->porosity),
                                                 static_cast<float*>(s->dpdr), st);
  return cuda_check(e, "sphere porosity");
}

int lbm_set_geometry_mask(lbm_sim* s, const int32_t* solid, const void* q, double default_q,
                          const void* porosity, void* stream) {
  if (!s || !solid) return set_error(LBM_ERR_ARG, "lbm_set_geometry_mask: null argument");
  LBM_TRY(check_align(solid, 4, "solid"));
  LBM_TRY(check_align(q, s->re_bytes, "q"));
  LBM_TRY(check_align(porosity, s->re_bytes, "porosity"));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaFree(s->porosity);
  cudaFree(s->dpdr);
  s->porosity = s->dpdr = nullptr;
  s->sphere_porosity = 0;
  if (porosity) {
    LBM_TRY(dev_alloc(&s->porosity, s->n * s->re_bytes));
    LBM_TRY(cuda_check(cudaMemcpyAsync(s->porosity, porosity, s->n * s->re_bytes,
                                       cudaMemcpyDeviceToDevice, st),
                       "porosity copy"));
    s->porosity_mode = LBM_POROSITY_SOFT;
  } else {
    s->porosity_mode = LBM_POROSITY_HARD;
  }
  return is_fp64(s) ? set_mask_impl<double>(s, solid, q, default_q, st)
                    : set_mask_impl<float>(s, solid, q, default_q, st);
}

int lbm_set_inlet_profile(lbm_sim* s, const void* u_face, void* stream) {
  if (!s) return set_error(LBM_ERR_ARG, "lbm_set_inlet_profile: null handle");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!u_face) {
    cudaFree(s->u_face);
    s->u_face = nullptr;
    return LBM_OK;
  }
  LBM_TRY(check_align(u_face, s->re_bytes, "u_face"));
  const size_t bytes = size_t(3) * s->g.ny * s->g.nz * s->re_bytes;
  if (!s->u_face) LBM_TRY(dev_alloc(&s->u_face, bytes));
  return cuda_check(cudaMemcpyAsync(s->u_face, u_face, bytes, cudaMemcpyDeviceToDevice, st),
                    "inlet copy");
}

int lbm_set_state(lbm_sim* s, const void* f, void* stream) {
  if (!s || !f) return set_error(LBM_ERR_ARG, "lbm_set_state: null argument");
  LBM_TRY(check_align(f, s->re_bytes, "f"));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_TRY(cuda_check(cudaMemcpyAsync(s->fbuf, f, s->n * Q * s->re_bytes, cudaMemcpyDeviceToDevice, st),
                     "state copy"));
  s->state_is_S = 0;
  s->steps = 0;
  s->fbuf_step = 0;
  s->aa_needs_state = 0;
  return LBM_OK;
}

int lbm_set_state_host(lbm_sim* s, const void* f_host, void* stream) {
  if (!s || !f_host) return set_error(LBM_ERR_ARG, "lbm_set_state_host: null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_TRY(cuda_check(cudaMemcpyAsync(s->fbuf, f_host, s->n * Q * s->re_bytes,
                                     cudaMemcpyHostToDevice, st),
                     "state H2D"));
  s->state_is_S = 0;
  s->steps = 0;
  s->fbuf_step = 0;
  s->aa_needs_state = 0;
  return LBM_OK;
}

int lbm_get_state_host(lbm_sim* s, void* f_host, void* stream) {
  if (!s || !f_host) return set_error(LBM_ERR_ARG, "lbm_get_state_host: null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (s->state_is_S && s->fbuf_step != s->steps) {
    // f of the current step is not in fbuf yet: one stream-only pass (the
    // first-step input f_0 it overwrites is no longer needed)
    if (!s->have_geometry) return set_error(LBM_ERR_STATE, "lbm_get_state_host: no geometry");
    if (s->aa)
      LBM_TRY(aa_launch(s, SF_STREAM_ONLY, s->fbuf, st));
    else
      LBM_TRY(launch(s, s->S[s->cur], s->fbuf, SF_STREAM_ONLY, st));
    s->fbuf_step = s->steps;
  }
  return cuda_check(cudaMemcpyAsync(f_host, s->fbuf, s->n * Q * s->re_bytes,
                                    cudaMemcpyDeviceToHost, st),
                    "state D2H");
}

int lbm_get_state(lbm_sim* s, void* f, void* stream) {
  if (!s || !f) return set_error(LBM_ERR_ARG, "lbm_get_state: null argument");
  LBM_TRY(check_align(f, s->re_bytes, "f"));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!s->state_is_S)
    return cuda_check(cudaMemcpyAsync(f, s->fbuf, s->n * Q * s->re_bytes, cudaMemcpyDeviceToDevice, st),
                      "state copy");
  if (!s->have_geometry) return set_error(LBM_ERR_STATE, "lbm_get_state: no geometry");
  if (s->fbuf_step == s->steps)
    // the last run's final sample pass already wrote f of this step
    return cuda_check(cudaMemcpyAsync(f, s->fbuf, s->n * Q * s->re_bytes, cudaMemcpyDeviceToDevice,
                                      st),
                      "state copy");
  if (s->aa) return aa_launch(s, SF_STREAM_ONLY, f, st);
  return launch(s, s->S[s->cur], f, SF_STREAM_ONLY, st);
}

int lbm_get_state_and_step(lbm_sim* s, void* f, void* stream) {
  if (!s || !f) return set_error(LBM_ERR_ARG, "lbm_get_state_and_step: null argument");
  LBM_TRY(check_align(f, s->re_bytes, "f"));
  if (!s->have_geometry)
    return set_error(LBM_ERR_STATE, "lbm_get_state_and_step: set a geometry first");
  if (s->aa_needs_state)
    return set_error(LBM_ERR_STATE,
                     "lbm_get_state_and_step: the streaming scheme changed, or the geometry "
                     "changed under an in-place (AA) state; call lbm_set_state");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!s->state_is_S || s->aa || s->fbuf_step == s->steps) {
    // nothing to fuse: f is already at hand, or the in-place scheme
    LBM_TRY(lbm_get_state(s, f, stream));
    return lbm_run(s, 1, 0, nullptr, stream);
  }
  LBM_TRY(ensure_ab(s));
  LBM_TRY(launch(s, s->S[s->cur], s->S[1 - s->cur], SF_EMIT_F, st, f));
  s->cur = 1 - s->cur;
  s->steps += 1;
  return LBM_OK;
}

int lbm_run(lbm_sim* s, int n_steps, int sample_every, double* samples, void* stream) {
  if (!s) return set_error(LBM_ERR_ARG, "lbm_run: null handle");
  if (n_steps < 0) return set_error(LBM_ERR_ARG, "lbm_run: n_steps < 0");
  if (sample_every < 0 || (sample_every > 0 && !samples))
    return set_error(LBM_ERR_ARG, "lbm_run: sample_every > 0 needs a samples buffer");
  LBM_TRY(check_align(samples, 8, "samples"));
  if (!s->have_geometry) return set_error(LBM_ERR_STATE, "lbm_run: set a geometry first");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double da = dyn_area(s);
  // force after global step k is computed by the launch that reads S_{k-1}
  auto want_sample = [&](long long k_global, long long k0) -> long long {
    if (sample_every <= 0) return -1;
    const long long rel = k_global - k0;
    if (rel <= 0 || rel % sample_every) return -1;
    return rel / sample_every - 1;
  };
  const long long k0 = s->steps;
  if (s->aa_needs_state)
    return set_error(LBM_ERR_STATE,
                     "lbm_run: the streaming scheme changed, or the geometry changed under an "
                     "in-place (AA) state; call lbm_set_state");
  if (s->aa) {
    for (int L = 1; L <= n_steps; ++L) {
      if (!s->state_is_S) {
        LBM_TRY(aa_launch(s, SF_COLLIDE_ONLY, nullptr, st));
        s->state_is_S = 1;
      } else {
        const long long si = want_sample(s->steps, k0);
        LBM_TRY(aa_launch(s, si >= 0 ? SF_FORCE : 0, nullptr, st));
        if (si >= 0)
          LBM_TRY(cuda_check(launch_force_finalize(s->partials, s->nblocks, da, samples + 4 * si,
                                                   st),
                             "force finalize"));
      }
      s->steps += 1;
    }
    const long long si = want_sample(s->steps, k0);
    if (si >= 0) {
      LBM_TRY(aa_launch(s, SF_STREAM_ONLY | SF_FORCE, s->fbuf, st));
      s->fbuf_step = s->steps;
      LBM_TRY(cuda_check(launch_force_finalize(s->partials, s->nblocks, da, samples + 4 * si, st),
                         "force finalize"));
    }
    return LBM_OK;
  }
  LBM_TRY(ensure_ab(s));
  for (int L = 1; L <= n_steps; ++L) {
    if (!s->state_is_S) {
      LBM_TRY(launch(s, s->fbuf, s->S[s->cur], SF_COLLIDE_ONLY, st));
      s->state_is_S = 1;
    } else {
      const long long kdone = s->steps;  // this launch computes f_{kdone}
      const long long si = want_sample(kdone, k0);
      const int extra = si >= 0 ? SF_FORCE : 0;
      LBM_TRY(launch(s, s->S[s->cur], s->S[1 - s->cur], extra, st));
      if (si >= 0)
        LBM_TRY(cuda_check(launch_force_finalize(s->partials, s->nblocks, da, samples + 4 * si, st),
                           "force finalize"));
      s->cur = 1 - s->cur;
    }
    s->steps += 1;
  }
  const long long si = want_sample(s->steps, k0);
  if (si >= 0) {
    // sample after the last step: stream-only pass with the force, state
    // unchanged; fbuf then holds the reference f of this step
    LBM_TRY(launch(s, s->S[s->cur], s->fbuf, SF_STREAM_ONLY | SF_FORCE, st));
    s->fbuf_step = s->steps;
    LBM_TRY(cuda_check(launch_force_finalize(s->partials, s->nblocks, da, samples + 4 * si, st),
                       "force finalize"));
  }
  return LBM_OK;
}

namespace {

// One gradient evaluation from the state set by lbm_set_state.  Without
// `seed_f` the backward pass starts from the drag coefficient (Cd and dCd/dr
// returned); with `seed_f`, a cotangent on the final f_N (compute type), it
// starts from that and cd / dcd_dr are not computed.  dcd_dq / dcd_df0 (may
// be null) receive the cotangents of q and f_0.
int cd_and_grad_impl(lbm_sim* s, int n_steps, int checkpoint_every, double* cd_host,
                     double* dcd_dr_host, void* dcd_dq, void* dcd_df0, cudaStream_t st,
                     const void* seed_f) {
  const int N = n_steps;
  LBM_TRY(ensure_ab(s));
  const size_t state_bytes = s->n * Q * s->st_bytes;
  for (int b = 0; b < 2; ++b)
    if (!s->nu[b]) LBM_TRY(dev_alloc(&s->nu[b], s->n * Q * s->re_bytes));
  // per-warp dJ/dr slots: nblocks * 8 of the step launches, then as many for
  // the list launch of the pair kernels' boundary pairs
  if (!s->gr_partials)
    LBM_TRY(dev_alloc((void**)&s->gr_partials, size_t(s->nblocks) * 16 * sizeof(double)));
  if (!s->scal) LBM_TRY(dev_alloc((void**)&s->scal, 8 * sizeof(double)));
  if (s->gq_cap < s->nrec) {
    cudaFree(s->gq);
    s->gq = nullptr;
    s->gq_cap = 0;
    LBM_TRY(dev_alloc((void**)&s->gq, size_t(s->nrec > 0 ? s->nrec : 1) * Q * sizeof(double)));
    s->gq_cap = s->nrec;
  }
  // Segment length K: the last segment's populations come straight from the
  // forward pass, earlier segments are recomputed from their checkpoints, so
  // N - K steps are recomputed and ceil(N/K) - 1 + K states are stored
  // (a checkpoint per segment start after the first, K stashed states).
  int K = checkpoint_every;
  if (K <= 0) {
    size_t free_b = 0, total_b = 0;
    LBM_TRY(cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo"));
    free_b += s->states_cap * state_bytes;   // the current workspace is reusable
    const size_t reserve = (size_t(2) << 30) + total_b / 50;
    size_t avail = free_b > reserve ? free_b - reserve : 0;
    if (s->workspace_limit && s->workspace_limit < avail) avail = s->workspace_limit;
    LBM_TRY(plan_segment(N, (long long)(avail / state_bytes), state_bytes, &K));
  }
  if (K > N) K = N;
  const int nseg = (N + K - 1) / K;
  const size_t need = size_t(nseg - 1) + size_t(K);
  if (s->states_cap < need) {
    cudaFree(s->states);
    s->states = nullptr;
    s->states_cap = 0;
    LBM_TRY(dev_alloc(&s->states, need * state_bytes));
    s->states_cap = need;
  }
  s->plan_K = K;
  s->plan_recompute = N - K;
  s->plan_bytes = need * state_bytes;
  char* base = static_cast<char*>(s->states);
  auto ckpt = [&](int c) -> void* { return base + size_t(c) * state_bytes; };  // S_{a_{c+1}-1}
  // stash(j), j = 1..K: S_{a+j-1} of the segment [a, a+K) being run backwards
  auto stash = [&](int j) -> void* { return base + size_t(nseg - 2 + j) * state_bytes; };
  // segment c covers [seg_a(c), seg_a(c+1)); the last one has exactly K steps
  auto seg_a = [&](int c) -> int {
    if (c <= 0) return 0;
    if (c >= nseg) return N;
    return N - (nseg - c) * K;
  };
  const int a_last = seg_a(nseg - 1);

  // ---- forward: checkpoints at segment starts, last segment straight into the stash
  const void* prev = s->fbuf;
  int next_ck = 1;
  for (int k = 0; k < N; ++k) {
    void* dst;
    if (k >= a_last) {
      dst = stash(k - a_last + 1);
    } else if (next_ck < nseg && k == seg_a(next_ck) - 1) {
      dst = ckpt(next_ck - 1);
      ++next_ck;
    } else {
      dst = s->S[k & 1];
      if (dst == prev) dst = s->S[(k + 1) & 1];
    }
    LBM_TRY(launch(s, prev, dst, k == 0 ? SF_COLLIDE_ONLY : 0, st));
    prev = dst;
  }
  if (!seed_f) {
    // the force of f_N (the pass writes no populations: dst null)
    LBM_TRY(launch(s, prev, nullptr, SF_STREAM_ONLY | SF_FORCE, st));
    LBM_TRY(cuda_check(launch_force_finalize(s->partials, s->nblocks, dyn_area(s), s->scal, st),
                       "force"));
    LBM_TRY(cuda_check(launch_dj_dfx(s->scal, dyn_area(s), s->scal + 4, st), "dJ/dFx"));
  } else {
    LBM_TRY(cuda_check(cudaMemsetAsync(s->scal, 0, 8 * sizeof(double), st), "memset"));
  }

  // ---- backward
  LBM_TRY(cuda_check(cudaMemsetAsync(s->gr_partials, 0, size_t(s->nblocks) * 16 * sizeof(double), st), "memset"));
  LBM_TRY(cuda_check(cudaMemsetAsync(s->gq, 0, size_t(s->gq_cap > 0 ? s->gq_cap : 1) * Q * sizeof(double), st), "memset"));
  int cur = 0;
  if (seed_f)
    LBM_TRY(adjoint_seed_dense(s, seed_f, s->nu[cur], st));
  else
    LBM_TRY(adjoint_seed(s, s->nu[cur], st));
  for (int c = nseg - 1; c >= 0; --c) {
    const int a0 = seg_a(c), b0 = seg_a(c + 1);
    const void* slot0 = a0 == 0 ? s->fbuf : ckpt(c - 1);
    if (c != nseg - 1) {
      const void* pv = slot0;
      for (int k = a0; k < b0; ++k) {
        void* dst = stash(k - a0 + 1);
        LBM_TRY(launch(s, pv, dst, k == 0 ? SF_COLLIDE_ONLY : 0, st));
        pv = dst;
      }
    }
    for (int k = b0 - 1; k >= a0; --k) {
      const void* Sprev = (k == a0) ? slot0 : stash(k - a0);
      LBM_TRY(adjoint_launch(s, Sprev, stash(k - a0 + 1), s->nu[cur], s->nu[1 - cur], k == 0,
                             k == N - 1 && !seed_f, st));
      cur = 1 - cur;
    }
  }
  LBM_TRY(cuda_check(launch_reduce_sum(s->gr_partials, s->nblocks * 16, s->scal + 5, st), "reduce"));
  if (dcd_dq) {
    cudaError_t e = is_fp64(s)
        ? launch_scatter_gq<double>(s->g, s->tag, s->rec, s->gq, static_cast<double*>(dcd_dq), st)
        : launch_scatter_gq<float>(s->g, s->tag, s->rec, s->gq, static_cast<float*>(dcd_dq), st);
    LBM_TRY(cuda_check(e, "scatter dq"));
  }
  if (dcd_df0)
    LBM_TRY(cuda_check(cudaMemcpyAsync(dcd_df0, s->nu[cur], s->n * Q * s->re_bytes,
                                       cudaMemcpyDeviceToDevice, st), "df0 copy"));
  double h[8];
  LBM_TRY(cuda_check(cudaMemcpyAsync(h, s->scal, 8 * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H"));
  LBM_TRY(cuda_check(cudaStreamSynchronize(st), "sync"));
  *cd_host = h[3];
  *dcd_dr_host = h[5];
  return LBM_OK;
}

}  // namespace

int lbm_cd_and_grad(lbm_sim* s, int n_steps, int checkpoint_every, double* cd_host,
                    double* dcd_dr_host, void* dcd_dq, void* dcd_df0, void* stream) {
  if (!s || !cd_host || !dcd_dr_host) return set_error(LBM_ERR_ARG, "lbm_cd_and_grad: null argument");
  if (n_steps < 1) return set_error(LBM_ERR_ARG, "lbm_cd_and_grad: n_steps < 1");
  if (!s->have_geometry) return set_error(LBM_ERR_STATE, "lbm_cd_and_grad: set a geometry first");
  if (s->state_is_S)
    return set_error(LBM_ERR_STATE, "lbm_cd_and_grad: needs the initial state; call lbm_set_state");
  if (s->p.guard != LBM_GUARD_OFF)
    return set_error(LBM_ERR_UNSUPPORTED,
                     "lbm_cd_and_grad: the stability guard is not differentiated (the reference "
                     "gradient drivers run without it)");
  LBM_TRY(check_align(dcd_dq, s->re_bytes, "dcd_dq"));
  LBM_TRY(check_align(dcd_df0, s->re_bytes, "dcd_df0"));
  return cd_and_grad_impl(s, n_steps, checkpoint_every, cd_host, dcd_dr_host, dcd_dq, dcd_df0,
                          static_cast<cudaStream_t>(stream), nullptr);
}

int lbm_vjp_run(lbm_sim* s, int n_steps, int checkpoint_every, const void* g_f_final,
                void* g_f0, void* g_q, void* stream) {
  if (!s || !g_f_final || !g_f0) return set_error(LBM_ERR_ARG, "lbm_vjp_run: null argument");
  if (n_steps < 1) return set_error(LBM_ERR_ARG, "lbm_vjp_run: n_steps < 1");
  if (!s->have_geometry) return set_error(LBM_ERR_STATE, "lbm_vjp_run: set a geometry first");
  if (s->state_is_S)
    return set_error(LBM_ERR_STATE, "lbm_vjp_run: needs the initial state; call lbm_set_state");
  if (s->porosity_mode == LBM_POROSITY_SOFT)
    return set_error(LBM_ERR_UNSUPPORTED,
                     "lbm_vjp_run: porosity blends are differentiated by lbm_cd_and_grad only");
  LBM_TRY(check_align(g_f_final, s->re_bytes, "g_f_final"));
  LBM_TRY(check_align(g_f0, s->re_bytes, "g_f0"));
  LBM_TRY(check_align(g_q, s->re_bytes, "g_q"));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool guarded = s->p.guard != LBM_GUARD_OFF;
  unsigned long long r0 = 0, r1 = 0;
  if (guarded) {
    LBM_TRY(cuda_check(cudaMemcpyAsync(&r0, s->guard_count, sizeof(r0), cudaMemcpyDeviceToHost,
                                       st), "guard D2H"));
    LBM_TRY(cuda_check(cudaStreamSynchronize(st), "sync"));
  }
  double cd = 0.0, gr = 0.0;
  LBM_TRY(cd_and_grad_impl(s, n_steps, checkpoint_every, &cd, &gr, g_q, g_f0, st, g_f_final));
  if (guarded) {
    LBM_TRY(cuda_check(cudaMemcpyAsync(&r1, s->guard_count, sizeof(r1), cudaMemcpyDeviceToHost,
                                       st), "guard D2H"));
    LBM_TRY(cuda_check(cudaStreamSynchronize(st), "sync"));
    if (r1 != r0)
      return set_error(LBM_ERR_UNSUPPORTED,
                       "lbm_vjp_run: the stability guard reset cells in these steps; the "
                       "gradient through a reset is not provided");
  }
  return LBM_OK;
}

int lbm_sphere_fields(int dtype, int nx, int ny, int nz, const lbm_sphere* sphere,
                      int32_t* solid, void* q, void* dqdr, void* porosity, void* stream) {
  if (!sphere || !q) return set_error(LBM_ERR_ARG, "lbm_sphere_fields: null argument");
  if (dtype != LBM_F32 && dtype != LBM_F64)
    return set_error(LBM_ERR_UNSUPPORTED, "lbm_sphere_fields: LBM_F32 or LBM_F64");
  if (nx < 1 || ny < 1 || nz < 1) return set_error(LBM_ERR_ARG, "lbm_sphere_fields: bad dims");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == LBM_F64)
    return sphere_fields_impl<double>(nx, ny, nz, sphere, solid, (double*)q, (double*)dqdr,
                                      (double*)porosity, st);
  return sphere_fields_impl<float>(nx, ny, nz, sphere, solid, (float*)q, (float*)dqdr,
                                   (float*)porosity, st);
}

int lbm_box_fields(int dtype, int nx, int ny, int nz, const double* corner_min,
                   const double* corner_max, int32_t* solid_out, void* q, void* stream) {
  if (!corner_min || !corner_max || !q || !solid_out)
    return set_error(LBM_ERR_ARG, "lbm_box_fields: null argument");
  if (dtype != LBM_F32 && dtype != LBM_F64)
    return set_error(LBM_ERR_UNSUPPORTED, "lbm_box_fields: LBM_F32 or LBM_F64");
  if (nx < 1 || ny < 1 || nz < 1) return set_error(LBM_ERR_ARG, "lbm_box_fields: bad dims");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Grid g = make_grid(nx, ny, nz, 1);
  uint8_t* solid = nullptr;
  LBM_TRY(dev_alloc((void**)&solid, size_t(g.n)));
  lbm_sphere none{};
  SphereSpec spec{};
  cudaError_t e = dtype == LBM_F64
      ? launch_box_fields<double>(g, corner_min, corner_max, solid, (double*)q, st)
      : launch_box_fields<float>(g, corner_min, corner_max, solid, (float*)q, st);
  int rc = cuda_check(e, "box fields");
  if (rc == LBM_OK) {
    e = dtype == LBM_F64
        ? launch_export_fields<double>(g, spec, 0, solid, solid_out, (double*)nullptr, st)
        : launch_export_fields<float>(g, spec, 0, solid, solid_out, (float*)nullptr, st);
    rc = cuda_check(e, "export");
  }
  (void)none;
  cudaStreamSynchronize(st);
  cudaFree(solid);
  return rc;
}

int lbm_q_from_solid(int dtype, const int32_t* solid_i32, double default_q, void* q, int nx,
                     int ny, int nz, void* stream) {
  if (!solid_i32 || !q) return set_error(LBM_ERR_ARG, "lbm_q_from_solid: null argument");
  if (dtype != LBM_F32 && dtype != LBM_F64)
    return set_error(LBM_ERR_UNSUPPORTED, "lbm_q_from_solid: LBM_F32 or LBM_F64");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Grid g = make_grid(nx, ny, nz, 1);
  uint8_t* solid = nullptr;
  LBM_TRY(dev_alloc((void**)&solid, size_t(g.n)));
  int rc = cuda_check(launch_solid_from_i32(g.n, solid_i32, solid, st), "solid");
  if (rc == LBM_OK) {
    cudaError_t e = dtype == LBM_F64 ? launch_q_from_solid<double>(g, solid, default_q, (double*)q, st)
                                     : launch_q_from_solid<float>(g, solid, default_q, (float*)q, st);
    rc = cuda_check(e, "q from solid");
  }
  cudaStreamSynchronize(st);
  cudaFree(solid);
  return rc;
}

int lbm_get_projected_area(lbm_sim* s, double* area_host) {
  if (!s || !area_host) return set_error(LBM_ERR_ARG, "lbm_get_projected_area: null argument");
  if (!s->have_geometry) return set_error(LBM_ERR_STATE, "lbm_get_projected_area: no geometry");
  *area_host = s->area;
  return LBM_OK;
}

int lbm_get_link_count(lbm_sim* s, int* links_host, int* special_host) {
  if (!s || !links_host || !special_host)
    return set_error(LBM_ERR_ARG, "lbm_get_link_count: null argument");
  *links_host = s->nlinks;
  *special_host = s->nrec;
  return LBM_OK;
}

int lbm_get_guard_resets(lbm_sim* s, unsigned long long* count_host, void* stream) {
  if (!s || !count_host) return set_error(LBM_ERR_ARG, "lbm_get_guard_resets: null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_TRY(cuda_check(cudaMemcpyAsync(count_host, s->guard_count, sizeof(unsigned long long),
                                     cudaMemcpyDeviceToHost, st),
                     "guard D2H"));
  return cuda_check(cudaStreamSynchronize(st), "sync");
}

int lbm_plan_checkpoints(int n_steps, long long max_states, int* segment_steps) {
  if (n_steps < 1 || !segment_steps)
    return set_error(LBM_ERR_ARG, "lbm_plan_checkpoints: n_steps < 1 or null segment_steps");
  return plan_segment(n_steps, max_states, 1, segment_steps);
}

int lbm_get_adjoint_plan(lbm_sim* s, int* segment_steps, int* recomputed_steps,
                         unsigned long long* workspace_bytes) {
  if (!s || !segment_steps || !recomputed_steps || !workspace_bytes)
    return set_error(LBM_ERR_ARG, "lbm_get_adjoint_plan: null argument");
  *segment_steps = s->plan_K;
  *recomputed_steps = s->plan_recompute;
  *workspace_bytes = (unsigned long long)s->plan_bytes;
  return LBM_OK;
}

int lbm_set_streaming(lbm_sim* s, int mode) {
  if (!s) return set_error(LBM_ERR_ARG, "lbm_set_streaming: null handle");
  if (mode != LBM_STREAM_AB && mode != LBM_STREAM_AA)
    return set_error(LBM_ERR_ARG, "lbm_set_streaming: mode must be LBM_STREAM_AB or LBM_STREAM_AA");
  if (mode == LBM_STREAM_AA &&
      (!s->g.periodic_yz || (s->p.storage != LBM_F32 && s->p.storage != LBM_F64)))
    return set_error(LBM_ERR_UNSUPPORTED,
                     "lbm_set_streaming: in-place streaming needs periodic y/z and FP32 or FP64 "
                     "storage");
  if (mode == (s->aa ? LBM_STREAM_AA : LBM_STREAM_AB)) return LBM_OK;
  s->aa = mode == LBM_STREAM_AA;
  // a running state's layout belongs to the old scheme: lbm_set_state first
  if (s->state_is_S) {
    s->state_is_S = 0;
    s->steps = 0;
    s->fbuf_step = -1;
    s->aa_needs_state = 1;
  }
  s->aa_layout_l = 0;
  s->sb_cur = 0;
  if (s->aa) {
    cudaFree(s->S[1]);     // one population buffer: the second is allocated again on demand
    s->S[1] = nullptr;
    s->cur = 0;
  }
  return LBM_OK;
}

int lbm_set_workspace_limit(lbm_sim* s, unsigned long long max_bytes) {
  if (!s) return set_error(LBM_ERR_ARG, "lbm_set_workspace_limit: null handle");
  s->workspace_limit = size_t(max_bytes);
  return LBM_OK;
}

int lbm_release_workspace(lbm_sim* s) {
  if (!s) return set_error(LBM_ERR_ARG, "lbm_release_workspace: null handle");
  cudaFree(s->states);
  s->states = nullptr;
  s->states_cap = 0;
  return LBM_OK;
}

int lbm_get_steps(lbm_sim* s, long long* steps_host) {
  if (!s || !steps_host) return set_error(LBM_ERR_ARG, "lbm_get_steps: null argument");
  *steps_host = s->steps;
  return LBM_OK;
}

}  // extern "C"
