/*
 * lbm_gb300.h -- C ABI of the GB300 (sm_103a) D3Q19 lattice-Boltzmann hot path.
 *
 * Drop-in boundary for jax_lbm (MarcosAsh/LBM_JAX_Autodiff).  The reference's
 * "operator API" is its set of pure JAX functions; each entry point below names
 * the function it replaces (file:line inside the reference project).  A host
 * binding (jax.ffi custom call, ctypes, a torch extension) passes device
 * pointers, sizes and a cudaStream_t; no framework types cross this boundary.
 *
 * Conventions
 *  - All array arguments are device pointers unless named *_host.
 *  - Populations use the reference layout [19][nx][ny][nz] (z fastest); fields
 *    [nx][ny][nz]; velocity [3][nx][ny][nz]; inlet faces [3][ny][nz].
 *  - dtype arguments take lbm_dtype; per-op kernels support LBM_F32/LBM_F64.
 *  - Every function returning int returns an lbm_status; LBM_OK = 0.
 *    lbm_last_error() gives a message for the last failure on the calling
 *    thread.  (The XLA targets return nothing; see their section.)
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *    asynchronous with respect to the host unless stated otherwise.
 *  - Outputs are distinct from inputs (the reference functions are pure).
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_GB300_API_VERSION 1

typedef enum {
  LBM_OK = 0,
  LBM_ERR_ARG = 1,         /* invalid argument (null pointer, bad size, bad enum) */
  LBM_ERR_ALIGN = 2,       /* pointer not aligned to its element size */
  LBM_ERR_UNSUPPORTED = 3, /* valid but unsupported combination */
  LBM_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  LBM_ERR_CUDA = 5,        /* CUDA runtime error */
  LBM_ERR_NOMEM = 6,       /* device allocation failed */
  LBM_ERR_STATE = 7        /* call not valid in the handle's current state */
} lbm_status;

typedef enum { LBM_F32 = 0, LBM_F64 = 1, LBM_F16 = 2, LBM_BF16 = 3 } lbm_dtype;
typedef enum { LBM_BGK = 0, LBM_MRT = 1 } lbm_collision;
typedef enum { LBM_GUARD_OFF = 0, LBM_GUARD_PRE = 1, LBM_GUARD_POST = 2 } lbm_guard;
typedef enum { LBM_POROSITY_NONE = 0, LBM_POROSITY_HARD = 1, LBM_POROSITY_SOFT = 2 } lbm_porosity;
typedef enum { LBM_Q_HALFWAY = 0, LBM_Q_BOUZIDI = 1 } lbm_qmode;
typedef enum { LBM_SPHERE_DIST_MASK = 0, LBM_SPHERE_SIGMOID_MASK = 1 } lbm_sphere_kind;
typedef enum { LBM_STREAM_AB = 0, LBM_STREAM_AA = 1 } lbm_streaming;

/* Solver configuration; mirrors jax_lbm LBMParams (state.py:57-84) plus the
 * storage precision and the driver-level options of the examples. */
typedef struct lbm_params {
  int nx, ny, nz;
  int storage;             /* lbm_dtype of the stored populations */
  int collision;           /* lbm_collision      (LBMParams.collision_mode) */
  double tau;              /*                    (LBMParams.tau) */
  int use_smagorinsky;     /*                    (LBMParams.use_smagorinsky) */
  double smagorinsky_cs;   /*                    (LBMParams.smagorinsky_cs) */
  int periodic_yz;         /*                    (LBMParams.periodic_yz) */
  int guard;               /* lbm_guard: state.py:161-169 (POST) or examples/10:163-168 (PRE) */
  double inlet_velocity[3];/*                    (LBMParams.inlet_velocity) */
  double rho_out;          /* zou_he_outlet rho_out (boundary.py:127) */
  double u_ref;            /* velocity in Cd = |Fx| / (0.5 rho U^2 A + 1e-10) */
  double area_min;         /* A = max(projected_area, area_min) (examples/11:164) */
  int exact_constants;     /* 0: float32-rounded weights/MRT rates like lattice.py; 1: exact */
} lbm_params;

/* Sphere obstacle in the reference world frame x in [-4,4], y,z in [-2,2]
 * (primitives.py:26-53). */
typedef struct lbm_sphere {
  double center[3];
  double radius;
  double sharpness;        /* sigmoid alpha (smooth.py:81) */
  int kind;                /* lbm_sphere_kind: mask by dist^2 <= r^2 (primitives.py:112)
                              or sigmoid > 0.5 (smooth.py:201, examples/11:62) */
  int q_mode;              /* lbm_qmode (examples/11:87-104) */
  int porosity;            /* lbm_porosity (examples/11:64-67) */
  double disc_floor;       /* sqrt(max(disc, floor)): 0 (primitives.py:162), 1e-10 (smooth.py:236) */
  double denom_eps;        /* t = (-b - sqrt)/(2a + eps): 1e-20 (primitives.py:163) */
} lbm_sphere;

typedef struct lbm_sim lbm_sim;

/* ---- library ------------------------------------------------------------ */
int lbm_api_version(void);
const char* lbm_status_string(int status);
const char* lbm_last_error(void);
/* sizeof the ABI's structs, for bindings that restate them (ctypes, cgo, a
 * JNI shim) to check their layout against: which = 0 lbm_params, 1
 * lbm_sphere, 2 lbm_xla_desc, 3 lbm_xla_fused_desc, 4 lbm_adam; 0 for any
 * other code. */
size_t lbm_struct_size(int which);

/* ---- fused solver handle (replaces state.py:87-230 and the examples' -----
 * ---- step_fn / lax.scan loops, e.g. examples/10:162-193) ------------------ */

/* Allocate a solver for params->nx*ny*nz cells.  Owns its device memory. */
int lbm_create(const lbm_params* params, lbm_sim** out);
int lbm_destroy(lbm_sim* sim);

/* Sphere geometry: solid mask, ray-sphere q(r), dq/dr, projected area
 * (primitives.py:56-174, smooth.py:158-248, examples/11:56-119, forces.py:199). */
int lbm_set_geometry_sphere(lbm_sim* sim, const lbm_sphere* sphere, void* stream);

/* Mask geometry: solid int32 [n] (0 fluid, 1 body, 2 ground: state.py:41-44);
 * q [19][n] in the solver's compute dtype, or NULL for compute_q_from_solid(
 * default_q) (bouzidi.py:32-106); porosity [n] (compute dtype) or NULL for a
 * hard mask. */
int lbm_set_geometry_mask(lbm_sim* sim, const int32_t* solid, const void* q, double default_q,
                          const void* porosity, void* stream);

/* Per-(y,z) inlet velocity [3][ny][nz] (compute dtype); NULL = uniform
 * params->inlet_velocity (zou_he_inlet's broadcasting, boundary.py:95-122). */
int lbm_set_inlet_profile(lbm_sim* sim, const void* u_face, void* stream);

/* State f [19][n] in the compute dtype (f32 for F32/F16/BF16 storage, f64 for F64).
 * set: the state after 0 steps; get: the reference's f after the steps run so far. */
int lbm_set_state(lbm_sim* sim, const void* f, void* stream);
int lbm_get_state(lbm_sim* sim, void* f, void* stream);
/* The same with f in host memory (pinned for an asynchronous copy): one
 * cudaMemcpyAsync straight between the host buffer and the handle's own f
 * buffer, no device staging by the caller.  get: when the last lbm_run call
 * sampled its final step, that sample pass already left f in the handle and
 * the copy is all that runs; otherwise one stream-only pass writes it first.
 * For drivers that keep the state on the host between chunks of steps, as
 * the reference's examples do every sampling interval (examples/10:93-97). */
int lbm_set_state_host(lbm_sim* sim, const void* f_host, void* stream);
int lbm_get_state_host(lbm_sim* sim, void* f_host, void* stream);

/* lbm_get_state into the device buffer f, then one step (lbm_run with
 * n_steps 1, no samples), in one launch that reads the state once: the step's
 * pull writes the reference f it forms (after the post-BC guard) besides the
 * next state.  For a driver that holds f between single steps, as state.py's
 * step() does (state.py:87-171): f of step k out, the handle at step k + 1.
 * Falls back to the two calls when there is nothing to fuse (a state just
 * set, f already written by a sample pass, in-place streaming). */
int lbm_get_state_and_step(lbm_sim* sim, void* f, void* stream);

/* Streaming scheme of lbm_run / lbm_get_state (the states they produce are
 * the same):
 *  - LBM_STREAM_AB (default): two population buffers, read one, write the
 *    other;
 *  - LBM_STREAM_AA: one buffer updated in place, its layout alternating
 *    between steps; the boundary cells keep their post-collision vector in a
 *    small side buffer (records + x faces).  Halves the state's memory for
 *    forward runs (the second buffer is released, and allocated again if
 *    lbm_cd_and_grad needs it).  Periodic y/z, FP32 or FP64 storage.
 * The pull of streaming.py:109-142 either way.  Switching with a running
 * state discards it (LBM_ERR_STATE from lbm_run until lbm_set_state), and so
 * does a geometry change under an AA state. */
int lbm_set_streaming(lbm_sim* sim, int mode);

/* Advance n_steps.  If sample_every > 0, after every sample_every-th step of
 * this call the momentum-exchange force and Cd are written to
 * samples[4*s .. 4*s+3] = (Fx, Fy, Fz, Cd) (device doubles), computed from the
 * last post-collision populations and the post-BC state exactly as
 * momentum_exchange(f_post, f, q) + drag_coefficient (forces.py:37-120,237-276). */
int lbm_run(lbm_sim* sim, int n_steps, int sample_every, double* samples, void* stream);

/* Shape gradient: from the state set by lbm_set_state, run n_steps and return
 * Cd = drag_coefficient(momentum_exchange(f_post_last, f_final, q)) and its
 * derivative with respect to the sphere radius (through the ray-sphere q(r)
 * and the sigmoid porosity), as jax.grad of the reference drivers'
 * simulate_cd (examples/11:139-176, examples/08:69-93, tests/
 * test_gradients_f64.py:154-207).  The hand-written adjoint runs backwards
 * with the populations of the last `checkpoint_every` steps kept from the
 * forward pass and earlier segments of that length recomputed from
 * checkpoints (examples/08:49-66 does the same with jax.checkpoint);
 * checkpoint_every <= 0 picks the longest segment that fits in free HBM.
 * The adjoint workspace is kept in the handle between calls.  Optional outputs (device, compute dtype, NULL to
 * skip): dcd_dq [19][n] = dCd/dq on every link, dcd_df0 [19][n] = dCd/df_0.
 * Requires guard = LBM_GUARD_OFF.  Synchronises `stream`. */
int lbm_cd_and_grad(lbm_sim* sim, int n_steps, int checkpoint_every, double* cd_host,
                    double* dcd_dr_host, void* dcd_dq, void* dcd_df0, void* stream);

/* Vector-Jacobian product of n_steps of lbm_run from the state set by
 * lbm_set_state: given g_f_final [19][n] (compute dtype), the cotangent of
 * the reference f after the steps, writes g_f0 [19][n] = its cotangent on
 * the initial f and, if g_q is not NULL, g_q [19][n] = its cotangent on the
 * wall distances q of the geometry (zero where there is no link): the
 * gradient jax.grad takes through simulate (state.py:174-230) with respect
 * to state.f and state.q.  Forward with checkpoints and recompute as
 * lbm_cd_and_grad.  Hard-mask geometries only (LBMState has no porosity).
 * The guard is not differentiated: with a guard on, LBM_ERR_UNSUPPORTED if
 * it reset any cell in these steps (where no cell is reset the gradient is
 * that of the unguarded step).  Synchronises `stream`. */
int lbm_vjp_run(lbm_sim* sim, int n_steps, int checkpoint_every, const void* g_f_final,
                void* g_f0, void* g_q, void* stream);

/* The checkpoint plan the automatic setting (checkpoint_every <= 0) makes
 * for n_steps when max_states population states fit: the longest segment K
 * with ceil(n_steps / K) - 1 + K <= max_states (n_steps - K steps are then
 * recomputed).  LBM_ERR_NOMEM when no K fits.  No GPU call. */
int lbm_plan_checkpoints(int n_steps, long long max_states, int* segment_steps);

/* Plan of the last lbm_cd_and_grad: segment length, recomputed steps and
 * the bytes of the population workspace (checkpoints + stash). */
int lbm_get_adjoint_plan(lbm_sim* sim, int* segment_steps, int* recomputed_steps,
                         unsigned long long* workspace_bytes);
/* Free the adjoint population workspace. */
int lbm_release_workspace(lbm_sim* sim);
/* Cap, in bytes, on the population workspace (checkpoints + stash) that the
 * automatic plan (checkpoint_every <= 0) may take; 0 (the default) lets it
 * use the free device memory minus a reserve of 2 GiB + 2 % of the device.
 * For a library sharing the device with a framework that holds a memory
 * pool (JAX preallocates 75 % of the device, torch caches freed blocks).
 * A cap below the smallest workspace, ceil(N/K) - 1 + K states at
 * K ~ sqrt(N), makes lbm_cd_and_grad fail with LBM_ERR_NOMEM.  Counterpart
 * of jax.checkpoint's memory/recompute trade-off (examples/08:49-66). */
int lbm_set_workspace_limit(lbm_sim* sim, unsigned long long max_bytes);

/* Host-side queries (synchronise `stream`). */
int lbm_get_projected_area(lbm_sim* sim, double* area_host);
int lbm_get_link_count(lbm_sim* sim, int* links_host, int* special_cells_host);
int lbm_get_guard_resets(lbm_sim* sim, unsigned long long* count_host, void* stream);
int lbm_get_steps(lbm_sim* sim, long long* steps_host);

/* ---- geometry builders (jax_lbm.geometry), dense outputs -------------------
 * Synchronise `stream`.  dtype LBM_F32 / LBM_F64 for q, dqdr, porosity. */
/* solid [n] int32 (may be NULL), q [19][n], dq/dr [19][n] (may be NULL), porosity [n]
 * (may be NULL: sigmoid field for porosity = SOFT, else the 0/1 mask)
 * create_sphere (primitives.py:56-174), smooth_sphere_geometry (smooth.py:158-248),
 * examples/11:56-119 */
int lbm_sphere_fields(int dtype, int nx, int ny, int nz, const lbm_sphere* sphere,
                      int32_t* solid, void* q, void* dqdr, void* porosity, void* stream);
/* create_box: solid inside the world AABB, q = 0.5 on links (primitives.py:177-255) */
int lbm_box_fields(int dtype, int nx, int ny, int nz, const double* corner_min,
                   const double* corner_max, int32_t* solid, void* q, void* stream);
/* compute_q_from_solid (bouzidi.py:32-106) */
int lbm_q_from_solid(int dtype, const int32_t* solid, double default_q, void* q, int nx, int ny,
                     int nz, void* stream);

/* ---- per-op drop-ins (jax_lbm.core) --------------------------------------
 * One launch per reference function; dtype is LBM_F32 or LBM_F64, every array
 * a device pointer in the reference layout, outputs distinct from inputs.
 * `flags`: LBM_OP_EXACT_CONSTANTS uses the exact rational weights / MRT rates
 * instead of the reference's float32-rounded ones (lattice.py:53-60,106-126).
 * `tau_field` may be NULL (scalar `tau`) or a per-cell [n] field.
 * The *_vjp entry points are the vector-Jacobian products jax.grad derives for
 * the same functions; g_* inputs are cotangents of the outputs. */
#define LBM_OP_EXACT_CONSTANTS 1

/* rho = sum_i f_i                         equilibrium.py:22-48 */
int lbm_compute_density(int dtype, const void* f, void* rho, int nx, int ny, int nz, void* stream);
/* u = sum_i f_i e_i / rho                 equilibrium.py:51-87 */
int lbm_compute_velocity(int dtype, const void* f, const void* rho, void* u, int nx, int ny,
                         int nz, void* stream);
/* f_eq(rho, u)                            equilibrium.py:90-151 */
int lbm_equilibrium(int dtype, const void* rho, const void* u, void* feq, int nx, int ny, int nz,
                    int flags, void* stream);
/* f - (f - f_eq) / tau                    collision.py:46-100 */
int lbm_bgk(int dtype, const void* f, const void* tau_field, double tau, void* out, int nx,
            int ny, int nz, int flags, void* stream);
/* MRT collision                           collision.py:103-184 */
int lbm_mrt(int dtype, const void* f, const void* tau_field, double tau, void* out, int nx,
            int ny, int nz, int flags, void* stream);
/* Smagorinsky tau_eff field               collision.py:187-270 */
int lbm_smagorinsky_tau(int dtype, const void* f, double tau, double cs, void* tau_eff, int nx,
                        int ny, int nz, int flags, void* stream);
/* (1 - p) f + p f[opp]                    smooth.py:118-155 */
int lbm_soft_bounce_back(int dtype, const void* f, const void* porosity, void* out, int nx,
                         int ny, int nz, void* stream);
/* pull streaming + Bouzidi, dense q [19][n] streaming.py:40-185 */
int lbm_stream(int dtype, const void* f, const void* q, int periodic_yz, void* out, int nx, int ny,
               int nz, void* stream);
/* Zou-He velocity inlet at x = 0          boundary.py:35-124.  Velocity: u_face [3][ny][nz]
 * (device, dtype) or, if NULL, velocity[3] (host doubles); rho_target used when has_rho_target. */
int lbm_zou_he_inlet(int dtype, const void* f, const void* u_face, const double* velocity,
                     int has_rho_target, double rho_target, void* out, int nx, int ny, int nz,
                     void* stream);
/* Zou-He pressure outlet at x = nx-1      boundary.py:127-200 */
int lbm_zou_he_outlet(int dtype, const void* f, double rho_out, void* out, int nx, int ny, int nz,
                      void* stream);
/* F = sum over links of e_i (f*_i + f_opp) into force[3] (device doubles)  forces.py:37-120.
 * Uses a per-block partial-sum scratch from cudaMallocAsync on `stream`. */
int lbm_momentum_exchange(int dtype, const void* f_post, const void* f_streamed, const void* q,
                          double* force, int nx, int ny, int nz, void* stream);
/* Cd = |Fx| / (0.5 rho U^2 A + 1e-10) into cd[1] (device)  forces.py:237-276 */
int lbm_drag_coefficient(const double* force, double inlet_velocity, double area, double rho,
                         double* cd, void* stream);
/* number of columns along `axis` holding a body cell (solid == 1) into area[1]  forces.py:199-234 */
int lbm_projected_area(const int32_t* solid, int axis, double* area, int nx, int ny, int nz,
                       void* stream);

int lbm_compute_density_vjp(int dtype, const void* g_rho, void* g_f, int nx, int ny, int nz,
                            void* stream);
int lbm_compute_velocity_vjp(int dtype, const void* f, const void* rho, const void* g_u,
                             void* g_f, void* g_rho, int nx, int ny, int nz, void* stream);
int lbm_equilibrium_vjp(int dtype, const void* rho, const void* u, const void* g_feq, void* g_rho,
                        void* g_u, int nx, int ny, int nz, int flags, void* stream);
/* g_tau: per-cell cotangent of tau (NULL to skip) */
int lbm_bgk_vjp(int dtype, const void* f, const void* tau_field, double tau, const void* g_out,
                void* g_f, void* g_tau, int nx, int ny, int nz, int flags, void* stream);
int lbm_mrt_vjp(int dtype, const void* f, const void* tau_field, double tau, const void* g_out,
                void* g_f, void* g_tau, int nx, int ny, int nz, int flags, void* stream);
/* jax.grad of sqrt at Pi = 0 is NaN; this returns the subgradient 0 there */
int lbm_smagorinsky_tau_vjp(int dtype, const void* f, double tau, double cs,
                            const void* g_tau_eff, void* g_f, void* g_tau, int nx, int ny, int nz,
                            int flags, void* stream);
int lbm_soft_bounce_back_vjp(int dtype, const void* f, const void* porosity, const void* g_out,
                             void* g_f, void* g_porosity, int nx, int ny, int nz, void* stream);
/* g_q (NULL to skip): cotangent of the dense q, non-zero only on links */
int lbm_stream_vjp(int dtype, const void* f, const void* q, int periodic_yz, const void* g_out,
                   void* g_f, void* g_q, int nx, int ny, int nz, void* stream);
/* g_u_face (NULL to skip): [3][ny][nz] cotangent of the inlet velocity */
int lbm_zou_he_inlet_vjp(int dtype, const void* f, const void* u_face, const double* velocity,
                         int has_rho_target, double rho_target, const void* g_out, void* g_f,
                         void* g_u_face, int nx, int ny, int nz, void* stream);
/* g_rho_out_face (NULL to skip): [ny][nz] per-face-cell cotangent of rho_out */
int lbm_zou_he_outlet_vjp(int dtype, const void* f, double rho_out, const void* g_out, void* g_f,
                          void* g_rho_out_face, int nx, int ny, int nz, void* stream);
/* g_force: device doubles [3] */
int lbm_momentum_exchange_vjp(int dtype, const void* q, const double* g_force, void* g_f_post,
                              void* g_f_streamed, int nx, int ny, int nz, void* stream);

/* Same result as lbm_momentum_exchange, but allocates no device memory: for
 * callers that may not allocate inside a library call -- code running in a
 * framework that owns all device memory (e.g. an XLA custom call without a
 * workspace) or under a fixed memory budget.  No counterpart in the
 * reference.  The partial sums go to a fixed 1.5 MiB array compiled into the
 * library, which every GPU that loads the library keeps until exit.
 *  - Grids of at most 16,777,216 cells; larger ones return LBM_ERR_UNSUPPORTED.
 *  - The first call on a device looks up that array's device address
 *    (cudaGetSymbolAddress, with that device current), and so does the first
 *    call after the device's context was torn down and created again (e.g.
 *    cudaDeviceReset), which moves the array; make such a first call before
 *    any stream capture.
 *  - All calls on a device share the array: calls that overlap on the GPU
 *    (concurrent streams or threads) race and must be serialised.  Each call
 *    writes every partial it reads, so nothing needs clearing in between. */
int lbm_momentum_exchange_noalloc(int dtype, const void* f_post, const void* f_streamed,
                                  const void* q, double* force, int nx, int ny, int nz,
                                  void* stream);

/* ---- XLA custom-call targets (jax.ffi, legacy api_version = 0) ------------
 * Signature: void target(cudaStream_t stream, void** buffers, const char* opaque,
 * size_t opaque_len); buffers are the operands followed by the results, in the
 * order of the matching lbm_* entry point above; opaque is one lbm_xla_desc,
 * either as raw bytes or as the text "lbm1 nx ny nz dtype flags periodic_yz
 * tau_field u_face has_rho_target tau cs u0 u1 u2 rho" (doubles in C99 hex).
 * The legacy API has no status: failures are printed to stderr. */
typedef struct lbm_xla_desc {
  int32_t nx, ny, nz;
  int32_t dtype;          /* LBM_F32 / LBM_F64 */
  int32_t flags;          /* LBM_OP_EXACT_CONSTANTS */
  int32_t periodic_yz;
  int32_t tau_field;      /* 1: a per-cell tau operand follows f */
  int32_t u_face;         /* 1: a [3][ny][nz] inlet-velocity operand follows f */
  int32_t has_rho_target;
  int32_t pad;
  double tau;
  double cs;
  double u[3];
  double rho;             /* rho_target (inlet) or rho_out (outlet) */
} lbm_xla_desc;

void lbm_xla_compute_density(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_compute_velocity(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_equilibrium(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_bgk(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_mrt(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_smagorinsky_tau(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_soft_bounce_back(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_stream(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_zou_he_inlet(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_zou_he_outlet(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_momentum_exchange(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_compute_density_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_compute_velocity_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_equilibrium_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_bgk_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_mrt_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_smagorinsky_tau_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_soft_bounce_back_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_stream_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_zou_he_inlet_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_zou_he_outlet_vjp(void* stream, void** buffers, const char* opaque, size_t len);
void lbm_xla_momentum_exchange_vjp(void* stream, void** buffers, const char* opaque, size_t len);

/* ---- XLA custom-call targets of the fused solver --------------------------
 * Same legacy signature; opaque is one lbm_xla_fused_desc (raw bytes).  They
 * replace a jitted driver's whole loop: lbm_xla_run the lax.scan of
 * examples/10:69-106 (n_steps with the Cd sampled every sample_every steps),
 * lbm_xla_cd_and_grad the value_and_grad(simulate_cd) of examples/11:139-176.
 * The library keeps one solver handle per (device, params) for them, created
 * on first use; at most 8 are kept, the least recently used one that no call
 * is using being destroyed for a new parameter set.  The sphere geometry
 * (radius from the operand) is rebuilt when it changes, which reads the
 * radius back to the host (a stream synchronisation).  The last result of each is an int32
 * status (lbm_status): on failure it is non-zero, the other results are
 * filled with NaN and the message goes to stderr. */
typedef struct lbm_xla_fused_desc {
  lbm_params params;
  lbm_sphere sphere;      /* its radius is replaced by the radius operand */
  int32_t n_steps;
  int32_t sample_every;   /* lbm_xla_run: 0 = no samples (one zero row written) */
  int32_t checkpoint_every;
  int32_t pad;
} lbm_xla_fused_desc;

/* operands: f0 [19][n] (compute dtype), radius f64[1];
 * results: f [19][n] after n_steps, samples f64[max(1, n_steps / sample_every)][4]
 * (Fx, Fy, Fz, Cd), status int32[1] */
void lbm_xla_run(void* stream, void** buffers, const char* opaque, size_t len);
/* operands: f0 [19][n] (compute dtype), radius f64[1];
 * results: cd f64[1], dcd_dr f64[1], dcd_dq [19][n] (compute dtype), status int32[1] */
void lbm_xla_cd_and_grad(void* stream, void** buffers, const char* opaque, size_t len);

/* ---- batched instances --------------------------------------------------
 * Many independent sphere instances -- grids of different sizes, their own
 * radius, q mode, porosity mode and sigmoid sharpness -- advanced by one kernel
 * launch per step over all of them.  A gradient evaluation (forward with
 * checkpoints, recompute, adjoint) and the optimiser step on every radius can
 * run as one captured CUDA graph.  jax_lbm has no batched driver (its examples
 * loop over configurations in Python, examples/11:197-225); these entry points
 * have no counterpart there.  Instances use LBM_F32 storage and share the
 * collision model and guard setting. */
typedef struct lbm_batch lbm_batch;

enum { LBM_LOSS_CD = 0, LBM_LOSS_TARGET_CD = 1 };

/* optax.adam on the radius, then clip to [r_min, r_max] (examples/11:182-194).
 * loss LBM_LOSS_CD minimises Cd (optim/losses.py minimize_cd_loss);
 * LBM_LOSS_TARGET_CD minimises (Cd - target_cd)^2 (target_cd_loss). */
typedef struct lbm_adam {
  double lr;
  double b1, b2, eps; /* optax defaults: 0.9, 0.999, 1e-8 */
  double r_min, r_max;
  int loss;
  double target_cd;
} lbm_adam;

int lbm_batch_create(const lbm_params* params, int count, lbm_batch** out);
int lbm_batch_destroy(lbm_batch* batch);
int lbm_batch_size(lbm_batch* batch, int* count, long long* cells);
/* The solver handle of instance i (owned by the batch), for per-instance
 * queries such as lbm_get_state or lbm_get_projected_area. */
int lbm_batch_instance(lbm_batch* batch, int i, lbm_sim** sim);
/* One sphere per instance (spheres[count]); rebuilds each instance's geometry. */
int lbm_batch_set_spheres(lbm_batch* batch, const lbm_sphere* spheres, void* stream);
/* f_0 = f_eq(rho = 1, u = (inlet_velocity[0], 0, 0)) on every instance. */
int lbm_batch_set_equilibrium(lbm_batch* batch, void* stream);
int lbm_batch_set_state(lbm_batch* batch, int i, const void* f, void* stream);
/* Advance every instance n_steps.  With sample_every > 0, samples (device,
 * float64) receives [n_steps / sample_every][count][4] = (Fx, Fy, Fz, Cd). */
int lbm_batched_run(lbm_batch* batch, int n_steps, int sample_every, double* samples,
                    void* stream);
/* Cd after n_steps and dCd/dr of every instance (host arrays [count]), from
 * the initial state; checkpoint_every 0 picks the segment length from free
 * device memory.  use_graph runs the evaluation as a captured CUDA graph
 * (captured on first use, replayed while n_steps, the segment length and the
 * block size stay the same). */
int lbm_batch_cd_and_grad(lbm_batch* batch, int n_steps, int checkpoint_every, int use_graph,
                          double* cd_host, double* dcd_dr_host, void* stream);
/* n_iters optimisation iterations: gradient evaluation + Adam step on every
 * radius (on the device, inside the graph with use_graph), then the geometry
 * of the new radii.  Host histories [n_iters][count] (any may be NULL): the
 * radius evaluated, the loss, Cd and dloss/dr. */
int lbm_batch_optimize(lbm_batch* batch, int n_iters, int n_steps, int checkpoint_every,
                       const lbm_adam* opt, int use_graph, double* r_hist, double* loss_hist,
                       double* cd_hist, double* grad_hist, void* stream);
int lbm_batch_get_radii(lbm_batch* batch, double* radii_host);
/* Threads per block of the batched kernels: 128 or 256. */
int lbm_batch_set_block(lbm_batch* batch, int block);
/* Times a probe_steps gradient evaluation at each block size and keeps the
 * faster; sets the checkpoint interval for n_steps to the longest segment the
 * free device memory holds.  Returns both. */
int lbm_batch_autotune(lbm_batch* batch, int probe_steps, int n_steps, int* block_out,
                       int* checkpoint_out, void* stream);
int lbm_batch_get_plan(lbm_batch* batch, int* block, int* segment_steps, int* recomputed_steps,
                       unsigned long long* workspace_bytes, double* graph_build_seconds);
/* Cap, in bytes, on the population workspace of all instances together
 * under the automatic plan (checkpoint_every 0, lbm_batch_autotune); 0 = no
 * cap.  As lbm_set_workspace_limit. */
int lbm_batch_set_workspace_limit(lbm_batch* batch, unsigned long long max_bytes);
/* Kernel launches (graph nodes) of the last captured gradient evaluation
 * (0 before the first capture). */
int lbm_batch_graph_launches(lbm_batch* batch, long long* launches);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
