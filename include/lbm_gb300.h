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
 *  - Every function returns an lbm_status; LBM_OK = 0.  lbm_last_error() gives
 *    a message for the last failure on the calling thread.
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
 * with populations checkpointed every `checkpoint_every` steps (<= 0: store
 * every step) and recomputed segment by segment (examples/08:49-66 does the
 * same with jax.checkpoint).  Optional outputs (device, compute dtype, NULL to
 * skip): dcd_dq [19][n] = dCd/dq on every link, dcd_df0 [19][n] = dCd/df_0.
 * Requires guard = LBM_GUARD_OFF.  Synchronises `stream`. */
int lbm_cd_and_grad(lbm_sim* sim, int n_steps, int checkpoint_every, double* cd_host,
                    double* dcd_dr_host, void* dcd_dq, void* dcd_df0, void* stream);

/* Host-side queries (synchronise `stream`). */
int lbm_get_projected_area(lbm_sim* sim, double* area_host);
int lbm_get_link_count(lbm_sim* sim, int* links_host, int* special_cells_host);
int lbm_get_guard_resets(lbm_sim* sim, unsigned long long* count_host, void* stream);
int lbm_get_steps(lbm_sim* sim, long long* steps_host);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
