/*
 * merc.h - C ABI of the GB300 Mercurius integrator (libmerc.so).
 *
 * The reference (at2005/p9-integrator) has no library interface: its only
 * boundary is the `mint` executable, which launches one CUDA kernel per batch
 * of steps:
 *   mercurius_solver(double* omega, M, e, a, i, Omega, double* m,
 *                    double3* out_pos, int Nm, int batch, double dt)
 *     src/sim.cuh:615-625, launched from src/mercurius.cu:184-196.
 * Every entry point below replaces one piece of that launch sequence so the
 * drop-in `mint` CLI (and any FFI caller: ctypes, cgo, JNI) drives the GPU
 * through plain pointers and sizes.  No torch or CUDA types cross this ABI.
 *
 * Conventions
 *  - Every function returns an int status: MERC_OK (0) or a MERC_ERR_* code;
 *    merc_last_error(ctx) returns a message for the last failure.
 *  - Host buffers are owned by the caller and only read/written during the
 *    call.  Device buffers are owned by the context.
 *  - One context per host thread; a context is bound to one GPU.
 *  - Units: G = 1, M_sun = 1 (implicit, at the origin, not in the body list),
 *    AU, yr (reference README.md:2).  All state is IEEE binary64.
 *  - Bodies of a system are ordered massive first; the first n_massive bodies
 *    are the gravitating sources (reference src/mercurius.cu:4-15 counts them,
 *    src/sim.cuh:339 loops over the first Nm).
 *  - Arrays of a batch of systems are concatenated body-wise:
 *    system s owns bodies [body_offset[s], body_offset[s+1]).
 *  - Position/velocity arrays are structure-of-arrays, component-major:
 *    pos[c * n_total + j] for component c in {x, y, z} of body j.
 */
#ifndef MERC_H
#define MERC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MERC_OK 0
#define MERC_ERR_CONFIG 1   /* invalid argument, size or parameter */
#define MERC_ERR_CUDA 2     /* CUDA runtime error (message has details) */
#define MERC_ERR_TIMEOUT 3  /* a bounded device wait gave up */
#define MERC_ERR_NONCONV 4  /* a Kepler solve hit its iteration cap */
#define MERC_ERR_STATE 5    /* call out of order (e.g. step before load) */

/* drift formulations */
#define MERC_DRIFT_ELEMENTS 0  /* reference: cartesian->elements, M += n dt, Danby, back */
#define MERC_DRIFT_UNIVERSAL 1 /* universal-variable (Stumpff) f and g solve */

/* warm start of the universal-variable solve */
#define MERC_WARM_PLAIN 0  /* s0 = dt / r0 */
#define MERC_WARM_MLP 1    /* FP32 MLP guess for long drifts (dt / r0^1.5 >= 0.03), else the series guess; same FP64 Newton */
#define MERC_WARM_SERIES 2 /* the Kepler equation inverted to third order in dt (default) */

/* per-body flags (uint32) */
#define MERC_FLAG_CE_LAST 1u   /* close encounter detected in the most recent step */
#define MERC_FLAG_CE_EVER 2u   /* close encounter detected in any step since load */
#define MERC_FLAG_EJECTED 4u   /* heliocentric distance exceeded eject_r (sticky) */
#define MERC_FLAG_NONFINITE 8u /* position or velocity became NaN/inf (sticky) */
#define MERC_FLAG_MERGED 16u   /* absorbed in a physical collision and parked (sticky; merc_set_radii) */
#define MERC_FLAG_GREW 32u     /* absorbed another body in a physical collision (sticky) */

/* Integration parameters.  Defaults (merc_default_params) are the
 * reference's compile-time constants (src/constants.cuh:4-11) and its
 * hard-coded dt (src/mercurius.cu:43). */
typedef struct merc_params {
  double dt;            /* step, yr                          (ref 0.8219) */
  double softening2;    /* epsilon^2 of the pair/Sun forces  (ref 1e-8, constants.cuh:8) */
  double hill_factor;   /* r_crit = hill_factor * Hill radius of the source (ref 1) */
  double kepler_tol;    /* universal solve: stop when the Newton error estimate of s is <= tol*|s| (ref CUTOFF 1e-13) */
  double eject_r;       /* flag bodies beyond this distance; 0 = off */
  int32_t kepler_iters; /* Danby iterations, element drift (ref 8, constants.cuh:4) */
  int32_t bs_rows;      /* Richardson rows of the encounter sub-stepper (ref 3, constants.cuh:10), 1..4 */
  int32_t compat_block; /* 0: a body excludes itself by its index in the system.
                           B > 0: reproduce the reference, which compares the source
                           index with threadIdx.x = index % B (sim.cuh:172-175,364,608) */
  int32_t drift;        /* MERC_DRIFT_* */
  int32_t kepler_max_iter; /* universal solve iteration cap (>= 1) */
  int32_t warm_start;   /* MERC_WARM_* */
} merc_params;

typedef struct merc_stats {
  int64_t steps_done;        /* steps integrated since load */
  int64_t ce_body_steps;     /* sum over steps of bodies in close encounter */
  int64_t kepler_iterations; /* universal drift: Newton iterations summed over bodies */
  int64_t kepler_solves;     /* universal drift: number of solves */
  int64_t kepler_nonconverged; /* universal drift: solves that hit the cap */
  int64_t n_bodies;          /* total bodies loaded (all systems) */
  int64_t n_systems;
  double last_step_ms;       /* device time of the last merc_step call */
  int64_t kepler_simt_iterations; /* universal drift: iterations executed, per solve the most that any
                                     solve of its warp took (the SIMT cost of the Newton loop) */
} merc_stats;

typedef struct merc_ctx merc_ctx;

/* Fill *p with the reference defaults. */
void merc_default_params(merc_params* p);

/* Create a context on CUDA device `device`.  Replaces cudaSetDevice +
 * launch configuration, reference src/mercurius.cu:36,45-69. */
int merc_create(int device, const merc_params* p, merc_ctx** out);
int merc_destroy(merc_ctx* ctx);
const char* merc_last_error(const merc_ctx* ctx);
int merc_set_params(merc_ctx* ctx, const merc_params* p);

/* Load systems from orbital elements.  Replaces the host staging of the
 * element arrays (src/mercurius.cu:73-164) and the kernel prologue that turns
 * them into heliocentric positions and democratic-heliocentric velocities
 * (src/sim.cuh:654-677).  elements: 6 arrays of n_total doubles, in the order
 * inclination, longitude of ascending node, argument of perihelion, mean
 * anomaly, eccentricity, semi-major axis: elements[k * n_total + j]. */
int merc_load_elements(merc_ctx* ctx, int32_t n_systems, const int64_t* body_offset,
                       const int32_t* n_massive, const double* mass, const double* elements);

/* Load systems from heliocentric positions and democratic-heliocentric
 * velocities directly.  a_lag (may be NULL) is the semi-major axis the element
 * drift uses for its first mean motion (src/sim.cuh:692); NULL derives it from
 * the state. */
int merc_load_state(merc_ctx* ctx, int32_t n_systems, const int64_t* body_offset,
                    const int32_t* n_massive, const double* mass, const double* pos,
                    const double* vel, const double* a_lag);

/* One system of a batch for merc_load_systems: n_bodies bodies, the first
 * n_massive of them massive, SoA host arrays of this system only
 * (elements[k * n_bodies + j] as in merc_load_elements, pos/vel[c * n_bodies + j]).
 * Give elements for every system of the batch, or pos and vel for every one. */
typedef struct merc_system_desc {
  int32_t n_bodies;
  int32_t n_massive;
  const double* mass;      /* n_bodies */
  const double* elements;  /* 6 x n_bodies, or NULL */
  const double* pos;       /* 3 x n_bodies heliocentric (when elements is NULL) */
  const double* vel;       /* 3 x n_bodies democratic-heliocentric (when elements is NULL) */
} merc_system_desc;

/* Load a batch of systems given one descriptor each (copied; the host
 * arrays stay the caller's).  Equivalent to merc_load_elements or
 * merc_load_state on the concatenated arrays. */
int merc_load_systems(merc_ctx* ctx, const merc_system_desc* systems, int32_t n_systems);

/* Checkpoint: write the whole state of the context (parameters, layout,
 * masses, positions, velocities, a_lag, flags, counters, steps done, the
 * warm-start network if any) to a binary file, and restore it into a context
 * (any previous load is replaced).  Stepping a restored context gives the
 * same bits as stepping the saved one.  A damaged or foreign file is
 * rejected with MERC_ERR_CONFIG (hashed).  The reference writes text
 * positions and elements only (src/mercurius.cu:201-249). */
int merc_save_checkpoint(merc_ctx* ctx, const char* path);
int merc_load_checkpoint(merc_ctx* ctx, const char* path);

/* Overwrite the state of the loaded systems (same layout and sizes as the
 * load) from host buffers; a NULL pointer keeps that part.  Used to stream new
 * initial conditions through a loaded context without reallocation. */
int merc_set_state(merc_ctx* ctx, const double* pos, const double* vel, const double* a_lag);

/* Integrate n_steps Mercurius steps of every loaded system.  Replaces the
 * step loop of mercurius_solver (src/sim.cuh:679-742). */
int merc_step(merc_ctx* ctx, int64_t n_steps);

/* Batch boundary of the reference: reverse democratic-heliocentric
 * conversion, cartesian -> elements, then elements -> cartesian and forward
 * conversion (src/sim.cuh:744-765 then :654-677).  Updates a_lag. */
int merc_roundtrip(merc_ctx* ctx);

/* Copy state out.  pos: heliocentric positions (3*n_total), vel: democratic-
 * heliocentric velocities (3*n_total), flags: n_total.  Any pointer may be NULL.
 * Replaces the output D2H copy of src/mercurius.cu:203-206. */
int merc_get_state(merc_ctx* ctx, double* pos, double* vel, uint32_t* flags);
int merc_get_a_lag(merc_ctx* ctx, double* a_lag);

/* Orbital elements of the current state (reverse DH conversion, then
 * cartesian -> elements; src/sim.cuh:748-758).  Layout as merc_load_elements. */
int merc_get_elements(merc_ctx* ctx, double* elements);

int merc_get_stats(merc_ctx* ctx, merc_stats* out);

/* Energy of each system (massive bodies, Sun included, unsoftened), for
 * conservation checks.  energy: n_systems doubles. */
int merc_energy(merc_ctx* ctx, double* energy);

/* Angular momentum of each system (massive bodies; sum of m x cross v in the
 * context's heliocentric positions and democratic-heliocentric velocities,
 * which is the system's total).  L: 3 doubles per system, L[3 s + c]. */
int merc_angular_momentum(merc_ctx* ctx, double* L);

/* ---- physical collisions ----
 * No counterpart in the reference: its encounter test only chooses the
 * sub-stepper (src/sim.cuh:589-613, 699-730) and bodies pass through each
 * other.  merc_set_radii switches detection on for the loaded systems:
 * radius[j] (AU, n_total values, >= 0; 0 for a point body) for every body;
 * NULL switches it off (the default; every load switches it off).
 * Once per step, after the drift and the encounter sub-step, each body in
 * close encounter that step is tested against the massive bodies of its
 * system: |x_i - x_j| < R_i + R_j is a collision.  (Only bodies in encounter
 * are tested, so R_i + R_j must stay below the changeover radius, as it does
 * for physical radii.)  Colliding pairs (a < b, by index in the system)
 * merge in ascending order while both are unmerged: the heavier body
 * survives (the lower index on a tie) and takes the total mass and the
 * mass-weighted mean position and velocity (momentum and centre of mass are
 * kept; flag MERC_FLAG_GREW); the other body is flagged MERC_FLAG_MERGED,
 * keeps a mass of MERC_MERGED_MASS if it was massive (a source must keep a
 * non-zero critical radius for the reference's changeover formula) and is
 * parked on a circular orbit at MERC_PARK_R + 64 x its index AU in the
 * x-y plane, where it interacts with nothing.  A massless body that hits a
 * massive one is parked the same way and changes nothing else.  The element
 * and universal paths both support it (small systems then run the per-phase
 * kernels, not the persistent sweep kernel).  Masses: merc_get_masses. */
#define MERC_MERGED_MASS 1e-300
#define MERC_PARK_R 1e6
int merc_set_radii(merc_ctx* ctx, const double* radius);

/* One resolved collision: step (counted from the load, 1 = the first step),
 * and the global body indices of the survivor and of the absorbed body. */
typedef struct merc_collision {
  int64_t step;
  int64_t survivor;
  int64_t absorbed;
} merc_collision;

/* Collisions resolved since merc_set_radii, in the order they were resolved.
 * Copies min(total, max) records to out (may be NULL with max 0) and the
 * total count to *count; records beyond the context's log of 65536 are
 * counted but not kept.  Returns MERC_ERR_STATE (after copying) if some step
 * found more than 4096 colliding pairs, more than one step can resolve: pairs
 * beyond that were not merged. */
int merc_get_collisions(merc_ctx* ctx, merc_collision* out, int64_t max, int64_t* count);

/* Current masses (n_total doubles): the loaded masses, changed by collisions. */
int merc_get_masses(merc_ctx* ctx, double* mass);

/* Number of kernel launches issued by this context since creation. */
int64_t merc_launch_count(const merc_ctx* ctx);

/* ---- learned warm start of the universal-variable drift ----
 * No counterpart in the reference (its Kepler solve starts at E = M,
 * src/sim.cuh:93).  A 4 -> 32 -> 32 -> 1 SiLU network in FP32 predicts the
 * universal anomaly from the drift inputs; the FP64 Newton solve that follows
 * is unchanged.  Parameters: a blob of MERC_MLP_BLOB floats (network, input and
 * output normalisation, feature box). */
#define MERC_MLP_BLOB 1267

/* Log (features, target) of every universal drift solve into a device buffer
 * of `capacity` samples (0 turns logging off). */
int merc_mlp_log(merc_ctx* ctx, int64_t capacity);
int64_t merc_mlp_log_count(merc_ctx* ctx);
/* Copy up to max_samples logged samples (5 floats each: x1, x2, x3, x4, target). */
int merc_mlp_get_log(merc_ctx* ctx, float* out, int64_t max_samples);
/* Append n host samples (5 floats each) to the drift log, e.g. the log of
 * another context, to train on several workloads at once. */
int merc_mlp_append_log(merc_ctx* ctx, const float* samples, int64_t n);
/* Train the network on the logged samples on the GPU (hand-written forward,
 * backward and Adam kernels, minibatches drawn by a seeded hash), epochs x
 * (samples / batch) steps.  loss_per_epoch (may be NULL): epochs floats. */
int merc_mlp_train(merc_ctx* ctx, int32_t epochs, int32_t batch, float lr, uint64_t seed, float* loss_per_epoch);
int merc_mlp_set_weights(merc_ctx* ctx, const float* blob);
int merc_mlp_get_weights(merc_ctx* ctx, float* blob);

/* Bytes of the fixed device scratch array behind merc_step_static. */
#define MERC_STATIC_SCRATCH_BYTES (16u << 20)

/* Allocation-free stepping.  No counterpart in the reference (which has no
 * library interface); it exists for callers that cannot call cudaMalloc: an
 * application that gives the library device memory from its own pool or
 * framework allocator, a runtime that forbids allocation after start-up, or a
 * caller that must not add allocator traffic while it records GPU work.
 *
 * Integrates n_steps universal-drift steps (p->drift must be
 * MERC_DRIFT_UNIVERSAL) of ONE system whose state is in caller-owned device
 * memory: pos and vel (3 * n_bodies doubles each, component-major,
 * heliocentric positions and democratic-heliocentric velocities, updated in
 * place), mass (n_bodies doubles, massive bodies first) and flags
 * (n_bodies uint32, updated; may be NULL).  stream is a cudaStream_t or NULL
 * for the default stream; the call returns after the stream has finished the
 * work.  The function allocates nothing: every scratch buffer comes from one
 * fixed device array of MERC_STATIC_SCRATCH_BYTES, which every GPU that loads
 * the library holds until the process exits.  Sizes whose scratch does not
 * fit (about 100k bodies for a system with many massive bodies) return
 * MERC_ERR_CONFIG before any work is queued.
 *
 * The call makes `device` current while it works and restores the calling
 * thread's current device before it returns.  It must not be called while
 * `stream` (or, for the legacy default stream, any stream) is being captured
 * into a CUDA graph: it copies small tables from its own stack frame and
 * waits for the stream before returning, so it returns MERC_ERR_STATE
 * instead of queuing anything.  The first call on a device also looks up the
 * array's device address on that device (cudaGetSymbolAddress).  All calls
 * share the one array, and each call re-initialises the parts that must start
 * at zero, so calls that overlap on the GPU (other host threads, other
 * streams) race with each other: serialise them. */
int merc_step_static(int device, const merc_params* p, int32_t n_bodies, int32_t n_massive, double* pos,
                     double* vel, const double* mass, uint32_t* flags, int64_t n_steps, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MERC_H */
