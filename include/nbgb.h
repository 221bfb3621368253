/*
 * nbgb.h -- C ABI of the GB300 N-body step library (libnbgb.so).
 *
 * Drop-in for the per-step OpenCL path of Ace-of-Heartz/NBodySimulation:
 * the parameter surface of SimulationConfig / BarnesHutConfig / Simulation
 * (src/SimulationConfig.h:46-133, src/BarnesHutConfig.h:10-61), the body
 * buffers CMyApp owns (src/MyApp.h:152-167; packed float[3N] positions and
 * velocities, float[N] masses, src/MyApp.cpp:219-235) and the per-step entry
 * CMyApp::Update (src/MyApp.cpp:550-656).
 *
 * Conventions
 *   - Plain C types only; no exceptions cross this boundary.  Every call
 *     returns an nb_status; nb_last_error_message() explains the last failure
 *     of a handle.
 *   - Host arrays use the reference's packed layout: pos3/vel3/acc3 are
 *     float[3*N] (x,y,z per body), mass is float[N].  The caller owns them.
 *   - A handle owns one CUDA stream and all device memory of one system;
 *     use one handle from one host thread at a time.
 *   - Device errors (cell overflow, depth overflow, a wait that ran out of
 *     iterations, non-finite input) are reported through a device status
 *     word read back at the end of nb_step / nb_update; no kernel traps.
 */
#ifndef NBGB_H
#define NBGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#define NBGB_ABI_VERSION 1

typedef enum nb_status {
    NB_OK = 0,
    NB_ERR_INVALID_ARGUMENT = 1,
    NB_ERR_CUDA = 2,
    NB_ERR_OUT_OF_MEMORY = 3,
    NB_ERR_CELL_OVERFLOW = 4,  /* tree needed more cells than cell_capacity (build_tree.cl:109-114) */
    NB_ERR_DEPTH = 5,          /* tree deeper than NB_MAX_DEPTH (calculate_forces.cl:63-67) */
    NB_ERR_SPIN_TIMEOUT = 6,   /* a bounded device wait gave up */
    NB_ERR_NONFINITE = 7,      /* a body position is NaN or infinite */
    NB_ERR_NO_DEVICE = 8,
    NB_ERR_STATE = 9,          /* call out of order (e.g. step before state) */
    NB_ERR_UNSUPPORTED = 10
} nb_status;

#define NB_MAX_DEPTH 64 /* kernels/calculate_forces.hcl:1 */

/* NumericalMethod (src/SimulationConfig.h:10-14, kernels/common.hcl:21-24). */
enum {
    NB_LEAPFROG = 1,     /* the reference's "Leapfrog" formula as written */
    NB_EULER = 2,        /* kick-then-drift Euler, the reference default */
    NB_KDK_LEAPFROG = 3  /* addition: kick-drift-kick leapfrog, velocities at half steps */
};

/* PositionConfig (src/SimulationConfig.h:16-20) plus additions. */
enum {
    NB_SPHERE_POS = 0,       /* Fibonacci sphere of radius starting_volume_radius */
    NB_UNIFORM_POS = 1,      /* the reference's "uniform": normal(0, R) per axis */
    NB_BALL_POS = 2,         /* addition: uniform in the ball of radius R */
    NB_NORMAL_SIGMA_POS = 3  /* addition: normal(0, pos_sigma[k]) per axis */
};

/* VelocityConfig (src/SimulationConfig.h:22-29) plus one addition. */
enum {
    NB_RANDOM_VEL = 0,
    NB_STARTING_OUT_VEL = 1,
    NB_STARTING_IN_VEL = 2,
    NB_FUNC_ZERO_VEL = 3,
    NB_TANGENT_XZ_VEL = 4,
    NB_CIRCULAR_Z_VEL = 5    /* addition: tangential about z, |v| = sqrt(G*M(<r)/r), M(<r)=Mtot*(r/R)^3 */
};

/* AlgorithmConfig (src/SimulationConfig.h:32-38). */
enum { NB_BARNES_HUT = 0, NB_BRUTE_FORCE_GLOBAL = 1, NB_BRUTE_FORCE_LOCAL = 2 };

/* Mass distributions (src/MyApp.cpp:333-355 is NB_MASS_NORMAL_ABS). */
enum { NB_MASS_NORMAL_ABS = 0, NB_MASS_EQUAL = 1, NB_MASS_LOGNORMAL = 2 };

/* Tree geometry.  NB_TREE_GEOMETRIC: cubic root, octants halve every axis.
 * NB_TREE_REFERENCE: the reference's tree bit for bit -- axis-aligned box
 * root under a one-child super-root (build_tree.cl:57-65) and y bounds that
 * follow the x octant bit (build_tree.hcl:42-46). */
enum { NB_TREE_GEOMETRIC = 0, NB_TREE_REFERENCE = 1 };

/* Opening criterion.  NB_THETA_STANDARD: accept a cell of width w when
 * d^2 + eps^2 >= (w/theta)^2 + eps^2 (Burtscher).  NB_THETA_REFERENCE: the
 * reference's thresholds r^2/theta + eps (calculate_forces.cl:45-61). */
enum { NB_THETA_STANDARD = 0, NB_THETA_REFERENCE = 1 };

/* Force accumulation precision.  NB_PRECISION_COMPENSATED keeps a TwoSum
 * low word per component; each batch of up to 32 opened children is summed
 * in FP32 and then added with one TwoSum. */
enum { NB_PRECISION_FP32 = 0, NB_PRECISION_COMPENSATED = 1 };

/* Cell expansion of the Barnes-Hut force.  NB_MULTIPOLE_MONOPOLE is the
 * reference's centre-of-mass term; NB_MULTIPOLE_QUADRUPOLE adds each
 * accepted cell's traceless quadrupole about its centre of mass. */
enum { NB_MULTIPOLE_MONOPOLE = 0, NB_MULTIPOLE_QUADRUPOLE = 1 };

/* Direct-sum force law.  NB_FORCE_PLUMMER: a = G sum m r (r^2+eps^2)^-3/2.
 * NB_FORCE_REFERENCE_QUIRK: the reference's brute-force arithmetic,
 * a = G sum m n/(|n|^2+e^2) with n = normalize(r), e = 0.01 (global,
 * brute_force_update.cl:54-58) or 0.1 (local, :114-120). */
enum { NB_FORCE_PLUMMER = 0, NB_FORCE_REFERENCE_QUIRK = 1 };

typedef struct nb_config {
    /* SimulationConfig (src/SimulationConfig.h:85-104) */
    int32_t num_of_bodies;             /* 20000 */
    float gravitational_constant;      /* 6.67e-11 */
    float starting_speed_mul;          /* 1.0 */
    float starting_volume_radius;      /* 1.5 */
    int32_t number_of_massive_objects; /* 0 */
    float massive_object_mass;         /* 1.0 */
    int32_t collision;                 /* 0 */
    int32_t pos_config;                /* NB_UNIFORM_POS */
    int32_t vel_config;                /* NB_FUNC_ZERO_VEL */
    int32_t algo_config;               /* NB_BRUTE_FORCE_GLOBAL */
    float mass_mean;                   /* 0.5  (NormalDistribution) */
    float mass_deviation;              /* 0.25 */
    int32_t numerical_method;          /* NB_EULER */
    /* BarnesHutConfig (src/BarnesHutConfig.h:58-60) */
    int32_t max_octree_depth;          /* 32; informational, as in the reference */
    float theta;                       /* 1.5 */
    float epsilon;                     /* 0.01 */
    /* Simulation (src/SimulationConfig.h:131-132) */
    float simulation_speed_mul;        /* 1.0 */
    float particle_size;               /* 0.05 */
    /* additions of this library */
    int32_t tree_semantics;            /* NB_TREE_GEOMETRIC */
    int32_t theta_semantics;           /* NB_THETA_STANDARD */
    int32_t precision;                 /* NB_PRECISION_FP32 */
    int32_t force_law;                 /* NB_FORCE_PLUMMER */
    float direct_epsilon;              /* Plummer softening of the direct sums; < 0: use epsilon */
    int32_t cell_capacity;             /* 0: max(2N, 1024*SMs) rounded up to 16 (src/MyApp.cpp:75-79) */
    int32_t mass_config;               /* NB_MASS_NORMAL_ABS */
    float pos_sigma[3];                /* NB_NORMAL_SIGMA_POS */
    float mass_lognormal_sigma;        /* NB_MASS_LOGNORMAL, mu = 0, normalised to total 1 */
    uint64_t seed;                     /* initial-condition generator seed */
    int32_t device;                    /* CUDA device ordinal */
    int32_t multipole;                 /* NB_MULTIPOLE_MONOPOLE */
    int32_t reserved[6];
} nb_config;

typedef struct nb_sim nb_sim;

/* ---- versioning, errors, configuration ---- */
int32_t nb_abi_version(void);
const char *nb_status_string(nb_status s);
/* Fills the reference's defaults (src/SimulationConfig.h:85-104,
 * src/BarnesHutConfig.h:58-60, src/SimulationConfig.h:131-132). */
void nb_config_default(nb_config *cfg);

/* ---- lifetime (CMyApp::InitCL / InitParticles, src/MyApp.cpp:110-243) ---- */
/* Allocates every device buffer for cfg->num_of_bodies bodies. */
nb_status nb_create(const nb_config *cfg, nb_sim **out);
nb_status nb_destroy(nb_sim *sim);
nb_status nb_get_config(const nb_sim *sim, nb_config *out);

/* ---- body state (the cl_p / cl_v / cl_m / cl_a buffers) ---- */
/* Host arrays, reference layout.  vel3 may be NULL (zero velocities).
 * Resets the stored accelerations (InitObjectAcceleration,
 * src/MyApp.cpp:497-504).  n must equal num_of_bodies.  Page-locked arrays
 * (nb_host_alloc, cudaMallocHost, cudaHostRegister) are read by the device
 * directly, without a staging copy; others are copied through a staging
 * buffer. */
nb_status nb_set_state(nb_sim *sim, const float *pos3, const float *vel3, const float *mass, int32_t n);
/* Any output pointer may be NULL.  Page-locked pos3 / vel3 (with acc3 and
 * mass NULL) are written by the device directly. */
nb_status nb_get_state(nb_sim *sim, float *pos3, float *vel3, float *acc3, float *mass);
/* Seeded initial conditions of cfg (InitBodyAttributes, src/MyApp.cpp:331-495),
 * generated on the host.  Arrays: pos3/vel3 float[3N], mass float[N]. */
nb_status nb_generate_ic(const nb_config *cfg, float *pos3, float *vel3, float *mass);
/* nb_generate_ic for the handle's config, then nb_set_state. */
nb_status nb_init_bodies(nb_sim *sim);

/* ---- stepping (CMyApp::Update, src/MyApp.cpp:550-656) ---- */
/* nsteps steps of fixed dt through the configured algorithm, then waits
 * and returns the device status.  Positions are double-buffered: every force
 * of a step sees the step-start positions. */
nb_status nb_step(nb_sim *sim, float dt, int32_t nsteps);
/* One step with the reference's frame-time rule: dt = clamp(frame_dt,
 * 1e-4, 5e-3) * simulation_speed_mul (src/MyApp.cpp:556-561). */
nb_status nb_update(nb_sim *sim, float frame_dt_seconds);
/* Enqueue without waiting; nb_synchronize returns the device status. */
nb_status nb_step_async(nb_sim *sim, float dt, int32_t nsteps);
nb_status nb_synchronize(nb_sim *sim);

/* copy_vertices (kernels/copy_vertices.cl:3-17): float4{x,y,z,1} per body
 * into dst (device pointer if dst_is_device, 16-byte aligned; else host,
 * written directly when page-locked and 16-byte aligned). */
nb_status nb_copy_vertices(nb_sim *sim, float *dst4, int32_t dst_is_device);

/* ---- introspection of the last step (parity and debugging) ---- */
enum {
    NB_DEBUG_BBOX = 0,          /* float[6] min xyz, max xyz */
    NB_DEBUG_CHILDREN = 1,      /* int32[8*(N+C+1)] reference layout, octant slots, cell rows at node index */
    NB_DEBUG_NODE_POS = 2,      /* float[3*(N+C+1)] bodies then cell centres of mass */
    NB_DEBUG_NODE_MASS = 3,     /* float[N+C+1] */
    NB_DEBUG_BODY_COUNT = 4,    /* int32[N+C+1] subtree body counts (cells) */
    NB_DEBUG_SORTED = 5,        /* int32[N] in-order body placement */
    NB_DEBUG_TREE_INFO = 6,     /* int32[4] {N, C (cell capacity), bottom, max_depth} */
    NB_DEBUG_DQ = 7,            /* float[64] opening thresholds of the last force pass */
    NB_DEBUG_NODE_QUAD = 8      /* float[6*(N+C+1)] cell quadrupoles {xx,yy,zz,xy,xz,yz}, 0 for bodies */
};
nb_status nb_get_stage_debug(nb_sim *sim, int32_t which, void *dst, size_t bytes, size_t *written);
/* Per-stage GPU time in ms, averaged over the steps of the last nb_step
 * call (CUDA events on the handle's stream, at most 256 steps); stage order
 * {bbox+reset, build, summarize, sort, force, collision, direct}.  Needs
 * nb_set_profiling(sim, 1). */
nb_status nb_set_profiling(nb_sim *sim, int32_t on);
nb_status nb_get_timings(nb_sim *sim, float *stage_ms, int32_t n);
/* Kernel launches issued by the handle since creation. */
int64_t nb_kernel_launches(const nb_sim *sim);
/* nb_step bracketed by CUDA events on the handle's stream; *total_ms is the
 * device time of the nsteps steps. */
nb_status nb_time_steps(nb_sim *sim, float dt, int32_t nsteps, float *total_ms);
/* Work of the last nb_step call: out[0] body-node interactions of the force
 * passes (per body, per accepted node), out[1] cells opened by the warps,
 * out[2] the part of out[0] with cells (the rest are body-body pairs). */
nb_status nb_get_work_counters(nb_sim *sim, uint64_t out[3]);

/* ---- device-resident access (interop, benchmarking) ---- */
typedef struct nb_device_view {
    void *body_pm;   /* float4[N] {x,y,z,m}, current positions */
    void *vel;       /* float4[N] {vx,vy,vz,0} */
    void *acc;       /* float4[N] {ax,ay,az,0} of the last force pass */
    void *stream;    /* cudaStream_t of the handle */
    int32_t n;
} nb_device_view;
nb_status nb_get_device_view(nb_sim *sim, nb_device_view *out);
/* Device arrays in the reference layout (float[3N] / float[N]). */
nb_status nb_set_state_device(nb_sim *sim, const float *d_pos3, const float *d_vel3, const float *d_mass);
nb_status nb_get_state_device(nb_sim *sim, float *d_pos3, float *d_vel3);

/* ---- diagnostics (FP64 on the GPU) ---- */
/* FP64 direct-sum accelerations of the listed bodies at the positions of the
 * last force pass; out: max and RMS of |a - a64| / |a64| over the samples,
 * per-sample relative errors into rel_err (may be NULL). */
nb_status nb_force_error_probe(nb_sim *sim, const int32_t *sample, int32_t ns, double *max_rel, double *rms_rel,
                               double *rel_err);
/* out[0..8]: kinetic energy, momentum xyz, angular momentum xyz, total mass,
 * potential energy (FP64 pair sum; computed only when with_potential != 0).
 * Every sum is over the stored state, the one nb_get_state returns.  Under
 * NB_KDK_LEAPFROG the stored velocities are the half-step velocities
 * v(t - dt/2) of the drift that produced the positions x(t), so the kinetic
 * energy, momentum and angular momentum are those of v(t - dt/2) (with x(t)
 * for the angular momentum); under NB_EULER and NB_LEAPFROG velocity and
 * position belong to the same step. */
nb_status nb_diagnostics(nb_sim *sim, int32_t with_potential, double out[9]);

/* ---- failure-path test hook ----
 * Caps the iterations of the tree stages' bounded waits (the build's lock
 * retries and the sort's wait for a parent's start) at `cap` (0 restores the
 * default, 2^24).  With a tiny cap a step gives up with NB_ERR_SPIN_TIMEOUT
 * instead of waiting, keeps its step-start state, and the handle stays
 * usable: the way the timeout path is exercised without hanging a GPU. */
nb_status nb_debug_set_spin_cap(nb_sim *sim, int32_t cap);

/* ---- last error ---- */
nb_status nb_last_error(const nb_sim *sim);
const char *nb_last_error_message(const nb_sim *sim);

/* ---- pinned host memory for zero-staging transfers ---- */
void *nb_host_alloc(size_t bytes);
void nb_host_free(void *p);

/* ---- all-pairs accelerations without any device allocation ----
 * No counterpart in the reference: an addition of this library.
 *
 * For callers that cannot call cudaMalloc: a host application that owns the
 * whole device-memory budget and only lends the library its own buffers, or a
 * frame loop that must not enter the CUDA allocator (it can synchronise the
 * device and serialise on a lock).  Every other entry point allocates at
 * nb_create; this one allocates nothing.
 *
 * Computes a_i = G * sum_{j != i} m_j r_ij (|r_ij|^2 + eps^2)^-3/2 for the n
 * bodies of d_body4 (device float4 {x,y,z,m}, 16-byte aligned) into d_acc4
 * (device float4 {ax,ay,az,0}, 16-byte aligned), on `stream` (a
 * cudaStream_t; NULL for the default stream) of the current device.  The
 * call is synchronous: it returns after its work on `stream` has finished
 * (it synchronises that stream to read the status of its bounded waits).
 * Same arithmetic as the NB_BRUTE_FORCE_LOCAL Plummer sum.
 *
 * Limit: n <= NB_NOALLOC_MAX_BODIES; larger n returns NB_ERR_INVALID_ARGUMENT.
 * Its scratch is a fixed array inside the library (1 MiB), held by every GPU
 * that loads the library until the process exits.  The first call on a
 * device looks up that array's device address; make that first call before
 * any stream capture.  The address is kept for the life of the process, so
 * after a cudaDeviceReset of a device this entry point must not be called on
 * that device again.  All calls share the array, so calls that overlap on
 * the GPU race: serialise them. */
#define NB_NOALLOC_MAX_BODIES 65536
nb_status nb_direct_accel_noalloc(const float *d_body4, int32_t n, float eps, float G, float *d_acc4,
                                  void *stream);

/* ---- snapshot files ----
 * One system at one step: a 32-byte header (magic "NBSNAP01", uint32 version
 * 1, uint32 N, int64 step, float64 simulated time) followed by float32
 * positions[3N], velocities[3N], masses[N]; every field little-endian.  The
 * reference keeps no files (its state lives in OpenCL buffers); this is the
 * exchange format for snapshots of served jobs and of any handle.
 * nb_snapshot_write: vel3 may be NULL (zeros are written).
 * nb_snapshot_read: with all three arrays NULL only the header is read (*n,
 * *step, *time); otherwise N must be <= capacity; any array may be NULL.
 * nb_save_snapshot: the handle's current state (as nb_get_state). */
nb_status nb_snapshot_write(const char *path, int64_t step, double time, const float *pos3, const float *vel3,
                            const float *mass, int32_t n);
nb_status nb_snapshot_read(const char *path, int64_t *step, double *time, float *pos3, float *vel3, float *mass,
                           int32_t capacity, int32_t *n);
nb_status nb_save_snapshot(nb_sim *sim, const char *path, int64_t step, double time);

/* ---- batched systems ----
 * Many independent simulations of uneven N advanced together, each with its
 * own nb_config (the reference runs one CMyApp per simulation,
 * src/MyApp.cpp:110-656).  Every stage of a step is one kernel launch over
 * all systems, and one step is replayed as a CUDA graph.  Systems with
 * algo_config NB_BARNES_HUT take the tree path, the others the tiled direct
 * sum.  All systems must share numerical_method, precision, multipole and
 * device; epsilon (direct_epsilon for direct systems) must be > 0; the
 * reference quirk force law is not batched.  Systems with collision != 0 run
 * the collision update after their integration, as a standalone handle does
 * (one more launch per step over all of them).  Each system's step is the
 * same computation as nb_step on a standalone handle: the tree path and the
 * collision update are bit-identical, the direct sum differs only in
 * summation order. */
typedef struct nb_batch nb_batch;
nb_status nb_batch_create(const nb_config *cfgs, int32_t nsys, nb_batch **out);
nb_status nb_batch_destroy(nb_batch *b);
/* State of system k (host arrays, reference layout); vel3 may be NULL (zero). */
nb_status nb_batch_set_state(nb_batch *b, int32_t k, const float *pos3, const float *vel3, const float *mass);
nb_status nb_batch_get_state(nb_batch *b, int32_t k, float *pos3, float *vel3, float *acc3, float *mass);
/* nsteps steps of all systems with time step dt; returns the first failing
 * system's status (the others advanced normally; a failed system keeps the
 * state it had at the start of the failing step). */
nb_status nb_batch_step(nb_batch *b, float dt, int32_t nsteps);
/* As nb_batch_step, timed with CUDA events around the graph launches. */
nb_status nb_batch_time_steps(nb_batch *b, float dt, int32_t nsteps, float *total_ms);
/* Status of system k after the last nb_batch_step. */
nb_status nb_batch_system_status(nb_batch *b, int32_t k);
/* Chooses launch shapes by timing candidates on this batch with dt = 0
 * (positions, velocities and accelerations unchanged): the direct-sum kernel
 * shape (*chosen) and the tree stages' shape (nb_batch_tree_shape).  The
 * choices are cached in the JSON file cache_path (may be NULL) under keys of
 * the SM count and the batch's size profile (and, for the tree stages, its
 * multipole and precision).  No shape changes a result: a tuned batch's
 * systems stay bit-identical to standalone handles for the tree path. */
nb_status nb_batch_autotune(nb_batch *b, const char *cache_path, int32_t *chosen);
/* The tree stages' launch shape: warps per block of the force walk, percent
 * of its resident blocks launched, bodies per bbox / build block (0: the
 * default rule) and the cap on the top levels built before the insertions. */
nb_status nb_batch_tree_shape(nb_batch *b, int32_t out[4]);
/* out: systems, bodies, tree systems, direct systems, launches per step,
 * direct variant, kernels launched so far, body-node interactions of the
 * last step (tree systems). */
nb_status nb_batch_info(nb_batch *b, int64_t out[8]);
const char *nb_batch_last_error_message(const nb_batch *b);

/* ---- job server: continuous batching of simulation jobs ----
 * No counterpart in the reference (one interactive simulation per process);
 * a serving layer over the batched step.
 *
 * Jobs (an nb_config, initial conditions, a step count and dt) are queued by
 * nb_server_submit from any thread and admitted first come first served
 * while a slot (max_jobs) and their device memory (bodies plus up to
 * max(2N, 4096) tree cells, counted against hbm_budget_bytes) are free.  Their
 * state stays resident in HBM while they run.  Every round of
 * snapshot_every steps advances all running jobs together (one launch per
 * stage over all of them, replayed as a CUDA graph); jobs admitted while a
 * round runs join at the next round, and a job that finishes stops taking
 * part at once.  Positions are returned every snapshot_every steps and the
 * final positions and velocities at the end, through the callback (from a
 * library thread) or, without one, by nb_server_result.  A job's result does
 * not depend on what runs beside it (bit-identical alone and in a mix);
 * tree jobs are also bit-identical to a standalone handle's nb_step, direct
 * jobs equal to it within FP32 summation-order tolerance.  All jobs share
 * numerical_method, precision and multipole (set in the server config; a
 * job whose config differs is refused). */
typedef struct nb_server nb_server;
typedef struct nb_server_config {
    int32_t device;
    int32_t max_jobs;          /* jobs on the GPU at once */
    int64_t hbm_budget_bytes;  /* device memory for job state */
    int32_t snapshot_every;    /* steps between snapshots (0: none; rounds are then 10 steps) */
    int32_t numerical_method;
    int32_t precision;
    int32_t multipole;
    int32_t direct_variant;    /* direct-sum kernel shape (nb_batch_autotune's choice); -1: default */
    int32_t reserved[7];
} nb_server_config;
enum { NB_JOB_QUEUED = 0, NB_JOB_RUNNING = 1, NB_JOB_DONE = 2, NB_JOB_FAILED = 3 };
enum { NB_JOB_EVENT_SNAPSHOT = 0, NB_JOB_EVENT_DONE = 1, NB_JOB_EVENT_FAILED = 2 };
/* event SNAPSHOT: value = steps done, pos3 (vel3 NULL); DONE: value = steps,
 * pos3 and vel3; FAILED: value = the nb_status, no arrays.  The arrays are
 * valid during the call only.  The callback runs on the server's delivery
 * thread: it may call nb_server_submit, nb_server_job_info and
 * nb_server_get_stats, but not nb_server_wait or nb_server_destroy (those
 * wait for that thread), and a slow callback delays the later deliveries. */
typedef void (*nb_job_fn)(void *user, int64_t job, int32_t event, int32_t value, const float *pos3,
                          const float *vel3, int32_t n);
void nb_server_config_default(nb_server_config *c);
nb_status nb_server_create(const nb_server_config *c, nb_job_fn fn, void *user, nb_server **out);
/* Copies the inputs.  pos3 == NULL: initial conditions are generated from
 * cfg by nb_generate_ic on a server thread (vel3 and mass are then ignored);
 * vel3 == NULL: zero velocities. */
nb_status nb_server_submit(nb_server *s, const nb_config *cfg, int32_t steps, float dt, const float *pos3,
                           const float *vel3, const float *mass, int64_t *job);
typedef struct nb_job_info {
    int32_t state;        /* NB_JOB_* */
    int32_t status;       /* nb_status of a failed job */
    int32_t steps;
    int32_t n;
    double t_submit;      /* seconds since nb_server_create */
    double t_admit;
    double t_done;
    int64_t bytes;        /* device footprint */
} nb_job_info;
nb_status nb_server_job_info(nb_server *s, int64_t job, nb_job_info *out);
/* Waits until the job (job < 0: every job submitted so far) has finished;
 * NB_ERR_SPIN_TIMEOUT after timeout_s seconds (< 0: no limit). */
nb_status nb_server_wait(nb_server *s, int64_t job, double timeout_s);
/* Final state of a finished job when the server has no callback (copied
 * once, then released); either array may be NULL.  Without a callback the
 * results stay in host memory until fetched; every job keeps a small record
 * (its config and times, for nb_server_job_info) until nb_server_destroy. */
nb_status nb_server_result(nb_server *s, int64_t job, float *pos3, float *vel3);
typedef struct nb_server_stats {
    int64_t submitted, completed, failed, queued, running;
    int64_t rounds;
    int64_t bytes_in_use, peak_bytes;
    int32_t peak_jobs;
    int32_t pad;
    double body_updates;  /* sum of N * steps over completed jobs */
    double first_submit_s, last_done_s;
    double latency_p50_s, latency_p99_s, latency_max_s, latency_mean_s;
} nb_server_stats;
nb_status nb_server_get_stats(nb_server *s, nb_server_stats *out);
/* Stops admitting, cancels queued and running jobs, waits for the GPU and
 * frees everything. */
nb_status nb_server_destroy(nb_server *s);
const char *nb_server_last_error_message(const nb_server *s);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
