/*
 * assist.h -- C ABI of libassist_gb300: ASSIST's plugin surface for the
 * test-particle equations of motion, backed by sm_103a kernels.
 *
 * Every declaration below replaces the ASSIST v1.2.0 interface cited beside it
 * (paths are relative to the ASSIST source tree).  Struct layouts that the
 * ASSIST ctypes wrapper mirrors (assist/ephem.py:95-120, assist/extras.py:84-101)
 * keep ASSIST's member order and types so those mirrors read them unchanged.
 *
 * Beyond ASSIST's own surface this header adds the batched entry points
 * (assist_gb300_*) through which independent particles with their own
 * adaptive IAS15 steps are integrated in one persistent device kernel.
 */
#ifndef ASSIST_GB300_ASSIST_H
#define ASSIST_GB300_ASSIST_H

#include <stdint.h>
#include <stddef.h>
#include <stdio.h>
#include "rebound.h"

#ifdef __cplusplus
extern "C" {
#endif

extern const char* assist_build_str;      /* src/assist.h:36 */
extern const char* assist_version_str;    /* src/assist.h:37 */
extern const char* assist_githash_str;    /* src/assist.h:38 */

/* src/assist.h:53-58 */
typedef enum {
    FILE_FORMAT_VALID_BSP = 0,
    FILE_FORMAT_ASCII_BIN = 2,
    FILE_FORMAT_UNKNOWN = 3
} ephemeris_file_format_t;

int assist_detect_ascii_bin_signature(int fd);                               /* src/assist.h:65 */
ephemeris_file_format_t assist_detect_ephemeris_file_format(int fd);          /* src/assist.h:68 */
int assist_discover_planets_path(char* out_path, size_t out_path_size,
                                 const char* assist_dir);                     /* src/assist.h:72 */

/* Force selection bits, src/assist.h:76-87 */
enum ASSIST_FORCES {
    ASSIST_FORCE_NONE               = 0,
    ASSIST_FORCE_SUN                = 0x01,
    ASSIST_FORCE_PLANETS            = 0x02,
    ASSIST_FORCE_ASTEROIDS          = 0x04,
    ASSIST_FORCE_NON_GRAVITATIONAL  = 0x08,
    ASSIST_FORCE_EARTH_HARMONICS    = 0x10,
    ASSIST_FORCE_SUN_HARMONICS      = 0x20,
    ASSIST_FORCE_GR_EIH             = 0x40,
    ASSIST_FORCE_GR_SIMPLE          = 0x80,
    ASSIST_FORCE_GR_POTENTIAL       = 0x100,
};

/* Status codes, src/assist.h:90-98; messages in assist_error_messages[]. */
enum ASSIST_STATUS {
    ASSIST_SUCCESS,
    ASSIST_ERROR_EPHEM_FILE,
    ASSIST_ERROR_AST_FILE,
    ASSIST_ERROR_NAST,
    ASSIST_ERROR_NEPHEM,
    ASSIST_ERROR_COVERAGE,
    ASSIST_ERROR_N,
};

extern const char* assist_error_messages[];   /* src/assist.c:52-59 */
extern const int assist_error_messages_N;     /* src/assist.c:60 */

/* Body indices, src/assist.h:102-116.  Asteroids follow at 11.. */
enum ASSIST_BODY {
    ASSIST_BODY_SUN         = 0,
    ASSIST_BODY_MERCURY     = 1,
    ASSIST_BODY_VENUS       = 2,
    ASSIST_BODY_EARTH       = 3,
    ASSIST_BODY_MOON        = 4,
    ASSIST_BODY_MARS        = 5,
    ASSIST_BODY_JUPITER     = 6,
    ASSIST_BODY_SATURN      = 7,
    ASSIST_BODY_URANUS      = 8,
    ASSIST_BODY_NEPTUNE     = 9,
    ASSIST_BODY_PLUTO       = 10,
    ASSIST_BODY_NPLANETS    = 11,
};

struct ascii_s;
struct spk_s;

/* Ephemeris handle, src/assist.h:125-155 (layout mirrored by assist/ephem.py:95-120).
 * `planets_calc` keeps its slot for layout; this library evaluates bodies on the
 * device and leaves it pointing at a host dispatcher that launches the kernel. */
struct assist_ephem {
    double jd_ref;
    struct spk_s* spk_planets;
    struct spk_s* spk_asteroids;
    struct ascii_s* ascii_planets;
    int planets_source;
    enum ASSIST_STATUS (*planets_calc)(const struct assist_ephem*, double, double, int,
                                       double* const,
                                       double* const, double* const, double* const,
                                       double* const, double* const, double* const,
                                       double* const, double* const, double* const);
    int spk_target_index[ASSIST_BODY_NPLANETS];
    int spk_emb_index;
    double AU;
    double EMRAT;
    double J2E;
    double J3E;
    double J4E;
    double J2SUN;
    double RE;
    double CLIGHT;
    double ASUN;
    double Re_eq;
    double Rs_eq;
    double c_AU_per_day;
    double c_squared;
    double over_c_squared;
};

/* src/assist.h:157-168 */
struct assist_cache_item {
    double GM;
    double x, y, z;
    double vx, vy, vz;
    double ax, ay, az;
};

/* src/assist.h:171-175.  Kept for layout; the device path evaluates every
 * body once per distinct time and needs no host-side cache. */
struct assist_ephem_cache {
    double* t;
    double dt_sign;
    struct assist_cache_item* items;
};

/* Per-simulation extras, src/assist.h:177-195 (mirrored by assist/extras.py:84-101). */
struct assist_extras {
    struct reb_simulation* sim;
    struct assist_ephem* ephem;
    struct assist_ephem_cache* ephem_cache;
    int extras_should_free_ephem;
    int geocentric;
    struct reb_particle* last_state;
    struct reb_particle* current_state;
    double* particle_params;
    int steps_done;
    int forces;
    int gr_eih_sources;
    double alpha;
    double nk;
    double nm;
    double nn;
    double r0;
};

struct assist_extras* assist_attach(struct reb_simulation* sim, struct assist_ephem* ephem);  /* src/assist.h:202 */
void assist_free(struct assist_extras* assist);                                              /* src/assist.h:209 */
void assist_ephem_free(struct assist_ephem* ephem);                                          /* src/assist.h:211 */
void assist_detach(struct reb_simulation* sim, struct assist_extras* assist);                /* src/assist.h:218 */
void assist_error(struct assist_extras* assist, const char* const msg);                      /* src/assist.h:227 */
int assist_interpolate_simulation(struct reb_simulation* sim1, struct reb_simulation* sim2, double h);  /* src/assist.h:230 */
void assist_integrate_or_interpolate(struct assist_extras* ax, double t);                    /* src/assist.h:232 */
struct reb_particle assist_get_particle(const struct assist_ephem* ephem, const int particle_id, const double t);  /* src/assist.h:235 */
struct reb_particle assist_get_particle_with_error(const struct assist_ephem* ephem, const int particle_id,
                                                   const double t, int* error);              /* src/assist.h:245 */
void assist_ephem_time_bounds(const struct assist_ephem* ephem, double* t_beg, double* t_end);  /* src/assist.h:262 */
void assist_init(struct assist_extras* assist, struct reb_simulation* sim, struct assist_ephem* ephem);  /* src/assist.h:265 */
void assist_free_pointers(struct assist_extras* assist);                                     /* src/assist.h:266 */
void assist_ephem_free_pointers(struct assist_ephem* ephem);                                 /* src/assist.h:267 */
struct assist_ephem* assist_ephem_create(char* planets_file_name, char* asteroids_file_name);  /* src/assist.h:274 */
int assist_ephem_init(struct assist_ephem* ephem, char* user_planets_path, char* user_asteroids_path);  /* src/assist.h:290 */

/* REBOUND's additional_forces callback, src/forces.h / src/forces.c:49.
 * Reads sim->particles (host), evaluates ephemeris + forces + variational
 * partials on the device and adds the accelerations into sim->particles[].a*
 * exactly as the CPU callback does (REBOUND zeroes them before the call). */
void assist_additional_forces(struct reb_simulation* sim);

/* Body state at time t, src/forces.h / src/forces.c:175.  `ephem_cache` is
 * accepted for signature compatibility and ignored. */
int assist_all_ephem(const struct assist_ephem* ephem, struct assist_ephem_cache* ephem_cache,
                     const int i, const double t, double* const GM,
                     double* const x, double* const y, double* const z,
                     double* const vx, double* const vy, double* const vz,
                     double* const ax, double* const ay, double* const az);

/* ------------------------------------------------------------------------
 * Batched device API (no ASSIST counterpart: ASSIST integrates one REBOUND
 * simulation at a time on one CPU core).
 * ---------------------------------------------------------------------- */

/* Options shared by the batched entry points.  Force-model fields mean what
 * the assist_extras fields of the same name mean (src/assist.h:177-195). */
struct assist_gb300_options {
    int forces;             /* ASSIST_FORCES bits (ASSIST default 0x7F) */
    int gr_eih_sources;     /* EIH source bodies, ASSIST default 1 */
    int geocentric;         /* 0 barycentric (default), 1 geocentric */
    double alpha, nk, nm, nn, r0;   /* Marsden g(r) law, ASSIST defaults 1,0,2,5.093,1 */
    double epsilon;         /* IAS15 tolerance (1e-9); 0 => fixed step = dt0 */
    double min_dt;          /* IAS15 minimum |dt| (0 => none) */
    double dt0;             /* initial |dt| (REBOUND default 0.001 day) */
    int max_steps;          /* per-particle step budget, 0 => unlimited */
    int warm_start;         /* 0 plain predictor; 1 learned warm start (needs a network, see
                               assist_gb300_warm_*; group_steps = 2), except for batches whose
                               signature assist_gb300_autotune_device recorded the plain predictor
                               faster on; 2 learned warm start regardless.  Every 8th step of a
                               group is a plain probe; a member whose learned starts converge in
                               more iterations than its probes, and a group whose learned steps
                               take longer than its probes, fall back to the plain predictor.
                               3: as 2 without the group's time test (what the network saves in
                               iterations, whatever it costs) */
    int threads_per_block;  /* group_steps 0: 0 => 128, halved (down to 32) while the batch would
                               leave SMs idle */
    int group_steps;        /* 1: up to 32 particles with the same start time and similar
                               orbital timescale share each adaptive step (one warp);
                               2 (default): the same groups, each integrated by a 128-thread
                               block whose four warps split every force evaluation;
                               0: every particle takes its own adaptive step */
    double dt_floor;        /* a particle whose adaptive step falls below this |dt| (days)
                               stops with ASSIST_GB300_STEP_UNDERFLOW (an impact: any orbit
                               outside a body needs steps > 1e-4 day); 0 disables */
    int group_order;        /* how groups are formed (group_steps 1, 2): 0 (default) perihelion
                               distance, length, eccentricity in eighths, then time of pericentre
                               passage; 1 orbit size, length, then mean anomaly; 2 as 0 without
                               the eccentricity key */
    int blocks_per_sm;      /* group_steps 2 without variational particles or warm start:
                               0 (default) three resident blocks per SM when the batch has at
                               least 8 groups per such block, else two; 2 or 3 force it */
    int ephem_staging;      /* group_steps 2 without variational particles or warm start, .440
                               planets: 0 (default) the library's choice; 1 each block keeps its
                               group's active .440 record in shared memory, staged by bulk (TMA)
                               copies (two resident blocks per SM); 2 coefficients read from
                               global memory */
};

/* Fill `opt` with ASSIST's defaults (src/assist.c:408-447). */
void assist_gb300_default_options(struct assist_gb300_options* opt);

/* Per-particle result status word of the batched integrator. */
enum ASSIST_GB300_PARTICLE_STATUS {
    ASSIST_GB300_OK = 0,
    ASSIST_GB300_COVERAGE = 1,      /* a substep time fell outside the ephemeris */
    ASSIST_GB300_NONFINITE = 2,     /* NaN/Inf in state or acceleration */
    ASSIST_GB300_STEP_BUDGET = 3,   /* max_steps reached before t_end */
    ASSIST_GB300_STEP_UNDERFLOW = 4,/* the adaptive step fell below dt_floor (impact) */
    ASSIST_GB300_TIMEOUT = 5,       /* the kernel's run-time budget was spent */
};

/* Statistics returned by the batched integrator. */
struct assist_gb300_batch_stats {
    long long steps_accepted;
    long long steps_rejected;
    long long force_evals;          /* particle force evaluations (real particles) */
    long long pc_iterations;        /* predictor-corrector iterations summed over steps */
    long long warm_start_used;      /* steps whose learned start was accepted */
    long long warm_start_fallback;  /* steps that fell back to the plain predictor */
    double kernel_ms;               /* device time of the integration kernels */
    long long tables_built;         /* body tables evaluated (all bodies at one time): one per
                                       evaluation with independent steps, one per group and
                                       node time with shared steps */
};

/* Integrate n independent test particles, each from t0[i] to t_end[i] (days
 * relative to ephem->jd_ref) with its own adaptive IAS15 step.
 *   state  : host array n*6 doubles (x,y,z,vx,vy,vz), overwritten with the end state
 *   params : host array n*3 (A1,A2,A3 non-grav) or NULL
 *   n_var  : 0 or 6; with 6, `var_state` holds n*6*6 doubles (6 first-order
 *            variational states per particle) and is overwritten at the end
 *   status : host array n ints (ASSIST_GB300_PARTICLE_STATUS), may be NULL
 * Returns ASSIST_SUCCESS or an ASSIST_STATUS error. */
int assist_gb300_integrate_batch(const struct assist_ephem* ephem, const struct assist_gb300_options* opt,
                                 int n, const double* t0, const double* t_end,
                                 double* state, const double* params,
                                 int n_var, double* var_state,
                                 int* status, struct assist_gb300_batch_stats* stats);

/* Same as assist_gb300_integrate_batch but every array is a DEVICE pointer on
 * the current CUDA device and the call is asynchronous on `stream`
 * (cudaStream_t passed as void*).  `stats` (host) is filled after an internal
 * stream synchronisation when non-NULL. */
int assist_gb300_integrate_batch_device(const struct assist_ephem* ephem, const struct assist_gb300_options* opt,
                                        int n, const double* d_t0, const double* d_t_end,
                                        double* d_state, const double* d_params,
                                        int n_var, double* d_var_state,
                                        int* d_status, void* stream,
                                        struct assist_gb300_batch_stats* stats);

/* Batched IAS15 with dense output: as assist_gb300_integrate_batch_device
 * (group_steps = 2, no variational particles) and, on the way, particle i's
 * state at each of its output times d_out_t[d_out_start[i] ..
 * d_out_start[i+1]) into d_out_state (6 doubles each), interpolated from the
 * IAS15 step that contains the time as ASSIST's assist_integrate_or_interpolate
 * does for one simulation (src/assist.c:556-597, 642-680).  Output times lie
 * within [t0, t_end] of their particle, in the order of integration
 * (ASSIST_ERROR_N otherwise); d_out_start has n + 1 entries from 0.  A
 * particle that stops early (status != 0) leaves NaN at the times it did not
 * reach. */
int assist_gb300_integrate_batch_dense_device(const struct assist_ephem* ephem, const struct assist_gb300_options* opt,
                                              int n, const double* d_t0, const double* d_t_end, double* d_state,
                                              const double* d_params, const int* d_out_start, const double* d_out_t,
                                              double* d_out_state, int* d_status, void* stream,
                                              struct assist_gb300_batch_stats* stats);

/* Batched IAS15 that allocates nothing (no counterpart in the reference).
 * Same integration as assist_gb300_integrate_batch_device with
 * group_steps = 0 and n_var = 0 (independent per-particle steps, identical
 * end states), for callers that cannot allocate device memory at call time:
 * a process whose free device memory is already claimed by another
 * allocator, or a loop that must not take the implicit device-wide
 * synchronisation of cudaFree.  Its scratch (queue, counters, workspace) is
 * one fixed __device__ array of ASSIST_GB300_STATIC_SCRATCH_BYTES per device;
 * n above ASSIST_GB300_STATIC_MAX_PARTICLES is rejected with
 * ASSIST_ERROR_N.  opt->group_steps is ignored (always independent steps);
 * warm_start must be 0.  Particles are taken in index order (the
 * allocating entry point queues the longest integrations first), which can
 * leave a long integration near the end of a large batch running alone.
 * The ephemeris must already have a device view that matches its current
 * contents (one ordinary device call with it first, and again after editing
 * jd_ref or a constant): this entry point neither allocates nor uploads one
 * and refuses a stale one.  The first call on a device looks up
 * the scratch address and uploads the IAS15 tables: make it before any stream
 * capture.  One scratch per device: calls that overlap in time on one device
 * (other streams or threads) race on it and must be serialised by the caller.
 * stats->kernel_ms is -1 (not timed). */
#define ASSIST_GB300_STATIC_SCRATCH_BYTES (32 << 20)
#define ASSIST_GB300_STATIC_MAX_PARTICLES 1048576
int assist_gb300_integrate_batch_device_static(const struct assist_ephem* ephem,
                                               const struct assist_gb300_options* opt, int n,
                                               const double* d_t0, const double* d_t_end, double* d_state,
                                               const double* d_params, int* d_status, void* stream,
                                               struct assist_gb300_batch_stats* stats);

/* Plans: one batch integrated repeatedly (no counterpart in the reference).
 * assist_gb300_plan_create does the host work of an assist_gb300_integrate_
 * batch_device call once -- inputs read back, encounter pilot, grouping, the
 * kernel build -- from the arrays' current contents, and captures the device
 * work (queue and counter reset, the persistent kernel, the counters' copy
 * to host memory) as a CUDA graph.  Each assist_gb300_plan_launch replays it
 * on `stream` over the same device arrays: write the next initial states
 * (and times, if they keep the grouping's meaning) into them between
 * launches.  A replay gives the result of a direct call whose grouping is
 * the plan's (bit for bit when the inputs are the ones the plan was made
 * from).  No dense output or pair logging.  assist_gb300_plan_stats waits
 * for the last launch and returns its counters (kernel_ms -1: time launches
 * with events on their stream).  A plan belongs to the device that was
 * current at its creation. */
struct assist_gb300_plan;
int assist_gb300_plan_create(const struct assist_ephem* ephem, const struct assist_gb300_options* opt, int n,
                             const double* d_t0, const double* d_t_end, double* d_state, const double* d_params,
                             int n_var, double* d_var_state, int* d_status, void* stream,
                             struct assist_gb300_plan** plan);
int assist_gb300_plan_launch(struct assist_gb300_plan* plan, void* stream);
int assist_gb300_plan_stats(struct assist_gb300_plan* plan, struct assist_gb300_batch_stats* stats);
void assist_gb300_plan_free(struct assist_gb300_plan* plan);

/* Build selection of the default batched kernel (no counterpart in the
 * reference).  The block-cooperative kernel (group_steps = 2) without
 * variational particles has three builds that compute the same results: two
 * or three resident blocks per SM, and two with each block's active .440
 * record staged in shared memory by bulk copies.  This times each on the
 * caller's batch (device arrays; the state is copied, not changed), reports
 * the kernel times and records the fastest for the batch's signature
 * (device, group count, mean and longest length, non-gravitational share,
 * force model, planets format) in memory and in the file named by
 * ASSIST_GB300_TUNE_CACHE (default ~/.cache/assist_gb300/tune.txt; empty:
 * memory only).  Later calls with blocks_per_sm = 0 and ephem_staging = 0
 * use the recorded build for a batch of the same signature.  With
 * warm_start set in `opt` the learned warm-start build is a candidate too
 * (with variational particles: the plain and the learned build), and
 * warm_start = 1 calls use the plain predictor on batches of a signature
 * where it was faster.  It allocates scratch for a copy of the state (and of
 * d_var_state) and runs the batch twice per build. */
struct assist_gb300_tune_result {
    int chosen;              /* 2, 3: plain, blocks per SM; 4: plain, two with the staged .440
                                record; 5: the learned warm start */
    int n_candidates;
    int candidate[4];
    double kernel_ms[4];     /* best of two kernel times of each candidate */
    char signature[512];
};
int assist_gb300_autotune_device(const struct assist_ephem* ephem, const struct assist_gb300_options* opt, int n,
                                 const double* d_t0, const double* d_t_end, const double* d_state,
                                 const double* d_params, int n_var, const double* d_var_state, void* stream,
                                 struct assist_gb300_tune_result* result);

/* ---- Learned IAS15 warm start (no counterpart in the reference).
 * One network per process: 32 step features -> 256 -> 256 -> 21 corrections
 * of IAS15's predicted b coefficients (GELU, weights [out][in]; the flat
 * parameter order is W1, b1, W2, b2, W3, b3).  Training is FP32 on the
 * device; inference is BF16 on the tensor cores inside the batched kernel,
 * where IAS15's own convergence test and error estimate still decide and the
 * plain predictor takes over for a particle whose learned starts converge
 * slower.  Device pointers are float32, row-major. */
int assist_gb300_warm_n_params(void);
int assist_gb300_warm_init(unsigned long long seed);                 /* random weights, zero biases */
int assist_gb300_warm_set_params(const float* params, int n);        /* host array of n_params */
int assist_gb300_warm_get_params(float* params, int n);
/* Loss 1/(2n) sum (Y - T)^2 over n pairs and its gradient (host array of n_params). */
int assist_gb300_warm_grad(const float* d_x, const float* d_t, int n, float* grad, double* loss);
/* One Adam step (0.9, 0.999, 1e-8) with a given gradient (host array). */
int assist_gb300_warm_adam_step(const float* grad, float lr);
/* `steps` Adam steps on minibatches of `batch` consecutive pairs chosen at
 * random (seeded) from n pairs; *loss = last minibatch loss. */
int assist_gb300_warm_train(const float* d_x, const float* d_t, int n, int steps, int batch, float lr,
                            unsigned long long seed, double* loss);
/* BF16 tensor-core inference of n feature rows into d_y [n][21]. */
int assist_gb300_warm_infer(const float* d_x, int n, float* d_y);
/* Log (features, target) pairs of every `every`-th accepted step in the next
 * batched integrations (group_steps = 2, n_var = 0) into d_x [cap][32],
 * d_t [cap][21]; NULL stops logging.  Resets the count. */
int assist_gb300_warm_set_log(float* d_x, float* d_t, int capacity, int every);
int assist_gb300_warm_log_count(void);

/* One force evaluation for n particles at per-particle times t[i] (device
 * pointers): acc[3i..3i+2] = a(x_i, v_i, t_i) for the force model in `opt`.
 * With n_var = 6, var_state holds per-particle 6 variational states (6 doubles
 * each) and var_acc receives their accelerations.  status (device, may be NULL)
 * receives per-particle ASSIST_STATUS codes. */
int assist_gb300_forces_device(const struct assist_ephem* ephem, const struct assist_gb300_options* opt,
                               int n, const double* d_t, const double* d_state, const double* d_params,
                               int n_var, const double* d_var_state,
                               double* d_acc, double* d_var_acc, int* d_status, void* stream);

/* One force evaluation for n particles at ONE time t (device pointers), by
 * the block-cooperative evaluation the batched and the shared-step
 * integrators run: one 128-thread block per 32 particles builds the body
 * table of t once and its four warps split each particle's force terms, the
 * asteroids' terms in double-float arithmetic (within 1e-16 of the
 * acceleration).  acc[3i..3i+2] = a(x_i, v_i, t); state n*6, params n*3 or
 * NULL; status (device, may be NULL) receives ASSIST_ERROR_COVERAGE for every
 * particle when t is outside the ephemeris.  No variational particles. */
int assist_gb300_forces_shared_time_device(const struct assist_ephem* ephem, const struct assist_gb300_options* opt,
                                           int n, double t, const double* d_state, const double* d_params,
                                           double* d_acc, int* d_status, void* stream);

/* Evaluate all 11+N_ast bodies at n times (device pointers).  out holds, per
 * time, (11+N_ast) records of 10 doubles: GM, x,y,z, vx,vy,vz, ax,ay,az, with
 * the same meaning as assist_all_ephem (asteroid velocity/acceleration NaN).
 * status (device, may be NULL) receives an ASSIST_STATUS per time. */
int assist_gb300_ephem_device(const struct assist_ephem* ephem, int n, const double* d_t,
                              double* d_out, int* d_status, void* stream);

/* Close-encounter cost ratio of each particle: the IAS15 steps its close
 * planetary encounters add over [t0, t_end], as a fraction of its plain
 * steps, from the two-body pilot by which the grouped batched kernels order
 * their work queue (FP32 estimate; device arrays, d_ratio receives n floats).
 * No counterpart in the reference: a scheduling aid, e.g. to shard particles
 * across GPUs by expected cost. */
int assist_gb300_encounter_ratio_device(const struct assist_ephem* ephem, int n, const double* d_t0,
                                        const double* d_t_end, const double* d_state, float* d_ratio,
                                        void* stream);

/* The grouping of the grouped batched kernels, on host arrays and without
 * device work: order[n] receives the particles in key order, gstart[] and
 * gsize[] (room for n each) the groups of at most 32 consecutive entries of
 * order, most expensive first, *n_groups their count.  params (3 doubles per
 * particle) and ratio (the encounter pilot's output, n floats) may be NULL;
 * gm_sun is the Sun's GM in AU^3/day^2.  No counterpart in the reference. */
int assist_gb300_group_plan(int n, const double* t0, const double* t_end, const double* state, const double* params,
                            const float* ratio, int group_order, double gm_sun, int* order, int* gstart, int* gsize,
                            int* n_groups);

/* FP64 fused multiply-add throughput of the current CUDA device in GFLOP/s,
 * measured with independent FMA chains (the roofline denominator of these
 * FP64-bound kernels). */
double assist_gb300_fp64_peak_gflops(void);

/* Number of bodies (11 + asteroids) of a loaded ephemeris. */
int assist_gb300_n_bodies(const struct assist_ephem* ephem);

/* Last CUDA/library error text of this thread ("" if none). */
const char* assist_gb300_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* ASSIST_GB300_ASSIST_H */
