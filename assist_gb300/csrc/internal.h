/*
 * internal.h -- host-side declarations shared by the library's translation units.
 */
#ifndef ASSIST_GB300_INTERNAL_H
#define ASSIST_GB300_INTERNAL_H

#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "device_ephem.cuh"

#include <nvtx3/nvToolsExt.h>

/* A named NVTX range over a host scope (the phases of a batched call show
 * in a profiler's timeline; without a profiler attached it costs nothing). */
struct AgRange {
    explicit AgRange(const char* name) { nvtxRangePushA(name); }
    ~AgRange() { nvtxRangePop(); }
    AgRange(const AgRange&) = delete;
    AgRange& operator=(const AgRange&) = delete;
};

struct ForceCfg;

/* Particle I/O of the shared-time force kernel (one REBOUND simulation). */
struct AgForceIO {
    int n_real;             /* real particles (slots 0..n_real-1) */
    int stride;             /* SoA stride of x, v, a (>= particle count) */
    const double* x;        /* [3][stride] positions of all particles */
    const double* v;        /* [3][stride] velocities */
    double* a;              /* [3][stride] accelerations (written) */
    const double* params;   /* 3*(n_real + n_var_config) Marsden parameters, or null */
    const int* var_start;   /* n_real+1 offsets into var_index/var_cfg, or null */
    const int* var_index;   /* particle slot of each variational particle */
    const int* var_cfg;     /* its var_config index (row n_real + cfg of params) */
    int* status;            /* one int, atomically max-ed with an ASSIST status */
};

#define AG_SM_SLOTS 1024

/* Device-side state of the batched integrator. */
struct AgBatchArgs {
    int n;                          /* particles */
    int nslots;                     /* persistent threads */
    const int* order;               /* queue order (indices into the particle arrays) */
    int* queue;                     /* next queue position (atomic) */
    const double* t0;
    const double* t_end;
    double* state;                  /* [n][6], overwritten with the end state */
    const double* params;           /* [n][3] or null */
    double* var_state;              /* [n][NV][6] */
    int* status;                    /* [n] or null */
    double* ws;                     /* per-slot workspace, see kernels_ias15.cu */
    unsigned long long* counters;   /* accepted, rejected, evals, iterations, warm used, warm fallback, tables */
    int* sm_slots;                  /* AG_SM_SLOTS per-SM block counters, zero at launch (block-cooperative
                                       kernel's role rotation), or null */
    double epsilon, min_dt, dt0, dt_floor;
    long long max_steps;
    long long watchdog_cycles;      /* per-thread clock64 budget; 0 = none */
    /* warp-synchronous groups (K4g): group g = order[grp_start[g] .. + grp_size[g]) */
    const int* grp_start;
    const int* grp_size;
    int n_groups;
    /* learned warm start (block-cooperative kernel, no variational particles) */
    const struct AgMlpDev* mlp;     /* network for the warm start, or null (plain predictor) */
    int warm_no_time_fallback;      /* keep the learned start in groups where it costs time */
    float* log_x;                   /* [log_cap][32] features of logged steps, or null */
    float* log_t;                   /* [log_cap][21] their targets */
    int* log_count;                 /* next log row (atomic) */
    int log_cap, log_every;
    /* dense output (block-cooperative kernel, no variational particles):
     * particle i's output times out_t[out_start[i] .. out_start[i+1]) */
    const int* out_start;
    const double* out_t;
    double* out_state;              /* [*][6] state at each output time */
};

/* launchers (kernels_forces.cu, kernels_ias15.cu) */
int ag_launch_forces_table(const DevEphem& E, const ForceCfg& c, double t, const AgForceIO& io, cudaStream_t s);
/* n particles (state n x 6) at one time t, block-cooperative evaluation (kernels_shared.cu) */
int ag_launch_forces_coop(const DevEphem& E, const ForceCfg& c, int n, double t, const double* state,
                          const double* params, double* acc, int* status, cudaStream_t s);
int ag_launch_forces_each(const DevEphem& E, const ForceCfg& c, int n, const double* t, const double* state,
                          const double* params, int nv, const double* var_state, double* acc, double* var_acc,
                          int* status, cudaStream_t s);
int ag_launch_bodies(const DevEphem& E, int n, const double* t, double* out, int* status, cudaStream_t s);
size_t ag_batch_ws_doubles(int nslots, int nv);
int ag_launch_batch(const DevEphem& E, const ForceCfg& c, const AgBatchArgs& a, int nv, int tpb, cudaStream_t s);
int ag_batch_max_slots(int nv, int tpb);
int ag_group_max_slots(int nv);
int ag_launch_group(const DevEphem& E, const ForceCfg& c, const AgBatchArgs& a, int nv, cudaStream_t s);
int ag_coop_max_slots(int nv, int occ, int stage, int warm);
/* Per-particle encounter cost ratio (extra steps / base steps) from a
 * two-body pilot on a G-point time grid over [tmin, tmax]. */
int ag_pilot_encounters(const DevEphem& E, int n, const double* d_t0, const double* d_te, const double* d_state,
                        double tmin, double tmax, float* d_ratio, float4* d_grid, float2* d_sunv, int G,
                        cudaStream_t s);
int ag_launch_coop(const DevEphem& E, const ForceCfg& c, const AgBatchArgs& a, int nv, int occ, int stage,
                   cudaStream_t s);
double ag_fp64_probe_gflops(void);
/* first-use set-up of the batched kernels (tables, shared-memory opt-ins), ahead of a stream capture */
int ag_batch_ready(void);
int ag_coop_ready(void);

/* shared-step device IAS15 (kernels_shared.cu) */
struct AgSharedSim;
AgSharedSim* ag_shared_create(void);
void ag_shared_free(AgSharedSim* s);

struct assist_gb300_options;
ForceCfg ag_make_cfg(const struct assist_gb300_options* o);

struct assist_ephem;
/* The device view of an ephemeris (uploaded on first use). */
int ag_ephem_device(const struct assist_ephem* e, DevEphem* out);

/* The device view of an ephemeris that already has one matching its current
 * contents, without allocating or uploading anything (an error otherwise). */
int ag_ephem_device_current(const struct assist_ephem* e, DevEphem* out);

/* 1 when the ephemeris's device view exists (ag_ephem_device will not allocate) */
int ag_ephem_view_ready(const struct assist_ephem* e);

/* warm-start network (kernels_mlp.cu) */
const struct AgMlpDev* ag_mlp_device_view(void);
int ag_mlp_log_config(float** x, float** t, int* cap, int* every, int** count);

/* build selection of the block-cooperative kernel (autotune.cpp): a batch's
 * signature, the recorded build for it (0 none; 2, 3 blocks per SM; 4 two
 * with the staged record) and the signature of the last batch formed */
std::string ag_tune_key(int n_groups, int n, const double* t0, const double* te, const unsigned char* has_ng,
                        int forces, int gr_eih_sources, int geocentric, int planets_spk);
int ag_tune_lookup(const std::string& key);
void ag_tune_note(const std::string& key);

/* library error state */
void ag_set_error(const std::string& msg);
int ag_cuda_check(cudaError_t e, const char* what);

#endif
