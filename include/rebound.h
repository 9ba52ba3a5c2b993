/*
 * rebound.h -- the subset of the REBOUND N-body API that ASSIST's equations of
 * motion are driven through, implemented by libassist_gb300 with a device
 * (sm_103a) IAS15 integrator.
 *
 * REBOUND itself is a third-party dependency of ASSIST (pinned
 * rebound>=4.4.11,<5.0.0 in setup.py:177-178; CI tag 4.6.0 in
 * .github/workflows/c.yml:19-21) and is not vendored with ASSIST.  This header
 * declares the field and function names that ASSIST touches
 * (src/assist.c:379-501, 556-758, src/forces.c:49-173, src/tools.c:32-70) so
 * that ASSIST-style C code compiles unchanged against this library.
 *
 * Compatibility statement:
 *   - struct reb_particle follows REBOUND 4.x's published layout (x..az, m, r,
 *     last_collision, c, hash, ap, sim), so a ctypes mirror of
 *     rebound.Particle reads it byte-for-byte.
 *   - struct reb_simulation is SOURCE compatible (same member names for every
 *     member ASSIST and its users touch), not binary compatible with a
 *     librebound build: it is a compact struct owned by this library.
 */
#ifndef ASSIST_GB300_REBOUND_H
#define ASSIST_GB300_REBOUND_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

struct reb_simulation;
struct reb_treecell;

/* One particle: position, velocity, acceleration (AU, AU/day, AU/day^2 under ASSIST). */
struct reb_particle {
    double x, y, z;
    double vx, vy, vz;
    double ax, ay, az;
    double m;                 /* ASSIST stores GM here for ephemeris bodies */
    double r;
    double last_collision;
    struct reb_treecell* c;
    uint32_t hash;
    void* ap;
    struct reb_simulation* sim;
};

/* A first-order variational configuration: particle `index` holds the
 * variation of real particle `testparticle` (REBOUND's test-particle variant). */
struct reb_variational_configuration {
    struct reb_simulation* sim;
    int order;
    int index;
    int testparticle;
    int index_1st_order_a;
    int index_1st_order_b;
    double lrescale;
};

/* Seven pointers to the per-node IAS15 coefficient arrays (3*N doubles each). */
struct reb_dp7 {
    double* p0;
    double* p1;
    double* p2;
    double* p3;
    double* p4;
    double* p5;
    double* p6;
};

enum REB_INTEGRATOR {
    REB_INTEGRATOR_IAS15 = 0,
    REB_INTEGRATOR_WHFAST = 1,
    REB_INTEGRATOR_SEI = 2,
    REB_INTEGRATOR_LEAPFROG = 4,
    REB_INTEGRATOR_NONE = 7,
};

enum REB_GRAVITY {
    REB_GRAVITY_NONE = 0,
    REB_GRAVITY_BASIC = 1,
};

/* Simulation status: negative while running, 0 on success, >0 on error. */
enum REB_STATUS {
    REB_STATUS_PAUSED = -3,
    REB_STATUS_LAST_STEP = -2,
    REB_STATUS_RUNNING = -1,
    REB_STATUS_SUCCESS = 0,
    REB_STATUS_GENERIC_ERROR = 1,
    REB_STATUS_NO_PARTICLES = 2,
    REB_STATUS_ENCOUNTER = 3,
    REB_STATUS_ESCAPE = 4,
    REB_STATUS_USER = 5,
    REB_STATUS_SIGINT = 6,
    REB_STATUS_COLLISION = 7,
};

enum reb_simulation_binary_error_codes {
    REB_SIMULATION_BINARY_WARNING_NONE = 0,
};

/* IAS15 integrator state.  `br`, `x0`, `v0`, `a0` hold the last completed
 * step in host memory after every step (ASSIST's interpolation reads them,
 * src/assist.c:556-597, 682-751). */
struct reb_simulation_integrator_ias15 {
    double epsilon;                 /* 0 => fixed step */
    double min_dt;
    unsigned int adaptive_mode;     /* 0 individual, 1 global (ASSIST sets 1) */
    unsigned long iterations_max_exceeded;
    int N_allocated;
    double* x0;
    double* v0;
    double* a0;
    struct reb_dp7 br;              /* b coefficients of the last accepted step */
    double dt_last_success;
};

struct reb_simulationarchive {
    long nblobs;
    double* t;
};

struct reb_simulation {
    double t;
    double G;
    double dt;
    double dt_last_done;
    unsigned long long steps_done;
    int N;
    int N_var;
    int N_var_config;
    int N_active;
    int N_allocated;
    int N_allocated_var_config;
    struct reb_variational_configuration* var_config;
    struct reb_particle* particles;
    int exact_finish_time;
    int force_is_velocity_dependent;
    int status;
    enum REB_INTEGRATOR integrator;
    enum REB_GRAVITY gravity;
    struct reb_simulation_integrator_ias15 ri_ias15;
    void (*additional_forces)(struct reb_simulation* const r);
    void (*pre_timestep_modifications)(struct reb_simulation* const r);
    void (*post_timestep_modifications)(struct reb_simulation* const r);
    void* extras;
    void (*extras_cleanup)(struct reb_simulation* const r);
    char error_message[1024];
    void* gb300;                    /* device integrator state (library-owned) */
};

struct reb_simulation* reb_simulation_create(void);
void reb_simulation_free(struct reb_simulation* r);
void reb_simulation_add(struct reb_simulation* r, struct reb_particle pt);
int reb_simulation_add_variation_1st_order(struct reb_simulation* r, int testparticle);
int reb_simulation_integrate(struct reb_simulation* r, double tmax);
void reb_simulation_step(struct reb_simulation* r);
void reb_simulation_update_acceleration(struct reb_simulation* r);
void reb_simulation_error(struct reb_simulation* r, const char* msg);
void reb_simulation_warning(struct reb_simulation* r, const char* msg);

#ifdef __cplusplus
}
#endif

#endif /* ASSIST_GB300_REBOUND_H */
