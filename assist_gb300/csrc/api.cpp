/*
 * api.cpp -- the C ABI: ASSIST's plugin surface (src/assist.h), the REBOUND
 * subset it is driven through, and the batched entry points.
 *
 * Every compute call goes to the device; a missing or failing CUDA device is
 * reported as an error (ASSIST status / sim->status / return code), never
 * answered on the CPU.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/assist.h"
#include "device_forces.cuh"
#include "internal.h"
#include "shared_sim.h"

#define AG_STR2(s) #s
#define AG_STR(s) AG_STR2(s)
#ifndef ASSIST_GB300_GITHASH
#define ASSIST_GB300_GITHASH notavailable
#endif

extern "C" {
const char* assist_build_str = __DATE__ " " __TIME__;
const char* assist_version_str = "1.2.0";
const char* assist_githash_str = AG_STR(ASSIST_GB300_GITHASH);
const char* assist_error_messages[] = {
    "No error has occured.",
    "The JPL planet ephemeris file has not been found.",
    "The JPL asteroid ephemeris file has not been found. Asteroid forces have been disabled.",
    "The requested asteroid ID has not been found.",
    "The requested planet ID has not been found.",
    "The requested time is outside the coverage provided by the ephemeris file.",
};
const int assist_error_messages_N = ASSIST_ERROR_N;
}

int ag_ephem_device(const struct assist_ephem* e, DevEphem* out);
int ag_ephem_n_bodies(const struct assist_ephem* e);
double ag_sun_gm(const struct assist_ephem* e);

/* ---------------------------------------------------------------- errors */
static thread_local std::string g_last_error;
void ag_set_error(const std::string& msg) { g_last_error = msg; }
int ag_cuda_check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return 0;
    ag_set_error(std::string(what) + ": " + cudaGetErrorString(e));
    std::fprintf(stderr, "(ASSIST gb300) %s: %s\n", what, cudaGetErrorString(e));
    return 1;
}
extern "C" const char* assist_gb300_last_error(void) { return g_last_error.c_str(); }

/* ---------------------------------------------------------------- force config */
static ForceCfg make_cfg(int forces, int gr, int geo, double alpha, double nk, double nm, double nn, double r0) {
    ForceCfg c;
    std::memset(&c, 0, sizeof(c));
    c.forces = forces;
    c.gr_eih_sources = gr < 0 ? 0 : (gr > ASSIST_BODY_NPLANETS ? ASSIST_BODY_NPLANETS : gr);
    c.geocentric = geo;
    c.alpha = alpha; c.nk = nk; c.nm = nm; c.nn = nn; c.r0 = r0;
    c.nongrav_rm2 = (nm == 2.0 && nk == 0.0) ? 1 : 0;
    /* pole directions exactly as ASSIST forms them (src/forces.c:484-490, 670-676) */
    const double rae = 0.0 * M_PI / 180., dece = 90.0 * M_PI / 180.;
    c.e_ca = std::cos(rae); c.e_sa = std::sin(rae); c.e_cd = std::cos(dece); c.e_sd = std::sin(dece);
    const double ras = 286.13 * M_PI / 180., decs = 63.87 * M_PI / 180.;
    c.s_ca = std::cos(ras); c.s_sa = std::sin(ras); c.s_cd = std::cos(decs); c.s_sd = std::sin(decs);
    return c;
}

/* The force configuration of a set of batch options (used by the other
 * translation units' entry points). */
ForceCfg ag_make_cfg(const struct assist_gb300_options* o) {
    return make_cfg(o->forces, o->gr_eih_sources, o->geocentric, o->alpha, o->nk, o->nm, o->nn, o->r0);
}
static ForceCfg cfg_of(const struct assist_extras* ax) {
    return make_cfg(ax->forces, ax->gr_eih_sources, ax->geocentric, ax->alpha, ax->nk, ax->nm, ax->nn, ax->r0);
}

/* ---------------------------------------------------------------- bodies */
struct BodyScratch {
    double* d_t = nullptr;
    double* d_out = nullptr;
    int* d_st = nullptr;
    int cap = 0;
};
static std::mutex g_body_mu;
static BodyScratch g_body;

extern "C" int ag_bodies_at(const struct assist_ephem* e, double t, double* out_all) {
    DevEphem D;
    int st = ag_ephem_device(e, &D);
    if (st) return st;
    const int nb = ag_ephem_n_bodies(e);
    std::lock_guard<std::mutex> lk(g_body_mu);
    if (g_body.cap < nb) {
        if (g_body.d_out) cudaFree(g_body.d_out);
        if (!g_body.d_t && ag_cuda_check(cudaMalloc(&g_body.d_t, sizeof(double)), "cudaMalloc")) return ASSIST_ERROR_EPHEM_FILE;
        if (!g_body.d_st && ag_cuda_check(cudaMalloc(&g_body.d_st, sizeof(int)), "cudaMalloc")) return ASSIST_ERROR_EPHEM_FILE;
        if (ag_cuda_check(cudaMalloc(&g_body.d_out, sizeof(double) * 10 * nb), "cudaMalloc")) return ASSIST_ERROR_EPHEM_FILE;
        g_body.cap = nb;
    }
    cudaMemcpy(g_body.d_t, &t, sizeof(double), cudaMemcpyHostToDevice);
    cudaMemset(g_body.d_st, 0, sizeof(int));
    if (ag_cuda_check((cudaError_t)ag_launch_bodies(D, 1, g_body.d_t, g_body.d_out, g_body.d_st, 0), "body kernel"))
        return ASSIST_ERROR_EPHEM_FILE;
    int hst = 0;
    if (ag_cuda_check(cudaMemcpy(out_all, g_body.d_out, sizeof(double) * 10 * nb, cudaMemcpyDeviceToHost), "body kernel") ||
        ag_cuda_check(cudaMemcpy(&hst, g_body.d_st, sizeof(int), cudaMemcpyDeviceToHost), "body kernel"))
        return ASSIST_ERROR_EPHEM_FILE;
    return hst;
}

extern "C" int assist_all_ephem(const struct assist_ephem* ephem, struct assist_ephem_cache* cache, const int i,
                                const double t, double* const GM, double* const x, double* const y, double* const z,
                                double* const vx, double* const vy, double* const vz, double* const ax,
                                double* const ay, double* const az) {
    (void)cache;
    const int nb = ag_ephem_n_bodies(ephem);
    if (i < 0 || i >= nb) {
        if (i >= ASSIST_BODY_NPLANETS && !ephem->spk_asteroids) return ASSIST_ERROR_AST_FILE;
        return i < ASSIST_BODY_NPLANETS ? ASSIST_ERROR_NEPHEM : ASSIST_ERROR_NAST;
    }
    std::vector<double> all((size_t)nb * 10);
    int st = ag_bodies_at(ephem, t, all.data());
    /* a body's own coverage decides, as the per-body reference call does */
    const double* o = all.data() + 10 * (size_t)i;
    *GM = o[0];
    if (st != ASSIST_SUCCESS) {
        double tb, te;
        assist_ephem_time_bounds(ephem, &tb, &te);
        if (st == ASSIST_ERROR_COVERAGE) return st;
        return st;
    }
    *x = o[1]; *y = o[2]; *z = o[3]; *vx = o[4]; *vy = o[5]; *vz = o[6]; *ax = o[7]; *ay = o[8]; *az = o[9];
    return ASSIST_SUCCESS;
}

extern "C" struct reb_particle assist_get_particle_with_error(const struct assist_ephem* ephem, const int id,
                                                              const double t, int* error) {
    struct reb_particle p;
    std::memset(&p, 0, sizeof(p));
    double GM = 0;
    *error = assist_all_ephem(ephem, nullptr, id, t, &GM, &p.x, &p.y, &p.z, &p.vx, &p.vy, &p.vz, &p.ax, &p.ay, &p.az);
    p.m = GM;
    return p;
}

extern "C" struct reb_particle assist_get_particle(const struct assist_ephem* ephem, const int id, const double t) {
    int error = 0;
    struct reb_particle p = assist_get_particle_with_error(ephem, id, t, &error);
    if (error != ASSIST_SUCCESS) {
        std::fprintf(stderr, "(ASSIST) An error occured while trying to initialize particle from ephemeris data.\n");
        std::fprintf(stderr, "(ASSIST) %s\n", assist_error_messages[error]);
    }
    return p;
}

/* ---------------------------------------------------------------- extras */
static std::mutex g_ws_mu;
static std::map<const void*, AgSharedSim*> g_ws;   /* per assist_extras device workspace */

static AgSharedSim* workspace(const struct assist_extras* ax) {
    std::lock_guard<std::mutex> lk(g_ws_mu);
    auto it = g_ws.find(ax);
    if (it != g_ws.end()) return it->second;
    AgSharedSim* s = ag_shared_create();
    g_ws[ax] = s;
    return s;
}
static void workspace_free(const struct assist_extras* ax) {
    std::lock_guard<std::mutex> lk(g_ws_mu);
    auto it = g_ws.find(ax);
    if (it == g_ws.end()) return;
    ag_shared_free(it->second);
    g_ws.erase(it);
}

static void assist_extras_cleanup(struct reb_simulation* sim) {
    struct assist_extras* a = (struct assist_extras*)sim->extras;
    if (a) a->sim = nullptr;
}

extern "C" void assist_init(struct assist_extras* assist, struct reb_simulation* sim, struct assist_ephem* ephem) {
    assist->sim = sim;
    assist->ephem_cache = nullptr;
    assist->gr_eih_sources = 1;
    assist->ephem = ephem;
    assist->particle_params = nullptr;
    assist->forces = ASSIST_FORCE_SUN | ASSIST_FORCE_PLANETS | ASSIST_FORCE_ASTEROIDS | ASSIST_FORCE_NON_GRAVITATIONAL |
                     ASSIST_FORCE_EARTH_HARMONICS | ASSIST_FORCE_SUN_HARMONICS | ASSIST_FORCE_GR_EIH;
    assist->last_state = nullptr;
    assist->current_state = nullptr;
    assist->alpha = 1.0;
    assist->nk = 0.0;
    assist->nm = 2.0;
    assist->nn = 5.093;
    assist->r0 = 1.0;
    sim->integrator = REB_INTEGRATOR_IAS15;
    sim->gravity = REB_GRAVITY_NONE;
    sim->extras = assist;
    sim->extras_cleanup = assist_extras_cleanup;
    sim->additional_forces = assist_additional_forces;
    sim->force_is_velocity_dependent = 1;
    sim->ri_ias15.adaptive_mode = 1;
}

extern "C" struct assist_extras* assist_attach(struct reb_simulation* sim, struct assist_ephem* ephem) {
    if (!sim) {
        std::fprintf(stderr, "(ASSIST) Error: Simulation pointer passed to assist_attach was NULL.\n");
        return nullptr;
    }
    int own = 0;
    if (!ephem) {
        ephem = assist_ephem_create(nullptr, nullptr);
        if (!ephem) {
            std::fprintf(stderr, "(ASSIST) Error: Ephemeris pointer passed to assist_attach was NULL. Initialization with default path failed.\n");
            return nullptr;
        }
        own = 1;
    }
    struct assist_extras* a = (struct assist_extras*)std::calloc(1, sizeof(*a));
    assist_init(a, sim, ephem);
    a->extras_should_free_ephem = own;
    return a;
}

extern "C" void assist_detach(struct reb_simulation* sim, struct assist_extras* assist) {
    if (assist->sim) {
        sim->extras = nullptr;
        sim->extras_cleanup = nullptr;
        sim->additional_forces = nullptr;
        sim->pre_timestep_modifications = nullptr;
    }
    assist->sim = nullptr;
}

extern "C" void assist_free_pointers(struct assist_extras* assist) {
    if (assist->sim) {
        assist_detach(assist->sim, assist);
        assist->sim = nullptr;
    }
    std::free(assist->last_state);
    assist->last_state = nullptr;
    std::free(assist->current_state);
    assist->current_state = nullptr;
    workspace_free(assist);
    if (assist->extras_should_free_ephem && assist->ephem) {
        assist_ephem_free(assist->ephem);
        assist->ephem = nullptr;
    }
}

extern "C" void assist_free(struct assist_extras* assist) {
    if (!assist) return;
    assist_free_pointers(assist);
    std::free(assist);
}

extern "C" void assist_error(struct assist_extras* assist, const char* const msg) {
    if (assist->sim == nullptr)
        std::fprintf(stderr, "(ASSIST) Error: A Simulation is no longer attached to the ASSIST extras instance. Most likely the Simulation has been freed.\n");
    else
        reb_simulation_error(assist->sim, msg);
}

/* REBOUND's additional_forces callback: every particle of the simulation at
 * sim->t on the device, accelerations added into sim->particles. */
extern "C" void assist_additional_forces(struct reb_simulation* sim) {
    struct assist_extras* ax = (struct assist_extras*)sim->extras;
    if (!ax || !ax->ephem) return;
    DevEphem D;
    int st = ag_ephem_device(ax->ephem, &D);
    if (st != ASSIST_SUCCESS) {
        reb_simulation_error(sim, assist_error_messages[st]);
        sim->status = REB_STATUS_GENERIC_ERROR;
        return;
    }
    const ForceCfg c = cfg_of(ax);
    int fst = 0;
    if (ag_shared_forces(workspace(ax), D, c, sim, ax->particle_params, &fst)) {
        reb_simulation_error(sim, ("(ASSIST gb300) device error: " + g_last_error).c_str());
        sim->status = REB_STATUS_GENERIC_ERROR;
        return;
    }
    if (fst != ASSIST_SUCCESS) {
        reb_simulation_error(sim, assist_error_messages[fst < ASSIST_ERROR_N ? fst : ASSIST_ERROR_COVERAGE]);
        sim->status = REB_STATUS_GENERIC_ERROR;
    }
}

/* ---------------------------------------------------------------- REBOUND subset */
extern "C" struct reb_simulation* reb_simulation_create(void) {
    struct reb_simulation* r = (struct reb_simulation*)std::calloc(1, sizeof(*r));
    r->G = 1.0;
    r->dt = 0.001;
    r->status = REB_STATUS_RUNNING;
    r->exact_finish_time = 1;
    r->integrator = REB_INTEGRATOR_IAS15;
    r->gravity = REB_GRAVITY_BASIC;
    r->ri_ias15.epsilon = 1e-9;
    r->ri_ias15.min_dt = 0.0;
    r->ri_ias15.adaptive_mode = 2;
    return r;
}

static void free_dense(struct reb_simulation* r) {
    std::free(r->ri_ias15.x0); std::free(r->ri_ias15.v0); std::free(r->ri_ias15.a0);
    std::free(r->ri_ias15.br.p0);
    r->ri_ias15.x0 = r->ri_ias15.v0 = r->ri_ias15.a0 = nullptr;
    std::memset(&r->ri_ias15.br, 0, sizeof(r->ri_ias15.br));
    r->ri_ias15.N_allocated = 0;
}

extern "C" void reb_simulation_free(struct reb_simulation* r) {
    if (!r) return;
    if (r->extras_cleanup) r->extras_cleanup(r);
    free_dense(r);
    std::free(r->particles);
    std::free(r->var_config);
    std::free(r);
}

extern "C" void reb_simulation_add(struct reb_simulation* r, struct reb_particle p) {
    if (r->N >= r->N_allocated) {
        r->N_allocated = r->N_allocated ? 2 * r->N_allocated : 16;
        r->particles = (struct reb_particle*)std::realloc(r->particles, sizeof(struct reb_particle) * (size_t)r->N_allocated);
    }
    p.sim = r;
    r->particles[r->N++] = p;
}

extern "C" int reb_simulation_add_variation_1st_order(struct reb_simulation* r, int testparticle) {
    if (r->N_var_config >= r->N_allocated_var_config) {
        r->N_allocated_var_config = r->N_allocated_var_config ? 2 * r->N_allocated_var_config : 8;
        r->var_config = (struct reb_variational_configuration*)std::realloc(
            r->var_config, sizeof(struct reb_variational_configuration) * (size_t)r->N_allocated_var_config);
    }
    struct reb_variational_configuration* vc = &r->var_config[r->N_var_config++];
    std::memset(vc, 0, sizeof(*vc));
    vc->sim = r;
    vc->order = 1;
    vc->testparticle = testparticle;
    vc->index = r->N;
    vc->index_1st_order_a = -1;
    vc->index_1st_order_b = -1;
    vc->lrescale = 0.0;
    struct reb_particle p;
    std::memset(&p, 0, sizeof(p));
    reb_simulation_add(r, p);
    r->N_var++;
    return vc->index;
}

extern "C" void reb_simulation_error(struct reb_simulation* r, const char* msg) {
    if (!r) return;
    std::strncpy(r->error_message, msg, sizeof(r->error_message) - 1);
    r->error_message[sizeof(r->error_message) - 1] = '\0';
    std::fprintf(stderr, "REBOUND Error: %s\n", msg);
}

extern "C" void reb_simulation_warning(struct reb_simulation* r, const char* msg) {
    (void)r;
    std::fprintf(stderr, "REBOUND Warning: %s\n", msg);
}

extern "C" void reb_simulation_update_acceleration(struct reb_simulation* r) {
    for (int i = 0; i < r->N; i++) r->particles[i].ax = r->particles[i].ay = r->particles[i].az = 0.0;
    if (r->additional_forces) r->additional_forces(r);
}

static int integrate_device(struct reb_simulation* r, double tmax, long long max_steps, bool dense) {
    AgRange range("assist_gb300: shared-step IAS15");
    struct assist_extras* ax = (struct assist_extras*)r->extras;
    if (!ax || !ax->ephem || r->additional_forces != assist_additional_forces) {
        reb_simulation_error(r, "this REBOUND subset integrates only simulations with ASSIST attached");
        r->status = REB_STATUS_GENERIC_ERROR;
        return r->status;
    }
    DevEphem D;
    int st = ag_ephem_device(ax->ephem, &D);
    if (st) {
        reb_simulation_error(r, assist_error_messages[st]);
        r->status = REB_STATUS_GENERIC_ERROR;
        return r->status;
    }
    ShIntegrateOut out;
    out.max_steps = max_steps;
    if (dense) {
        const int n = r->N;
        if (r->ri_ias15.N_allocated < n) {
            free_dense(r);
            r->ri_ias15.x0 = (double*)std::calloc(3 * (size_t)n, sizeof(double));
            r->ri_ias15.v0 = (double*)std::calloc(3 * (size_t)n, sizeof(double));
            r->ri_ias15.a0 = (double*)std::calloc(3 * (size_t)n, sizeof(double));
            double* b = (double*)std::calloc(21 * (size_t)n, sizeof(double));
            double** pp[7] = {&r->ri_ias15.br.p0, &r->ri_ias15.br.p1, &r->ri_ias15.br.p2, &r->ri_ias15.br.p3,
                              &r->ri_ias15.br.p4, &r->ri_ias15.br.p5, &r->ri_ias15.br.p6};
            for (int q = 0; q < 7; q++) *pp[q] = b + (size_t)q * 3 * n;
            r->ri_ias15.N_allocated = n;
        }
        out.dense = true;
        out.dense_x0 = r->ri_ias15.x0; out.dense_v0 = r->ri_ias15.v0; out.dense_a0 = r->ri_ias15.a0;
        double* pp[7] = {r->ri_ias15.br.p0, r->ri_ias15.br.p1, r->ri_ias15.br.p2, r->ri_ias15.br.p3,
                         r->ri_ias15.br.p4, r->ri_ias15.br.p5, r->ri_ias15.br.p6};
        for (int q = 0; q < 7; q++) out.dense_b[q] = pp[q];
    }
    r->status = REB_STATUS_RUNNING;
    if (ag_shared_integrate(workspace(ax), D, cfg_of(ax), r, ax->particle_params, tmax, &out)) {
        reb_simulation_error(r, ("(ASSIST gb300) device error: " + g_last_error).c_str());
        r->status = REB_STATUS_GENERIC_ERROR;
        return r->status;
    }
    r->steps_done += (unsigned long long)out.accepted;
    ax->steps_done += (int)out.accepted;
    if (out.dt_last_done != 0.0) r->dt_last_done = out.dt_last_done;
    if (out.status > 0) {
        reb_simulation_error(r, assist_error_messages[out.status < ASSIST_ERROR_N ? out.status : ASSIST_ERROR_COVERAGE]);
        r->status = REB_STATUS_GENERIC_ERROR;
    } else {
        r->status = REB_STATUS_SUCCESS;
    }
    return r->status;
}

extern "C" int reb_simulation_integrate(struct reb_simulation* r, double tmax) {
    return integrate_device(r, tmax, 0, false);
}

/* One step of size r->dt (possibly retried with a smaller one after a
 * rejection): integrate to t + dt without forcing the end time. */
extern "C" void reb_simulation_step(struct reb_simulation* r) {
    integrate_device(r, r->t + r->dt, 1, false);
}

/* ---------------------------------------------------------------- dense output */
static void gauss_radau_eval(const double* x0, const double* v0, const double* a0, double* const b[7], double dt,
                             double h, int N, struct reb_particle* out) {
    double s[9], sv[8];
    s[0] = dt * h;
    s[1] = s[0] * s[0] / 2.;
    s[2] = s[1] * h / 3.;
    s[3] = s[2] * h / 2.;
    s[4] = 3. * s[3] * h / 5.;
    s[5] = 2. * s[4] * h / 3.;
    s[6] = 5. * s[5] * h / 7.;
    s[7] = 3. * s[6] * h / 4.;
    s[8] = 7. * s[7] * h / 9.;
    sv[0] = dt * h;
    for (int k = 1; k < 8; k++) sv[k] = (double)k * sv[k - 1] * h / (double)(k + 1);
    for (int j = 0; j < N; j++)
        for (int k = 0; k < 3; k++) {
            const int q = 3 * j + k;
            double x = s[8] * b[6][q] + s[7] * b[5][q] + s[6] * b[4][q] + s[5] * b[3][q] + s[4] * b[2][q] + s[3] * b[1][q] +
                       s[2] * b[0][q] + s[1] * a0[q] + s[0] * v0[q];
            double v = sv[7] * b[6][q] + sv[6] * b[5][q] + sv[5] * b[4][q] + sv[4] * b[3][q] + sv[3] * b[2][q] +
                       sv[2] * b[1][q] + sv[1] * b[0][q] + sv[0] * a0[q];
            (&out[j].x)[k] = x0[q] + x;
            (&out[j].vx)[k] = v0[q] + v;
        }
}

/* src/assist.c:642-680: integrate only when t is outside the last step,
 * otherwise evaluate the Gauss-Radau polynomial of the last step. */
extern "C" void assist_integrate_or_interpolate(struct assist_extras* ax, double t) {
    struct reb_simulation* sim = ax->sim;
    const int N = sim->N;
    if (!ax->current_state) {
        ax->current_state = (struct reb_particle*)std::malloc(sizeof(struct reb_particle) * (size_t)N);
        ax->last_state = (struct reb_particle*)std::malloc(sizeof(struct reb_particle) * (size_t)N);
        std::memcpy(ax->current_state, sim->particles, sizeof(struct reb_particle) * (size_t)N);
        std::memcpy(ax->last_state, sim->particles, sizeof(struct reb_particle) * (size_t)N);
    } else {
        struct reb_particle* p = sim->particles;
        sim->particles = ax->current_state;
        ax->current_state = p;
    }
    const double dts = std::copysign(1., sim->dt_last_done);
    if (dts * (sim->t - sim->dt_last_done) > dts * t || dts * t > dts * sim->t || sim->dt_last_done == 0.0) {
        sim->exact_finish_time = 0;
        /* integrate past t without forcing the end time: steps until t is inside the last step */
        const double dir = std::copysign(1.0, t - sim->t);
        while (dir * (t - sim->t) > 0 && sim->status <= 0) {
            if (sim->dt * dir <= 0) sim->dt = dir * std::fabs(sim->dt);
            integrate_device(sim, sim->t + sim->dt, 1, true);
            if (sim->status > 0) break;
        }
    }
    const double h = 1.0 - (sim->t - t) / sim->dt_last_done;
    if (sim->status > 0) {
        std::printf("Error: simulation exited with status %d.\n", sim->status);
    } else if (sim->t - t == 0.) {
        std::memcpy(ax->current_state, sim->particles, sizeof(struct reb_particle) * (size_t)N);
    } else if (h < 0.0 || h >= 1.0 || !std::isnormal(h)) {
        std::printf("Error: cannot interpolate beyond timestep bounds (h=%e).\n", h);
    } else if (sim->ri_ias15.br.p0 == nullptr) {
        std::printf("Error: cannot interpolate before first timestep is complete (h=%e).\n", h);
    } else {
        /* the polynomial of the last step, evaluated on the device from the
         * step-start state and b it holds */
        std::memcpy(ax->current_state, sim->particles, sizeof(struct reb_particle) * (size_t)N);
        if (ag_shared_interpolate(workspace(ax), N, sim->dt_last_done, h, ax->current_state)) {
            reb_simulation_error(sim, ("(ASSIST gb300) device interpolation failed: " + g_last_error).c_str());
            sim->status = REB_STATUS_GENERIC_ERROR;
        }
    }
    struct reb_particle* p = sim->particles;
    sim->particles = ax->current_state;
    ax->current_state = p;
}

/* src/assist.c:682-752: positions/velocities of sim1 advanced by h of sim2's
 * last step from sim1's stored start state. */
extern "C" int assist_interpolate_simulation(struct reb_simulation* sim1, struct reb_simulation* sim2, double h) {
    if (!sim1->ri_ias15.x0 || !sim2->ri_ias15.br.p0) return 0;
    double* b[7] = {sim2->ri_ias15.br.p0, sim2->ri_ias15.br.p1, sim2->ri_ias15.br.p2, sim2->ri_ias15.br.p3,
                    sim2->ri_ias15.br.p4, sim2->ri_ias15.br.p5, sim2->ri_ias15.br.p6};
    gauss_radau_eval(sim1->ri_ias15.x0, sim1->ri_ias15.v0, sim2->ri_ias15.a0, b, sim2->dt_last_done, h, sim1->N,
                     sim1->particles);
    sim1->t += sim2->dt_last_done * h;
    return 1;
}

/* ---------------------------------------------------------------- batched API */
extern "C" void assist_gb300_default_options(struct assist_gb300_options* o) {
    std::memset(o, 0, sizeof(*o));
    o->forces = ASSIST_FORCE_SUN | ASSIST_FORCE_PLANETS | ASSIST_FORCE_ASTEROIDS | ASSIST_FORCE_NON_GRAVITATIONAL |
                ASSIST_FORCE_EARTH_HARMONICS | ASSIST_FORCE_SUN_HARMONICS | ASSIST_FORCE_GR_EIH;
    o->gr_eih_sources = 1;
    o->geocentric = 0;
    o->alpha = 1.0; o->nk = 0.0; o->nm = 2.0; o->nn = 5.093; o->r0 = 1.0;
    o->epsilon = 1e-9;
    o->min_dt = 0.0;
    o->dt0 = 0.001;
    o->max_steps = 1000000;
    o->warm_start = 0;
    o->threads_per_block = 0;
    o->group_steps = 2;
    o->dt_floor = 1e-8;
    o->group_order = 0;
    o->blocks_per_sm = 0;
    o->ephem_staging = 0;
}

extern "C" int assist_gb300_n_bodies(const struct assist_ephem* e) { return ag_ephem_n_bodies(e); }

extern "C" int assist_gb300_ephem_device(const struct assist_ephem* e, int n, const double* d_t, double* d_out,
                                         int* d_status, void* stream) {
    DevEphem D;
    int st = ag_ephem_device(e, &D);
    if (st) return st;
    if (d_status) cudaMemsetAsync(d_status, 0, sizeof(int) * (size_t)n, (cudaStream_t)stream);
    if (ag_cuda_check((cudaError_t)ag_launch_bodies(D, n, d_t, d_out, d_status, (cudaStream_t)stream), "body kernel"))
        return ASSIST_ERROR_EPHEM_FILE;
    return ASSIST_SUCCESS;
}

extern "C" int assist_gb300_forces_device(const struct assist_ephem* e, const struct assist_gb300_options* o, int n,
                                          const double* d_t, const double* d_state, const double* d_params, int n_var,
                                          const double* d_var_state, double* d_acc, double* d_var_acc, int* d_status,
                                          void* stream) {
    if (n_var != 0 && n_var != 6) { ag_set_error("n_var must be 0 or 6"); return ASSIST_ERROR_N; }
    DevEphem D;
    int st = ag_ephem_device(e, &D);
    if (st) return st;
    const ForceCfg c = make_cfg(o->forces, o->gr_eih_sources, o->geocentric, o->alpha, o->nk, o->nm, o->nn, o->r0);
    if (ag_cuda_check((cudaError_t)ag_launch_forces_each(D, c, n, d_t, d_state, d_params, n_var, d_var_state, d_acc,
                                                         d_var_acc, d_status, (cudaStream_t)stream), "force kernel"))
        return ASSIST_ERROR_EPHEM_FILE;
    return ASSIST_SUCCESS;
}

extern "C" int assist_gb300_forces_shared_time_device(const struct assist_ephem* e, const struct assist_gb300_options* o,
                                                      int n, double t, const double* d_state, const double* d_params,
                                                      double* d_acc, int* d_status, void* stream) {
    if (n < 0 || (n > 0 && (!d_state || !d_acc))) { ag_set_error("invalid arguments"); return ASSIST_ERROR_N; }
    if (n == 0) return ASSIST_SUCCESS;
    DevEphem D;
    int st = ag_ephem_device(e, &D);
    if (st) return st;
    const ForceCfg c = make_cfg(o->forces, o->gr_eih_sources, o->geocentric, o->alpha, o->nk, o->nm, o->nn, o->r0);
    if (ag_cuda_check((cudaError_t)ag_launch_forces_coop(D, c, n, t, d_state, d_params, d_acc, d_status,
                                                         (cudaStream_t)stream), "force kernel (shared time)"))
        return ASSIST_ERROR_EPHEM_FILE;
    return ASSIST_SUCCESS;
}

struct BatchScratch {
    int* d_grp = nullptr;           /* grp_start then grp_size */
    int grp_cap = 0;
    int* d_order = nullptr;
    int* d_queue = nullptr;
    unsigned long long* d_counters = nullptr;
    double* d_ws = nullptr;
    size_t ws_cap = 0;
    int order_cap = 0;
    float* d_ratio = nullptr;       /* pilot: encounter cost ratio per particle */
    int ratio_cap = 0;
    float4* d_grid = nullptr;       /* pilot: body positions on the time grid */
    float2* d_sunv = nullptr;
    double* h_in = nullptr;         /* pinned: t0, t_end, states, parameters read back for grouping */
    size_t h_in_cap = 0;
    float* h_ratio = nullptr;       /* pinned: the pilot's ratios */
    int h_ratio_cap = 0;
};
#define AG_PILOT_G 1024
static std::mutex g_batch_mu;
static BatchScratch g_batch;

static int ag_integrate_batch(const struct assist_ephem* e, const struct assist_gb300_options* o, int n,
                              const double* d_t0, const double* d_t_end, double* d_state, const double* d_params,
                              int n_var, double* d_var_state, int* d_status, void* stream,
                              struct assist_gb300_batch_stats* stats, const int* d_out_start, const double* d_out_t,
                              double* d_out_state);

extern "C" int assist_gb300_integrate_batch_device(const struct assist_ephem* e, const struct assist_gb300_options* o,
                                                   int n, const double* d_t0, const double* d_t_end, double* d_state,
                                                   const double* d_params, int n_var, double* d_var_state, int* d_status,
                                                   void* stream, struct assist_gb300_batch_stats* stats) {
    return ag_integrate_batch(e, o, n, d_t0, d_t_end, d_state, d_params, n_var, d_var_state, d_status, stream, stats,
                              nullptr, nullptr, nullptr);
}

extern "C" int assist_gb300_integrate_batch_dense_device(const struct assist_ephem* e,
                                                         const struct assist_gb300_options* o, int n,
                                                         const double* d_t0, const double* d_t_end, double* d_state,
                                                         const double* d_params, const int* d_out_start,
                                                         const double* d_out_t, double* d_out_state, int* d_status,
                                                         void* stream, struct assist_gb300_batch_stats* stats) {
    if (!o || o->group_steps != 2) {
        ag_set_error("dense output runs in the block-cooperative kernel: group_steps = 2");
        return ASSIST_ERROR_N;
    }
    if (n <= 0) { if (stats) std::memset(stats, 0, sizeof(*stats)); return ASSIST_SUCCESS; }
    if (!d_out_start || !d_out_t || !d_out_state) { ag_set_error("dense output needs out_start, out_t and out_state"); return ASSIST_ERROR_N; }
    /* the output times of each particle must lie in its span, in the order of integration */
    std::vector<int> os((size_t)n + 1);
    std::vector<double> t0((size_t)n), te((size_t)n);
    cudaStream_t s = (cudaStream_t)stream;
    if (ag_cuda_check(cudaMemcpyAsync(os.data(), d_out_start, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s), "read out_start") ||
        ag_cuda_check(cudaMemcpyAsync(t0.data(), d_t0, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "read t0") ||
        ag_cuda_check(cudaMemcpyAsync(te.data(), d_t_end, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "read t_end") ||
        ag_cuda_check(cudaStreamSynchronize(s), "read dense output layout"))
        return ASSIST_ERROR_EPHEM_FILE;
    if (os[0] != 0) { ag_set_error("out_start[0] must be 0"); return ASSIST_ERROR_N; }
    for (int i = 0; i < n; i++)
        if (os[(size_t)i + 1] < os[(size_t)i]) { ag_set_error("out_start must be non-decreasing"); return ASSIST_ERROR_N; }
    std::vector<double> ot((size_t)os[(size_t)n]);
    if (!ot.empty() &&
        (ag_cuda_check(cudaMemcpyAsync(ot.data(), d_out_t, sizeof(double) * ot.size(), cudaMemcpyDeviceToHost, s), "read out_t") ||
         ag_cuda_check(cudaStreamSynchronize(s), "read out_t")))
        return ASSIST_ERROR_EPHEM_FILE;
    for (int i = 0; i < n; i++) {
        const double dir = te[(size_t)i] >= t0[(size_t)i] ? 1.0 : -1.0;
        double prev = t0[(size_t)i];
        for (int q = os[(size_t)i]; q < os[(size_t)i + 1]; q++) {
            const double tq = ot[(size_t)q];
            if (!(dir * (tq - prev) >= 0.0) || !(dir * (tq - te[(size_t)i]) <= 0.0)) {
                char msg[200];
                std::snprintf(msg, sizeof(msg), "particle %d: output time %.17g outside its span or out of order", i, tq);
                ag_set_error(msg);
                return ASSIST_ERROR_N;
            }
            prev = tq;
        }
    }
    return ag_integrate_batch(e, o, n, d_t0, d_t_end, d_state, d_params, 0, nullptr, d_status, stream, stats,
                              d_out_start, d_out_t, d_out_state);
}

/* Run f(i0, i1) over [0, n) on up to 16 host threads (one for small n). */
template <class F>
static void ag_parallel_for(int n, const F& f) {
    int nt = (int)std::thread::hardware_concurrency();
    nt = nt < 1 ? 1 : (nt > 16 ? 16 : nt);
    if (n < 16384) nt = 1;
    if (nt == 1) { f(0, n); return; }
    std::vector<std::thread> th;
    for (int k = 0; k < nt; k++) {
        const int a = (int)((long long)n * k / nt), b = (int)((long long)n * (k + 1) / nt);
        th.emplace_back([a, b, &f] { f(a, b); });
    }
    for (auto& x : th) x.join();
}

/* Sort key of one particle for grouping: start time, then class (direction,
 * non-gravitational parameters, timescale bucket), then the two keys within
 * a class, then index: a strict total order (the result does not depend on
 * the sort algorithm). */
struct AgGroupKey {
    double t0;
    unsigned cls;
    int idx;
    double k1, k2;          /* within a class: ascending */
    double cost;            /* expected evaluations, L q^-0.6 (1 + encounter ratio) */
    bool operator<(const AgGroupKey& b) const {
        if (t0 != b.t0) return t0 < b.t0;
        if (cls != b.cls) return cls < b.cls;
        if (k1 != b.k1) return k1 < b.k1;
        if (k2 != b.k2) return k2 < b.k2;
        return idx < b.idx;
    }
};

/* Sort in chunks on host threads, then merge the chunks pairwise. */
static void ag_parallel_sort(std::vector<AgGroupKey>& v) {
    const int n = (int)v.size();
    int nt = (int)std::thread::hardware_concurrency();
    nt = nt < 1 ? 1 : (nt > 16 ? 16 : nt);
    if (n < 16384 || nt == 1) { std::sort(v.begin(), v.end()); return; }
    std::vector<int> cut((size_t)nt + 1);
    for (int k = 0; k <= nt; k++) cut[(size_t)k] = (int)((long long)n * k / nt);
    {
        std::vector<std::thread> th;
        for (int k = 0; k < nt; k++)
            th.emplace_back([&v, &cut, k] { std::sort(v.begin() + cut[(size_t)k], v.begin() + cut[(size_t)k + 1]); });
        for (auto& x : th) x.join();
    }
    for (int w = 1; w < nt; w *= 2) {
        std::vector<std::thread> th;
        for (int k = 0; k + w < nt; k += 2 * w) {
            const int lo = cut[(size_t)k], mid = cut[(size_t)(k + w)], hi = cut[(size_t)std::min(k + 2 * w, nt)];
            th.emplace_back([&v, lo, mid, hi] { std::inplace_merge(v.begin() + lo, v.begin() + mid, v.begin() + hi); });
        }
        for (auto& x : th) x.join();
    }
}

/* Sort keys of a batch for grouping (host arrays): class, the keys within
 * a class and the base cost of every particle, sorted.  has_ng may be NULL. */
static void ag_group_keys(int n, const double* t0, const double* te, const double* st0, const unsigned char* has_ng,
                          double gm, int group_order, std::vector<AgGroupKey>& key) {
    /* groups share t0, direction and whether non-gravitational
     * parameters are present; within them particles of similar orbital
     * timescale (perihelion distance q^1.5, eighth-octave bins), similar
     * length and similar time of pericentre passage sit together; groups
     * are queued most expensive first */
    key.assign((size_t)n, AgGroupKey{});
    ag_parallel_for(n, [&](int i0, int i1) {
    for (int i = i0; i < i1; i++) {
        const double* p = &st0[6 * (size_t)i];
        const double r = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        const double v2 = p[3] * p[3] + p[4] * p[4] + p[5] * p[5];
        const double rv = p[0] * p[3] + p[1] * p[4] + p[2] * p[5];
        double ev[3];
        for (int k = 0; k < 3; k++) ev[k] = ((v2 - gm / r) * p[k] - rv * p[3 + k]) / gm;
        const double ecc = std::sqrt(ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2]);
        const double inv_a = 2.0 / r - v2 / gm;
        double q = (std::fabs(inv_a) > 1e-12) ? (1.0 - ecc) / inv_a : r;
        if (!(q > 1e-4)) q = 1e-4;
        int bucket = (int)std::floor(8.0 * std::log2(std::pow(q, 1.5)));
        if (group_order == 1) {
            /* orbit size (half octaves of a; unbound orbits last), length
             * (factors of 2), then mean anomaly in 1/64 turns */
            const double L = std::fabs(te[(size_t)i] - t0[(size_t)i]);
            int ba = 1000, bm = 0;
            if (inv_a > 1e-12 && ecc < 1.0) {
                const double a = 1.0 / inv_a;
                ba = (int)std::floor(2.0 * std::log2(a));
                const double ce = (1.0 - r * inv_a), se = rv / std::sqrt(gm * a);
                const double E = std::atan2(se, ce);
                double M = E - se;                      /* e sin E = se */
                M = M - 2.0 * M_PI * std::floor(M / (2.0 * M_PI));
                bm = (int)std::floor(64.0 * M / (2.0 * M_PI));
            }
            const int bl = (int)std::floor(std::log2(std::max(L, 1e-3)));
            bucket = ((ba + 2000) * 64 + (bl + 32)) * 64 + bm;
        }
        /* class bits: 31 backward, 30 non-gravitational, 0..29 bucket */
        const double L = std::fabs(te[(size_t)i] - t0[(size_t)i]);
        AgGroupKey& k = key[(size_t)i];
        k.t0 = t0[(size_t)i];
        k.cls = ((te[(size_t)i] >= t0[(size_t)i]) ? 0u : (1u << 31)) | ((has_ng && has_ng[(size_t)i]) ? (1u << 30) : 0u) |
                ((unsigned)(bucket + (1 << 28)) & ((1u << 30) - 1));
        k.idx = i;
        if (group_order == 1) {
            k.k1 = -L;
            k.k2 = 0.0;
        } else {
            /* within a bucket: lengths in sixteenths of an octave (longest
             * first: a group's lanes end within 4.4 % of each other), then
             * the time to the next pericentre passage (the last one for
             * backward integrations), so that the members of a group
             * reach their smallest steps together */
            double tp = 0.0;
            if (inv_a > 1e-12 && ecc < 1.0 && ecc > 1e-9) {
                const double a = 1.0 / inv_a;
                const double ce = (1.0 - r * inv_a), se = rv / std::sqrt(gm * a);
                double M = std::atan2(se, ce) - se;                  /* e sin E = se */
                M = M - 2.0 * M_PI * std::floor(M / (2.0 * M_PI));
                const double nm = std::sqrt(gm * inv_a * inv_a * inv_a);
                tp = (te[(size_t)i] >= t0[(size_t)i]) ? (2.0 * M_PI - M) / nm : M / nm;
            }
            k.k1 = -std::floor(16.0 * std::log2(std::max(L, 1e-3)));
            /* then (group_order 0) eccentricity in eighths: members of a
             * group also share the shape of their orbit, which sets how much
             * their steps vary along it (2 % fewer evaluations and 2 % less
             * kernel time on a one-year 262,144-particle mixture) */
            if (group_order == 0) k.k1 = 16.0 * k.k1 + std::floor(8.0 * std::min(std::max(ecc, 0.0), 0.999));
            k.k2 = tp;
            if (inv_a > 1e-12 && ecc < 1.0 && ecc > 1e-9 && tp > L) {
                /* an interval shorter than half an orbit without a pericentre
                 * passage: its smallest heliocentric distance, at one of its
                 * ends, sets the steps rather than q; bucket by it and order
                 * by that end */
                const double a = 1.0 / inv_a;
                const double nm = std::sqrt(gm * inv_a * inv_a * inv_a);
                if (L * nm < M_PI) {
                    const double ce = (1.0 - r * inv_a), se = rv / std::sqrt(gm * a);
                    double M = std::atan2(se, ce) - se;
                    double M1 = M + ((te[(size_t)i] >= t0[(size_t)i]) ? nm * L : -nm * L);
                    M1 = M1 - 2.0 * M_PI * std::floor(M1 / (2.0 * M_PI));
                    double E1 = M1 + ecc * std::sin(M1);
                    for (int it = 0; it < 30; it++) {
                        const double dE = (E1 - ecc * std::sin(E1) - M1) / (1.0 - ecc * std::cos(E1));
                        E1 -= dE;
                        if (std::fabs(dE) < 1e-12) break;
                    }
                    const double r1 = a * (1.0 - ecc * std::cos(E1));
                    const double rmin = std::min(r, r1);
                    k.k2 = (r1 < r) ? L : 0.0;
                    const int b2 = (int)std::floor(8.0 * std::log2(std::pow(std::max(rmin, 1e-4), 1.5)));
                    k.cls = (k.cls & (3u << 30)) | ((unsigned)(b2 + (1 << 28)) & ((1u << 30) - 1));
                }
            }
        }
        k.cost = L * std::pow(q, -0.6);
    }
    });
    ag_parallel_sort(key);
}

/* Groups of 32 from the sorted keys, most expensive first: order receives
 * the particles in key order, gstart/gsize the groups in queue order.  ratio
 * (the encounter pilot's output, per particle) may be NULL. */
static void ag_group_form(std::vector<AgGroupKey>& key, const float* ratio, int group_order, std::vector<int>& order,
                          std::vector<int>& gstart, std::vector<int>& gsize) {
    const int n = (int)key.size();
    order.resize((size_t)n);
    gstart.clear();
    gsize.clear();
    for (int i = 0; i < n; i++) order[(size_t)i] = key[(size_t)i].idx;
    if (ratio)
        for (int i = 0; i < n; i++) key[(size_t)i].cost *= 1.0 + (double)ratio[key[(size_t)i].idx];
    /* group_order 1 orders by its bucket but breaks groups only at start
     * time, direction and the non-gravitational flag */
    const unsigned brk = group_order == 1 ? (3u << 30) : ~0u;
    std::vector<double> gl;
    int i = 0;
    while (i < n) {
        const AgGroupKey& a = key[(size_t)i];
        double m = a.cost;
        int j = i + 1;
        while (j < n && j - i < 32) {
            const AgGroupKey& b = key[(size_t)j];
            if (b.t0 != a.t0 || ((b.cls ^ a.cls) & brk)) break;
            m = std::max(m, b.cost);
            j++;
        }
        gstart.push_back(i);
        gsize.push_back(j - i);
        gl.push_back(m);
        i = j;
    }
    /* most expensive group first: a particle's evaluations grow with its
     * length and shrink with perihelion distance, about L q^-0.6 (fitted
     * to per-particle IAS15 evaluation counts of a main-belt/NEO/Trojan/TNO
     * mixture), times 1 + the pilot's encounter ratio; a group costs its
     * most expensive member */
    std::vector<int> gi(gstart.size());
    for (size_t k = 0; k < gi.size(); k++) gi[k] = (int)k;
    std::stable_sort(gi.begin(), gi.end(), [&](int a, int b) { return gl[(size_t)a] > gl[(size_t)b]; });
    std::vector<int> s2(gi.size()), z2(gi.size());
    for (size_t k = 0; k < gi.size(); k++) { s2[k] = gstart[(size_t)gi[k]]; z2[k] = gsize[(size_t)gi[k]]; }
    gstart.swap(s2);
    gsize.swap(z2);
}

/* Option checks of the batched entry points. */
static int ag_batch_validate(const struct assist_gb300_options* o, int n_var) {
    if (!o) { ag_set_error("options are required"); return ASSIST_ERROR_N; }
    if (n_var != 0 && n_var != 6) { ag_set_error("n_var must be 0 or 6"); return ASSIST_ERROR_N; }
    if (!(o->dt0 > 0) || !(o->epsilon >= 0)) { ag_set_error("dt0 must be > 0 and epsilon >= 0"); return ASSIST_ERROR_N; }
    if (o->group_order < 0 || o->group_order > 2) {
        ag_set_error("group_order must be 0, 1 or 2");
        return ASSIST_ERROR_N;
    }
    if (o->warm_start < 0 || o->warm_start > 3 || (o->warm_start && o->group_steps != 2)) {
        ag_set_error("warm_start is 0, 1, 2 or 3; the learned warm start runs in the block-cooperative kernel "
                     "(group_steps = 2)");
        return ASSIST_ERROR_N;
    }
    if (o->ephem_staging < 0 || o->ephem_staging > 2 || (o->ephem_staging == 1 && o->blocks_per_sm == 3)) {
        ag_set_error("ephem_staging must be 0, 1 or 2; staging runs two blocks per SM (blocks_per_sm 0 or 2)");
        return ASSIST_ERROR_N;
    }
    if (o->warm_start && !ag_mlp_device_view()) {
        ag_set_error("warm_start = 1 needs a network (assist_gb300_warm_init, _set_params or _train first)");
        return ASSIST_ERROR_N;
    }
    return ASSIST_SUCCESS;
}

/* What a batched launch needs from the host: the device view, the force
 * model, the queue order and groups, and the kernel build.  The inputs are
 * read back through g_batch's pinned staging and the encounter pilot runs
 * in g_batch's buffers, so the caller holds g_batch_mu. */
struct AgLaunchPlan {
    DevEphem D;
    ForceCfg c;
    std::vector<int> order, gstart, gsize;
    bool grouped = false, coop = false;
    bool learned = false;           /* the warm-start build of the block-cooperative kernel */
    int occ = 2, stage = 0, tpb = 128, nslots = 0;
};

static int ag_batch_prepare(const struct assist_ephem* e, const struct assist_gb300_options* o, int n,
                            const double* d_t0, const double* d_t_end, const double* d_state, const double* d_params,
                            int n_var, cudaStream_t s, AgLaunchPlan& P) {
    AgRange range("assist_gb300: read-back, encounter pilot, grouping");
    DevEphem D;
    int st = ag_ephem_device(e, &D);
    if (st) return st;
    const ForceCfg c = make_cfg(o->forces, o->gr_eih_sources, o->geocentric, o->alpha, o->nk, o->nm, o->nn, o->r0);
    const bool grouped = o->group_steps != 0;
    /* block size (independent steps): 128 threads, halved (down to one warp)
     * while the batch would leave SMs idle */
    int tpb = o->threads_per_block > 0 ? o->threads_per_block : 128;
    if (o->threads_per_block <= 0) {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        while (tpb > 32 && (n + tpb - 1) / tpb < sms) tpb /= 2;
    }
    /* inputs read back for grouping, through pinned staging (kept between calls) */
    const size_t need_in = (size_t)n * (grouped ? 11 : 2);
    if (g_batch.h_in_cap < need_in) {
        if (g_batch.h_in) cudaFreeHost(g_batch.h_in);
        g_batch.h_in = nullptr;
        g_batch.h_in_cap = 0;
        if (ag_cuda_check(cudaMallocHost(&g_batch.h_in, sizeof(double) * need_in), "cudaMallocHost(inputs)"))
            return ASSIST_ERROR_EPHEM_FILE;
        g_batch.h_in_cap = need_in;
    }
    double* const t0 = g_batch.h_in;
    double* const te = t0 + n;
    double* const st0 = te + n;                       /* grouped only: 6n states, then 3n parameters */
    double* const prm = st0 + 6 * (size_t)n;
    if (ag_cuda_check(cudaMemcpyAsync(t0, d_t0, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "read t0") ||
        ag_cuda_check(cudaMemcpyAsync(te, d_t_end, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "read t_end"))
        return ASSIST_ERROR_EPHEM_FILE;
    /* particles with non-gravitational parameters are grouped apart: a
     * group pays for the term when any member has it */
    const bool read_prm = grouped && d_params && (c.forces & AG_F_NONGRAV);
    if (grouped) {
        if (ag_cuda_check(cudaMemcpyAsync(st0, d_state, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, s), "read state"))
            return ASSIST_ERROR_EPHEM_FILE;
        if (read_prm &&
            ag_cuda_check(cudaMemcpyAsync(prm, d_params, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s), "read params"))
            return ASSIST_ERROR_EPHEM_FILE;
    }
    if (ag_cuda_check(cudaStreamSynchronize(s), "read inputs")) return ASSIST_ERROR_EPHEM_FILE;
    for (int i = 0; i < n; i++)
        if (!std::isfinite(t0[(size_t)i]) || !std::isfinite(te[(size_t)i])) {
            ag_set_error("t0 and t_end must be finite (particle " + std::to_string(i) + ")");
            return ASSIST_ERROR_N;
        }
    std::vector<unsigned char> has_ng((size_t)n, 0);
    if (read_prm)
        for (int i = 0; i < n; i++)
            has_ng[(size_t)i] = prm[3 * (size_t)i] != 0.0 || prm[3 * (size_t)i + 1] != 0.0 || prm[3 * (size_t)i + 2] != 0.0;
    /* close-encounter pilot (queue order of the groups only): it runs on the
     * device while the host sorts the batch; its ratios are read before the
     * group costs are formed */
    const float* enc = nullptr;
    if (grouped) {
        double tmin = t0[0], tmax = t0[0];
        for (int i = 0; i < n; i++) {
            tmin = std::min(tmin, std::min(t0[(size_t)i], te[(size_t)i]));
            tmax = std::max(tmax, std::max(t0[(size_t)i], te[(size_t)i]));
        }
        if (g_batch.ratio_cap < n) {
            if (g_batch.d_ratio) cudaFree(g_batch.d_ratio);
            if (g_batch.h_ratio) cudaFreeHost(g_batch.h_ratio);
            g_batch.d_ratio = nullptr;
            g_batch.h_ratio = nullptr;
            g_batch.ratio_cap = 0;
            if (ag_cuda_check(cudaMalloc(&g_batch.d_ratio, sizeof(float) * (size_t)n), "cudaMalloc(pilot)") ||
                ag_cuda_check(cudaMallocHost(&g_batch.h_ratio, sizeof(float) * (size_t)n), "cudaMallocHost(pilot)"))
                return ASSIST_ERROR_EPHEM_FILE;
            g_batch.ratio_cap = n;
        }
        if (!g_batch.d_grid &&
            (ag_cuda_check(cudaMalloc(&g_batch.d_grid, sizeof(float4) * AG_PILOT_G * 10), "cudaMalloc(pilot grid)") ||
             ag_cuda_check(cudaMalloc(&g_batch.d_sunv, sizeof(float2) * AG_PILOT_G), "cudaMalloc(pilot grid)")))
            return ASSIST_ERROR_EPHEM_FILE;
        if (ag_cuda_check((cudaError_t)ag_pilot_encounters(D, n, d_t0, d_t_end, d_state, tmin, tmax, g_batch.d_ratio,
                                                           g_batch.d_grid, g_batch.d_sunv, AG_PILOT_G, s),
                          "pilot kernels") ||
            ag_cuda_check(cudaMemcpyAsync(g_batch.h_ratio, g_batch.d_ratio, sizeof(float) * n, cudaMemcpyDeviceToHost, s),
                          "read pilot"))
            return ASSIST_ERROR_EPHEM_FILE;
        enc = g_batch.h_ratio;
    }
    std::vector<int> order((size_t)n), gstart, gsize;
    for (int i = 0; i < n; i++) order[(size_t)i] = i;
    if (!grouped) {
        /* queue order: longest integrations first, so the last particles taken are short */
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            return std::fabs(te[(size_t)a] - t0[(size_t)a]) > std::fabs(te[(size_t)b] - t0[(size_t)b]);
        });
    } else {
        const double gm = (e->ascii_planets || e->spk_planets) ? ag_sun_gm(e) : 2.9591220828411951e-04;
        std::vector<AgGroupKey> key;
        ag_group_keys(n, t0, te, st0, has_ng.data(), gm, o->group_order, key);
        if (ag_cuda_check(cudaStreamSynchronize(s), "pilot kernels")) return ASSIST_ERROR_EPHEM_FILE;
        ag_group_form(key, enc, o->group_order, order, gstart, gsize);
    }
    int nslots, occ = 2, stage = 0;
    const bool coop = o->group_steps == 2;
    if (coop) {
        /* one 32-particle group per 128-thread block */
        /* three resident blocks per SM (the plain kernel's 168-register
         * build) when the batch has at least 8 groups per such block: the
         * throughput gain outweighs the slower longest groups; two otherwise */
        float *lx = nullptr, *lt = nullptr;
        int lcap = 0, levery = 1, *lcnt = nullptr;
        const bool log_on = ag_mlp_log_config(&lx, &lt, &lcap, &levery, &lcnt) != 0;
        const std::string key = ag_tune_key((int)gstart.size(), n, t0, te, has_ng.data(), c.forces, c.gr_eih_sources,
                                            c.geocentric, e->spk_planets ? 1 : 0) +
                                (n_var ? "|nv6" : "") + (o->warm_start ? "|warm" : "");
        ag_tune_note(key);
        int tuned = 0;
        if (o->warm_start) {
            /* the learned warm start unless the autotuner found the plain
             * predictor faster on a batch of this signature (warm_start = 1;
             * 2 runs the learned start regardless) */
            tuned = o->warm_start == 1 ? ag_tune_lookup(key) : 0;   /* 2, 3: the learned start regardless */
            P.learned = !(tuned >= 2 && tuned <= 4);
        } else if (o->ephem_staging == 0 && o->blocks_per_sm == 0) {
            tuned = ag_tune_lookup(key);
        }
        if (log_on) P.learned = true;      /* pairs are logged by the warm-start build */
        if (n_var == 0 && !P.learned) {
            if (o->ephem_staging == 1 || tuned == 4) {
                occ = 2;
                stage = e->spk_planets ? 0 : 1;
            } else if (o->blocks_per_sm == 2 || o->blocks_per_sm == 3) {
                occ = o->blocks_per_sm;
            } else if (tuned == 2 || tuned == 3) {
                occ = tuned;              /* recorded by assist_gb300_autotune_device for this signature */
            } else {
                int dev = 0, sms = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                occ = (int)gstart.size() >= 8 * 3 * sms ? 3 : 2;
            }
        }
        nslots = ag_coop_max_slots(n_var, occ, stage, P.learned ? 1 : 0);
        const int need = 32 * (int)gstart.size();
        if (nslots > need) nslots = need;
    } else if (grouped) {
        nslots = ag_group_max_slots(n_var);
        const int need = 32 * (int)gstart.size();
        if (nslots > need) nslots = ((need + 127) / 128) * 128;
    } else {
        nslots = ag_batch_max_slots(n_var, tpb);
        if (nslots > n) nslots = n;
    }
    P.D = D;
    P.c = c;
    P.order.swap(order);
    P.gstart.swap(gstart);
    P.gsize.swap(gsize);
    P.grouped = grouped;
    P.coop = coop;
    P.occ = occ;
    P.stage = stage;
    P.tpb = tpb;
    P.nslots = nslots;
    return ASSIST_SUCCESS;
}

static int ag_integrate_batch(const struct assist_ephem* e, const struct assist_gb300_options* o, int n,
                              const double* d_t0, const double* d_t_end, double* d_state, const double* d_params,
                              int n_var, double* d_var_state, int* d_status, void* stream,
                              struct assist_gb300_batch_stats* stats, const int* d_out_start, const double* d_out_t,
                              double* d_out_state) {
    int rc = ag_batch_validate(o, n_var);
    if (rc) return rc;
    if (n <= 0) { if (stats) std::memset(stats, 0, sizeof(*stats)); return ASSIST_SUCCESS; }
    cudaStream_t s = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lk(g_batch_mu);
    AgLaunchPlan P;
    if ((rc = ag_batch_prepare(e, o, n, d_t0, d_t_end, d_state, d_params, n_var, s, P))) return rc;
    const DevEphem& D = P.D;
    const ForceCfg& c = P.c;
    const std::vector<int>& order = P.order;
    const std::vector<int>& gstart = P.gstart;
    const std::vector<int>& gsize = P.gsize;
    const bool grouped = P.grouped, coop = P.coop;
    const int occ = P.occ, stage = P.stage, tpb = P.tpb, nslots = P.nslots;
    if (g_batch.order_cap < n) {
        if (g_batch.d_order) cudaFree(g_batch.d_order);
        if (ag_cuda_check(cudaMalloc(&g_batch.d_order, sizeof(int) * (size_t)n), "cudaMalloc(order)")) return ASSIST_ERROR_EPHEM_FILE;
        g_batch.order_cap = n;
    }
    const int ng = (int)gstart.size();
    if (grouped && g_batch.grp_cap < ng) {
        if (g_batch.d_grp) cudaFree(g_batch.d_grp);
        if (ag_cuda_check(cudaMalloc(&g_batch.d_grp, sizeof(int) * 2 * (size_t)ng), "cudaMalloc(groups)")) return ASSIST_ERROR_EPHEM_FILE;
        g_batch.grp_cap = ng;
    }
    /* counters: 8 words, then the per-SM block counters of the role rotation */
    const size_t cnt_bytes = 8 * sizeof(unsigned long long) + AG_SM_SLOTS * sizeof(int);
    if (!g_batch.d_queue) {
        if (ag_cuda_check(cudaMalloc(&g_batch.d_queue, sizeof(int)), "cudaMalloc") ||
            ag_cuda_check(cudaMalloc(&g_batch.d_counters, cnt_bytes), "cudaMalloc"))
            return ASSIST_ERROR_EPHEM_FILE;
    }
    const size_t wsn = ag_batch_ws_doubles(nslots, n_var);
    if (wsn > g_batch.ws_cap) {
        if (g_batch.d_ws) cudaFree(g_batch.d_ws);
        g_batch.d_ws = nullptr;
        if (ag_cuda_check(cudaMalloc(&g_batch.d_ws, sizeof(double) * wsn), "cudaMalloc(IAS15 slots)")) {
            g_batch.ws_cap = 0;
            return ASSIST_ERROR_EPHEM_FILE;
        }
        g_batch.ws_cap = wsn;
    }
    cudaMemcpyAsync(g_batch.d_order, order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s);
    if (grouped) {
        cudaMemcpyAsync(g_batch.d_grp, gstart.data(), sizeof(int) * (size_t)ng, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(g_batch.d_grp + ng, gsize.data(), sizeof(int) * (size_t)ng, cudaMemcpyHostToDevice, s);
    }
    cudaMemsetAsync(g_batch.d_queue, 0, sizeof(int), s);
    cudaMemsetAsync(g_batch.d_counters, 0, cnt_bytes, s);
    AgBatchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = n; a.nslots = nslots; a.order = g_batch.d_order; a.queue = g_batch.d_queue;
    a.t0 = d_t0; a.t_end = d_t_end; a.state = d_state; a.params = d_params; a.var_state = d_var_state;
    a.status = d_status; a.ws = g_batch.d_ws; a.counters = g_batch.d_counters;
    a.sm_slots = reinterpret_cast<int*>(g_batch.d_counters + 8);
    a.epsilon = o->epsilon; a.min_dt = o->min_dt; a.dt0 = o->dt0; a.max_steps = o->max_steps;
    a.dt_floor = o->dt_floor;
    if (grouped) { a.grp_start = g_batch.d_grp; a.grp_size = g_batch.d_grp + ng; a.n_groups = ng; }
    a.out_start = d_out_start; a.out_t = d_out_t; a.out_state = d_out_state;
    if (coop && P.learned) {
        if (o->warm_start) a.mlp = ag_mlp_device_view();
        a.warm_no_time_fallback = o->warm_start == 3 ? 1 : 0;
        float *lx = nullptr, *lt = nullptr;
        int cap = 0, every = 1, *cnt = nullptr;
        if (ag_mlp_log_config(&lx, &lt, &cap, &every, &cnt)) {
            a.log_x = lx; a.log_t = lt; a.log_cap = cap; a.log_every = every; a.log_count = cnt;
        }
    }
    /* per-thread run-time budget: ASSIST_GB300_WATCHDOG_S seconds (default 300) at the boost clock */
    double wd = 300.0;
    if (const char* w = getenv("ASSIST_GB300_WATCHDOG_S")) wd = atof(w);
    a.watchdog_cycles = wd > 0 ? (long long)(wd * 2.1e9) : 0;
    AgRange range("assist_gb300: batched IAS15 kernel");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    int le = coop ? ag_launch_coop(D, c, a, n_var, occ, stage, s)
                  : (grouped ? ag_launch_group(D, c, a, n_var, s) : ag_launch_batch(D, c, a, n_var, tpb, s));
    cudaEventRecord(e1, s);
    if (le) { cudaEventDestroy(e0); cudaEventDestroy(e1); ag_cuda_check((cudaError_t)le, "batch kernel launch"); return ASSIST_ERROR_EPHEM_FILE; }
    if (stats) {
        unsigned long long cnt[8];
        cudaMemcpyAsync(cnt, g_batch.d_counters, sizeof(cnt), cudaMemcpyDeviceToHost, s);
        if (ag_cuda_check(cudaStreamSynchronize(s), "batch kernel")) { cudaEventDestroy(e0); cudaEventDestroy(e1); return ASSIST_ERROR_EPHEM_FILE; }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        stats->steps_accepted = (long long)cnt[0];
        stats->steps_rejected = (long long)cnt[1];
        stats->force_evals = (long long)cnt[2];
        stats->pc_iterations = (long long)cnt[3];
        stats->warm_start_used = (long long)cnt[4];
        stats->warm_start_fallback = (long long)cnt[5];
        stats->tables_built = (long long)cnt[6];
        stats->kernel_ms = ms;
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    return ASSIST_SUCCESS;
}

/* ---------------------------------------------------------------- plans
 * A batch integrated again and again with the same particles' times and
 * grouping (new initial states written into the same device arrays between
 * launches: clones of an orbit, Monte Carlo samples, restarts): the host
 * work of a call (read-back, encounter pilot, sort, upload) is done once, and
 * each launch replays a CUDA graph of the device work (queue and counter
 * reset, the persistent kernel, the counters' copy to pinned host memory). */
struct assist_gb300_plan {
    int n = 0;
    int device = 0;
    AgLaunchPlan P;
    AgBatchArgs a;
    int* d_order = nullptr;
    int* d_grp = nullptr;
    int* d_queue = nullptr;
    unsigned long long* d_counters = nullptr;
    double* d_ws = nullptr;
    unsigned long long* h_counters = nullptr;     /* pinned, written by the graph */
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t last = nullptr;                  /* stream of the last launch */
    long long launches = 0;
};

extern "C" void assist_gb300_plan_free(struct assist_gb300_plan* p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->d_order) cudaFree(p->d_order);
    if (p->d_grp) cudaFree(p->d_grp);
    if (p->d_queue) cudaFree(p->d_queue);
    if (p->d_counters) cudaFree(p->d_counters);
    if (p->d_ws) cudaFree(p->d_ws);
    if (p->h_counters) cudaFreeHost(p->h_counters);
    delete p;
}

extern "C" int assist_gb300_plan_create(const struct assist_ephem* e, const struct assist_gb300_options* o, int n,
                                        const double* d_t0, const double* d_t_end, double* d_state,
                                        const double* d_params, int n_var, double* d_var_state, int* d_status,
                                        void* stream, struct assist_gb300_plan** out) {
    if (!out) { ag_set_error("plan: an output pointer is required"); return ASSIST_ERROR_N; }
    *out = nullptr;
    int rc = ag_batch_validate(o, n_var);
    if (rc) return rc;
    if (n <= 0 || !d_t0 || !d_t_end || !d_state || (n_var && !d_var_state)) {
        ag_set_error("plan: n > 0 and the batch's device arrays are required");
        return ASSIST_ERROR_N;
    }
    cudaStream_t s = (cudaStream_t)stream;
    assist_gb300_plan* p = new assist_gb300_plan();
    p->n = n;
    cudaGetDevice(&p->device);
    {
        std::lock_guard<std::mutex> lk(g_batch_mu);
        if ((rc = ag_batch_prepare(e, o, n, d_t0, d_t_end, d_state, d_params, n_var, s, p->P))) {
            delete p;
            return rc;
        }
    }
    const AgLaunchPlan& P = p->P;
    const int ng = (int)P.gstart.size();
    const size_t wsn = ag_batch_ws_doubles(P.nslots, n_var);
    bool ok = !ag_cuda_check(cudaMalloc(&p->d_order, sizeof(int) * (size_t)n), "cudaMalloc(plan order)") &&
              (!P.grouped || !ag_cuda_check(cudaMalloc(&p->d_grp, sizeof(int) * 2 * (size_t)ng), "cudaMalloc(plan groups)")) &&
              !ag_cuda_check(cudaMalloc(&p->d_queue, sizeof(int)), "cudaMalloc(plan queue)") &&
              !ag_cuda_check(cudaMalloc(&p->d_counters, 8 * sizeof(unsigned long long) + AG_SM_SLOTS * sizeof(int)),
                             "cudaMalloc(plan counters)") &&
              !ag_cuda_check(cudaMalloc(&p->d_ws, sizeof(double) * wsn), "cudaMalloc(plan IAS15 slots)") &&
              !ag_cuda_check(cudaMallocHost(&p->h_counters, 8 * sizeof(unsigned long long)), "cudaMallocHost(plan counters)") &&
              !ag_cuda_check(cudaMemcpy(p->d_order, P.order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice), "plan order") &&
              (!P.grouped ||
               (!ag_cuda_check(cudaMemcpy(p->d_grp, P.gstart.data(), sizeof(int) * (size_t)ng, cudaMemcpyHostToDevice), "plan groups") &&
                !ag_cuda_check(cudaMemcpy(p->d_grp + ng, P.gsize.data(), sizeof(int) * (size_t)ng, cudaMemcpyHostToDevice), "plan groups"))) &&
              !ag_cuda_check((cudaError_t)ag_batch_ready(), "batched kernel set-up") &&
              !ag_cuda_check((cudaError_t)ag_coop_ready(), "batched kernel set-up");
    if (!ok) { assist_gb300_plan_free(p); return ASSIST_ERROR_EPHEM_FILE; }
    AgBatchArgs& a = p->a;
    std::memset(&a, 0, sizeof(a));
    a.n = n; a.nslots = P.nslots; a.order = p->d_order; a.queue = p->d_queue;
    a.t0 = d_t0; a.t_end = d_t_end; a.state = d_state; a.params = d_params; a.var_state = d_var_state;
    a.status = d_status; a.ws = p->d_ws; a.counters = p->d_counters;
    a.sm_slots = reinterpret_cast<int*>(p->d_counters + 8);
    a.epsilon = o->epsilon; a.min_dt = o->min_dt; a.dt0 = o->dt0; a.max_steps = o->max_steps;
    a.dt_floor = o->dt_floor;
    if (P.grouped) { a.grp_start = p->d_grp; a.grp_size = p->d_grp + ng; a.n_groups = ng; }
    if (P.coop && P.learned && o->warm_start) a.mlp = ag_mlp_device_view();
    a.warm_no_time_fallback = o->warm_start == 3 ? 1 : 0;
    double wd = 300.0;
    if (const char* w = getenv("ASSIST_GB300_WATCHDOG_S")) wd = atof(w);
    a.watchdog_cycles = wd > 0 ? (long long)(wd * 2.1e9) : 0;
    /* capture the device work on a private stream */
    cudaStream_t cs = nullptr;
    if (ag_cuda_check(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "plan capture stream")) {
        assist_gb300_plan_free(p);
        return ASSIST_ERROR_EPHEM_FILE;
    }
    int le = 0;
    ok = !ag_cuda_check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed), "plan capture");
    if (ok) {
        cudaMemsetAsync(p->d_queue, 0, sizeof(int), cs);
        cudaMemsetAsync(p->d_counters, 0, 8 * sizeof(unsigned long long) + AG_SM_SLOTS * sizeof(int), cs);
        le = P.coop ? ag_launch_coop(P.D, P.c, a, n_var, P.occ, P.stage, cs)
                    : (P.grouped ? ag_launch_group(P.D, P.c, a, n_var, cs) : ag_launch_batch(P.D, P.c, a, n_var, P.tpb, cs));
        cudaMemcpyAsync(p->h_counters, p->d_counters, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, cs);
        const cudaError_t ce = cudaStreamEndCapture(cs, &p->graph);
        ok = !le && !ag_cuda_check(ce, "plan capture") &&
             !ag_cuda_check(cudaGraphInstantiate(&p->exec, p->graph, 0), "plan graph instantiate");
    }
    cudaStreamDestroy(cs);
    if (!ok) {
        if (le) ag_cuda_check((cudaError_t)le, "plan kernel capture");
        assist_gb300_plan_free(p);
        return ASSIST_ERROR_EPHEM_FILE;
    }
    *out = p;
    return ASSIST_SUCCESS;
}

extern "C" int assist_gb300_plan_launch(struct assist_gb300_plan* p, void* stream) {
    if (!p || !p->exec) { ag_set_error("plan: no plan"); return ASSIST_ERROR_N; }
    AgRange range("assist_gb300: plan graph launch");
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != p->device) { ag_set_error("plan: launched on another device than it was made on"); return ASSIST_ERROR_N; }
    if (ag_cuda_check(cudaGraphLaunch(p->exec, (cudaStream_t)stream), "plan graph launch")) return ASSIST_ERROR_EPHEM_FILE;
    p->last = (cudaStream_t)stream;
    p->launches++;
    return ASSIST_SUCCESS;
}

extern "C" int assist_gb300_plan_stats(struct assist_gb300_plan* p, struct assist_gb300_batch_stats* stats) {
    if (!p || !stats) { ag_set_error("plan: plan and stats are required"); return ASSIST_ERROR_N; }
    std::memset(stats, 0, sizeof(*stats));
    if (!p->launches) return ASSIST_SUCCESS;
    if (ag_cuda_check(cudaStreamSynchronize(p->last), "plan launch")) return ASSIST_ERROR_EPHEM_FILE;
    const unsigned long long* cnt = p->h_counters;
    stats->steps_accepted = (long long)cnt[0];
    stats->steps_rejected = (long long)cnt[1];
    stats->force_evals = (long long)cnt[2];
    stats->pc_iterations = (long long)cnt[3];
    stats->warm_start_used = (long long)cnt[4];
    stats->warm_start_fallback = (long long)cnt[5];
    stats->tables_built = (long long)cnt[6];
    stats->kernel_ms = -1.0;    /* not timed: time a launch with events on its stream */
    return ASSIST_SUCCESS;
}

extern "C" int assist_gb300_integrate_batch(const struct assist_ephem* e, const struct assist_gb300_options* o, int n,
                                            const double* t0, const double* t_end, double* state, const double* params,
                                            int n_var, double* var_state, int* status,
                                            struct assist_gb300_batch_stats* stats) {
    if (n <= 0) { if (stats) std::memset(stats, 0, sizeof(*stats)); return ASSIST_SUCCESS; }
    double *d_t0 = nullptr, *d_te = nullptr, *d_st = nullptr, *d_p = nullptr, *d_v = nullptr;
    int* d_s = nullptr;
    const size_t nv = (size_t)n * (size_t)n_var * 6;
    bool ok = !ag_cuda_check(cudaMalloc(&d_t0, sizeof(double) * n), "cudaMalloc") &&
              !ag_cuda_check(cudaMalloc(&d_te, sizeof(double) * n), "cudaMalloc") &&
              !ag_cuda_check(cudaMalloc(&d_st, sizeof(double) * 6 * (size_t)n), "cudaMalloc") &&
              !ag_cuda_check(cudaMalloc(&d_s, sizeof(int) * (size_t)n), "cudaMalloc") &&
              (!params || !ag_cuda_check(cudaMalloc(&d_p, sizeof(double) * 3 * (size_t)n), "cudaMalloc")) &&
              (!nv || !ag_cuda_check(cudaMalloc(&d_v, sizeof(double) * nv), "cudaMalloc"));
    int rc = ASSIST_ERROR_EPHEM_FILE;
    if (ok) {
        cudaMemcpy(d_t0, t0, sizeof(double) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(d_te, t_end, sizeof(double) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(d_st, state, sizeof(double) * 6 * (size_t)n, cudaMemcpyHostToDevice);
        if (params) cudaMemcpy(d_p, params, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice);
        if (nv) cudaMemcpy(d_v, var_state, sizeof(double) * nv, cudaMemcpyHostToDevice);
        struct assist_gb300_batch_stats st;
        rc = assist_gb300_integrate_batch_device(e, o, n, d_t0, d_te, d_st, d_p, n_var, d_v, d_s, nullptr, &st);
        if (rc == ASSIST_SUCCESS) {
            if (ag_cuda_check(cudaMemcpy(state, d_st, sizeof(double) * 6 * (size_t)n, cudaMemcpyDeviceToHost), "copy back"))
                rc = ASSIST_ERROR_EPHEM_FILE;
            if (nv) cudaMemcpy(var_state, d_v, sizeof(double) * nv, cudaMemcpyDeviceToHost);
            if (status) cudaMemcpy(status, d_s, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost);
            if (stats) *stats = st;
        }
    }
    cudaFree(d_t0); cudaFree(d_te); cudaFree(d_st); cudaFree(d_s);
    if (d_p) cudaFree(d_p);
    if (d_v) cudaFree(d_v);
    return rc;
}

/* FP64 FMA throughput of the current device in GFLOP/s (roofline denominator). */
extern "C" double assist_gb300_fp64_peak_gflops(void) { return ag_fp64_probe_gflops(); }

extern "C" int assist_gb300_encounter_ratio_device(const struct assist_ephem* e, int n, const double* d_t0,
                                                   const double* d_t_end, const double* d_state, float* d_ratio,
                                                   void* stream) {
    if (n < 0 || (n > 0 && (!d_t0 || !d_t_end || !d_state || !d_ratio))) {
        ag_set_error("encounter ratio: n must be >= 0 and every array given");
        return ASSIST_ERROR_N;
    }
    if (n == 0) return ASSIST_SUCCESS;
    DevEphem D;
    int st = ag_ephem_device(e, &D);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<double> t0((size_t)n), te((size_t)n);
    if (ag_cuda_check(cudaMemcpyAsync(t0.data(), d_t0, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "read t0") ||
        ag_cuda_check(cudaMemcpyAsync(te.data(), d_t_end, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "read t_end") ||
        ag_cuda_check(cudaStreamSynchronize(s), "read times"))
        return ASSIST_ERROR_EPHEM_FILE;
    double tmin = t0[0], tmax = t0[0];
    for (int i = 0; i < n; i++) {
        tmin = std::min(tmin, std::min(t0[(size_t)i], te[(size_t)i]));
        tmax = std::max(tmax, std::max(t0[(size_t)i], te[(size_t)i]));
    }
    std::lock_guard<std::mutex> lk(g_batch_mu);
    if (!g_batch.d_grid &&
        (ag_cuda_check(cudaMalloc(&g_batch.d_grid, sizeof(float4) * AG_PILOT_G * 10), "cudaMalloc(pilot grid)") ||
         ag_cuda_check(cudaMalloc(&g_batch.d_sunv, sizeof(float2) * AG_PILOT_G), "cudaMalloc(pilot grid)")))
        return ASSIST_ERROR_EPHEM_FILE;
    if (ag_cuda_check((cudaError_t)ag_pilot_encounters(D, n, d_t0, d_t_end, d_state, tmin, tmax, d_ratio,
                                                       g_batch.d_grid, g_batch.d_sunv, AG_PILOT_G, s),
                      "pilot kernels") ||
        ag_cuda_check(cudaStreamSynchronize(s), "pilot kernels"))
        return ASSIST_ERROR_EPHEM_FILE;
    return ASSIST_SUCCESS;
}

extern "C" int assist_gb300_group_plan(int n, const double* t0, const double* t_end, const double* state,
                                       const double* params, const float* ratio, int group_order, double gm_sun,
                                       int* order, int* gstart, int* gsize, int* n_groups) {
    if (n < 0 || (n > 0 && (!t0 || !t_end || !state || !order || !gstart || !gsize || !n_groups)) ||
        (group_order < 0 || group_order > 2) || !(gm_sun > 0.0)) {
        ag_set_error("group plan: n >= 0, every output array, group_order 0, 1 or 2 and gm_sun > 0 are required");
        return ASSIST_ERROR_N;
    }
    if (n_groups) *n_groups = 0;
    if (n == 0) return ASSIST_SUCCESS;
    for (int i = 0; i < n; i++)
        if (!std::isfinite(t0[i]) || !std::isfinite(t_end[i])) {
            ag_set_error("group plan: t0 and t_end must be finite");
            return ASSIST_ERROR_N;
        }
    std::vector<unsigned char> has_ng((size_t)n, 0);
    if (params)
        for (int i = 0; i < n; i++)
            has_ng[(size_t)i] = params[3 * (size_t)i] != 0.0 || params[3 * (size_t)i + 1] != 0.0 || params[3 * (size_t)i + 2] != 0.0;
    std::vector<AgGroupKey> key;
    ag_group_keys(n, t0, t_end, state, has_ng.data(), gm_sun, group_order, key);
    std::vector<int> ord, gs, gz;
    ag_group_form(key, ratio, group_order, ord, gs, gz);
    std::copy(ord.begin(), ord.end(), order);
    std::copy(gs.begin(), gs.end(), gstart);
    std::copy(gz.begin(), gz.end(), gsize);
    *n_groups = (int)gs.size();
    return ASSIST_SUCCESS;
}
