/*
 * ref_harness.c -- test infrastructure, not product code.
 *
 * Linked together with the UNMODIFIED ASSIST sources (src/assist.c, forces.c,
 * spk.c, ascii_ephem.c, tools.c) into oracle/_ref/libassist_ref.so by
 * oracle/build_ref.sh.  It supplies the handful of REBOUND functions those
 * sources link against and exposes flat, ctypes-friendly entry points that
 * run the reference's own ephemeris loader (assist_ephem_create,
 * src/assist.c:350), body evaluation (assist_all_ephem, src/forces.c:175) and
 * force callback (assist_additional_forces, src/forces.c:49).  Outputs are
 * used to pin the C restatement under oracle/ and to write golden fixtures.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "assist.h"
#include "forces.h"

/* ---- REBOUND symbols the reference sources link against ------------------ */
void reb_simulation_error(struct reb_simulation* r, const char* msg) {
    if (r) {
        strncpy(r->error_message, msg, sizeof(r->error_message) - 1);
        r->error_message[sizeof(r->error_message) - 1] = '\0';
    }
}
void reb_simulation_warning(struct reb_simulation* r, const char* msg) { (void)r; (void)msg; }
struct reb_simulation* reb_simulation_create(void) {
    struct reb_simulation* r = calloc(1, sizeof(*r));
    r->G = 1.0; r->dt = 0.001; r->status = REB_STATUS_RUNNING; r->exact_finish_time = 1;
    r->ri_ias15.epsilon = 1e-9;
    return r;
}
void reb_simulation_free(struct reb_simulation* r) {
    if (!r) return;
    if (r->extras_cleanup) r->extras_cleanup(r);
    free(r->particles); free(r->var_config); free(r);
}
void reb_simulation_add(struct reb_simulation* r, struct reb_particle p) {
    if (r->N >= r->N_allocated) {
        r->N_allocated = r->N_allocated ? 2 * r->N_allocated : 16;
        r->particles = realloc(r->particles, sizeof(struct reb_particle) * (size_t)r->N_allocated);
    }
    r->particles[r->N++] = p;
}
int reb_simulation_integrate(struct reb_simulation* r, double tmax) {
    (void)tmax; reb_simulation_error(r, "integrate is not available in the reference harness");
    r->status = REB_STATUS_GENERIC_ERROR; return r->status;
}
void reb_simulation_step(struct reb_simulation* r) { (void)r; }
void reb_simulation_update_acceleration(struct reb_simulation* r) { (void)r; }
void reb_simulation_create_from_simulationarchive_with_messages(struct reb_simulation* r,
        struct reb_simulationarchive* sa, long snapshot, enum reb_simulation_binary_error_codes* w) {
    (void)r; (void)sa; (void)snapshot; (void)w;
}
struct reb_particle reb_particle_com_of_pair(struct reb_particle p1, struct reb_particle p2) {
    struct reb_particle p = {0};
    double m = p1.m + p2.m;
    p.x = (p1.x * p1.m + p2.x * p2.m) / m; p.y = (p1.y * p1.m + p2.y * p2.m) / m; p.z = (p1.z * p1.m + p2.z * p2.m) / m;
    p.vx = (p1.vx * p1.m + p2.vx * p2.m) / m; p.vy = (p1.vy * p1.m + p2.vy * p2.m) / m; p.vz = (p1.vz * p1.m + p2.vz * p2.m) / m;
    p.m = m;
    return p;
}

/* ---- ephemeris ------------------------------------------------------------ */
void* refh_ephem_create(const char* planets, const char* asteroids) {
    return assist_ephem_create((char*)planets, (char*)asteroids);
}
void refh_ephem_free(void* e) { if (e) assist_ephem_free((struct assist_ephem*)e); }

/* out: GM, x,y,z, vx,vy,vz, ax,ay,az (assist_all_ephem with no cache). */
int refh_get_body(void* e, int i, double t, double* out) {
    return assist_all_ephem((struct assist_ephem*)e, NULL, i, t, &out[0], &out[1], &out[2], &out[3],
                            &out[4], &out[5], &out[6], &out[7], &out[8], &out[9]);
}
void refh_time_bounds(void* e, double* tb, double* te) { assist_ephem_time_bounds((struct assist_ephem*)e, tb, te); }

/* out[16]: jd_ref AU EMRAT J2E J3E J4E J2SUN RE CLIGHT ASUN Re_eq Rs_eq c c2 1/c2 n_bodies */
void refh_constants(void* ev, double* out) {
    struct assist_ephem* e = (struct assist_ephem*)ev;
    double v[16] = {e->jd_ref, e->AU, e->EMRAT, e->J2E, e->J3E, e->J4E, e->J2SUN, e->RE, e->CLIGHT, e->ASUN,
                    e->Re_eq, e->Rs_eq, e->c_AU_per_day, e->c_squared, e->over_c_squared, 0};
    struct assist_extras tmp;
    (void)tmp;
    memcpy(out, v, sizeof(v));
}

/* ---- force callback --------------------------------------------------------
 * A context owns one REBOUND stand-in simulation with n_real real and n_var
 * first-order variational particles (var v belongs to real particle vtp[v])
 * attached to ASSIST exactly as assist_attach does. */
struct refh_ctx {
    struct reb_simulation* sim;
    struct assist_extras* ax;
    double* params;
    int n_real, n_var;
};

void* refh_ctx_create(void* ephem, int n_real, int n_var, const int* vtp, const double* params,
                      int forces, int gr_eih_sources, int geocentric,
                      double alpha, double nk, double nm, double nn, double r0, int use_cache) {
    struct refh_ctx* c = calloc(1, sizeof(*c));
    c->n_real = n_real; c->n_var = n_var;
    c->sim = reb_simulation_create();
    struct reb_particle p = {0};
    for (int i = 0; i < n_real + n_var; i++) reb_simulation_add(c->sim, p);
    c->sim->N_var = n_var;
    c->sim->N_var_config = n_var;
    c->sim->var_config = calloc((size_t)(n_var > 0 ? n_var : 1), sizeof(struct reb_variational_configuration));
    for (int v = 0; v < n_var; v++) {
        c->sim->var_config[v].sim = c->sim;
        c->sim->var_config[v].order = 1;
        c->sim->var_config[v].index = n_real + v;
        c->sim->var_config[v].testparticle = vtp[v];
    }
    c->ax = assist_attach(c->sim, (struct assist_ephem*)ephem);
    c->ax->forces = forces;
    c->ax->gr_eih_sources = gr_eih_sources;
    c->ax->geocentric = geocentric;
    c->ax->alpha = alpha; c->ax->nk = nk; c->ax->nm = nm; c->ax->nn = nn; c->ax->r0 = r0;
    if (params) {
        size_t np = 3 * (size_t)(n_real + n_var);
        c->params = malloc(np * sizeof(double));
        memcpy(c->params, params, np * sizeof(double));
        c->ax->particle_params = c->params;
    }
    if (!use_cache && c->ax->ephem_cache) {
        free(c->ax->ephem_cache->items); free(c->ax->ephem_cache->t); free(c->ax->ephem_cache);
        c->ax->ephem_cache = NULL;
    }
    return c;
}

void refh_ctx_free(void* cv) {
    struct refh_ctx* c = (struct refh_ctx*)cv;
    if (!c) return;
    assist_free(c->ax);
    c->sim->extras_cleanup = NULL;
    reb_simulation_free(c->sim);
    free(c->params);
    free(c);
}

/* Evaluate accelerations of all n_real+n_var particles at time t.
 * x, v, a: 3*(n_real+n_var) doubles.  dt_sign sets the cache direction.
 * Returns sim->status (0 / REB_STATUS_RUNNING on success). */
int refh_ctx_eval(void* cv, double t, double dt_sign, const double* x, const double* v, double* a) {
    struct refh_ctx* c = (struct refh_ctx*)cv;
    struct reb_simulation* s = c->sim;
    int n = c->n_real + c->n_var;
    for (int i = 0; i < n; i++) {
        s->particles[i].x = x[3 * i]; s->particles[i].y = x[3 * i + 1]; s->particles[i].z = x[3 * i + 2];
        s->particles[i].vx = v[3 * i]; s->particles[i].vy = v[3 * i + 1]; s->particles[i].vz = v[3 * i + 2];
        s->particles[i].ax = 0.0; s->particles[i].ay = 0.0; s->particles[i].az = 0.0;
    }
    s->t = t;
    s->dt_last_done = dt_sign;
    s->status = REB_STATUS_RUNNING;
    assist_additional_forces(s);
    for (int i = 0; i < n; i++) {
        a[3 * i] = s->particles[i].ax; a[3 * i + 1] = s->particles[i].ay; a[3 * i + 2] = s->particles[i].az;
    }
    return s->status == REB_STATUS_RUNNING ? 0 : s->status;
}

/* Force callback signature shared with the oracle's IAS15 restatement. */
int refh_force_cb(void* cv, double t, double dt_sign, const double* x, const double* v, double* a) {
    return refh_ctx_eval(cv, t, dt_sign, x, v, a);
}
