/*
 * device_forces.cuh -- ASSIST's test-particle force model for one particle on
 * sm_103a, with the first-order variational Jacobian.
 *
 * Terms and their accumulation order follow src/forces.c:120-147: Marsden
 * non-gravitational (:774-1057), Earth J2/J3/J4 (:435-642), Sun J2
 * (:644-772), EIH/PPN GR (:1288-1983), GR potential (:1059-1161), GR simple
 * (:1163-1286), then direct gravity body by body, asteroids first, then
 * Pluto, Moon, Mars, Mercury, Neptune, Uranus, Earth, Venus, Saturn, Jupiter,
 * Sun (:281-345); the geocentric indirect term last (:157-172).
 *
 * GB300 has 2 FP64 FMA lanes per SM per clock, so the formulation minimises
 * FP64 instructions: one rsqrt per particle-body distance (shared by every
 * term that needs it, where ASSIST recomputes sqrt and divides per term),
 * fused multiply-adds, and the variational partials built once per particle
 * as a 3x6 Jacobian (plus 3x3 in the non-grav parameters) that every
 * variational particle of that particle multiplies, replacing ASSIST's scan
 * over all variational configurations per term.
 *
 * Body states come from a `Bodies` policy: a per-time table in shared memory
 * (all particles at one time) or per-thread Chebyshev evaluation (every
 * particle at its own time).
 */
#ifndef ASSIST_GB300_DEVICE_FORCES_CUH
#define ASSIST_GB300_DEVICE_FORCES_CUH

#include "device_ephem.cuh"

#define AG_F_SUN 0x01
#define AG_F_PLANETS 0x02
#define AG_F_AST 0x04
#define AG_F_NONGRAV 0x08
#define AG_F_EARTH_H 0x10
#define AG_F_SUN_H 0x20
#define AG_F_EIH 0x40
#define AG_F_GR_SIMPLE 0x80
#define AG_F_GR_POT 0x100

/* Force-model configuration (assist_extras fields, src/assist.h:177-195) plus
 * the pole rotations ASSIST forms from hard-coded RA/Dec (computed on the host
 * with the same expressions, so cos(pi/2) = 6.1e-17 is kept, not 0). */
struct ForceCfg {
    int forces, gr_eih_sources, geocentric;
    int nongrav_rm2;                   /* nm == 2, nk == 0: g = alpha (r/r0)^-2, no pow() */
    double alpha, nk, nm, nn, r0;
    double e_sa, e_ca, e_sd, e_cd;     /* Earth pole: RA 0 deg, Dec 90 deg */
    double s_sa, s_ca, s_sd, s_cd;     /* Sun pole: RA 286.13 deg, Dec 63.87 deg */
};


/* Planet states at one time as a force evaluation needs them. */
struct PlanetState {
    double x[AG_NPL], y[AG_NPL], z[AG_NPL];
    double vx[AG_NPL], vy[AG_NPL], vz[AG_NPL];   /* only EIH sources and the Sun are filled */
    double ex_a[3];                               /* Earth acceleration (geocentric origin) */
};

/* Per-source EIH quantities that do not depend on the particle
 * (src/forces.c:1400-1448): Newtonian acceleration of source j by the other
 * planets and sum of GM_k / r_jk. */
__device__ __forceinline__ void ag_eih_source(const DevEphem& E, const PlanetState& P, int j, double* aj,
                                              double* term1) {
    double ax = 0.0, ay = 0.0, az = 0.0, s1 = 0.0;
#pragma unroll
    for (int k = 0; k < AG_NPL; k++) {
        if (k == j) continue;
        const double dx = P.x[j] - P.x[k], dy = P.y[j] - P.y[k], dz = P.z[j] - P.z[k];
        const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
        const double ri = rsqrt(r2);
        const double gri = E.gm[k] * ri;
        s1 += gri;
        const double f = gri * ri * ri;
        ax = fma(-f, dx, ax); ay = fma(-f, dy, ay); az = fma(-f, dz, az);
    }
    aj[0] = ax; aj[1] = ay; aj[2] = az;
    *term1 = s1;
}

/* Evaluate the eleven planets (positions; velocities of the Sun and the first
 * n_vel bodies; Earth's acceleration when geocentric) at time t with the
 * exact arithmetic of the reference. */
__device__ __forceinline__ int ag_planets_at(const DevEphem& E, double t, int n_vel, bool earth_acc, PlanetState& P) {
    if (E.pl_spk) {
        /* planets SPK: every body's full state (src/spk.c:550-608) */
#pragma unroll 1
        for (int b = 0; b < AG_NPL; b++) {
            double o[10];
            const int st = ag_spk_planet(E, b, t, o);
            if (st != AG_OK) return st;
            P.x[b] = o[1]; P.y[b] = o[2]; P.z[b] = o[3];
            P.vx[b] = o[4]; P.vy[b] = o[5]; P.vz[b] = o[6];
            if (b == AG_EAR && earth_acc) { P.ex_a[0] = o[7]; P.ex_a[1] = o[8]; P.ex_a[2] = o[9]; }
        }
        return AG_OK;
    }
    const double* rec;
    double tf;
    int st = ag_planet_record(E, t, &rec, &tf);
    if (st != AG_OK) return st;
    double u[3], v[3];
#pragma unroll 1
    for (int b = 0; b < AG_NPL; b++) {
        if (b == AG_EAR || b == AG_MOO) continue;
        if (b == AG_SUN || b < n_vel) {
            ag_planet_exact<true>(E, rec, tf, b, u, v);
            P.vx[b] = v[0]; P.vy[b] = v[1]; P.vz[b] = v[2];
        } else {
            ag_planet_exact<false>(E, rec, tf, b, u, v);
        }
        P.x[b] = u[0]; P.y[b] = u[1]; P.z[b] = u[2];
    }
    /* Earth and Moon share the EMB and geocentric-Moon columns */
    const bool vel_em = n_vel > AG_EAR;
    double eu[3], ev[3], lu[3], lv[3];
    if (vel_em) { ag_column_exact<true>(E, rec, AG_C_EMB, tf, eu, ev); ag_column_exact<true>(E, rec, AG_C_LUN, tf, lu, lv); }
    else { ag_column_exact<false>(E, rec, AG_C_EMB, tf, eu, ev); ag_column_exact<false>(E, rec, AG_C_LUN, tf, lu, lv); }
    for (int k = 0; k < 3; k++) {
        const double xe = __ddiv_rn(__dadd_rn(eu[k], __dmul_rn(lu[k], E.f_earth)), E.pl_cau);
        const double xm = __ddiv_rn(__dadd_rn(eu[k], __dmul_rn(lu[k], E.f_moon)), E.pl_cau);
        if (k == 0) { P.x[AG_EAR] = xe; P.x[AG_MOO] = xm; }
        else if (k == 1) { P.y[AG_EAR] = xe; P.y[AG_MOO] = xm; }
        else { P.z[AG_EAR] = xe; P.z[AG_MOO] = xm; }
        if (vel_em) {
            const double ve = __ddiv_rn(__dadd_rn(ev[k], __dmul_rn(lv[k], E.f_earth)), E.cau_per_day);
            const double vm = __ddiv_rn(__dadd_rn(ev[k], __dmul_rn(lv[k], E.f_moon)), E.cau_per_day);
            if (k == 0) { P.vx[AG_EAR] = ve; P.vx[AG_MOO] = vm; }
            else if (k == 1) { P.vy[AG_EAR] = ve; P.vy[AG_MOO] = vm; }
            else { P.vz[AG_EAR] = ve; P.vz[AG_MOO] = vm; }
        }
    }
    if (earth_acc) {
        double e_[10];
        ag_planet_full(E, AG_EAR, t, e_);
        P.ex_a[0] = e_[7]; P.ex_a[1] = e_[8]; P.ex_a[2] = e_[9];
        P.x[AG_EAR] = e_[1]; P.y[AG_EAR] = e_[2]; P.z[AG_EAR] = e_[3];
        P.vx[AG_EAR] = e_[4]; P.vy[AG_EAR] = e_[5]; P.vz[AG_EAR] = e_[6];
    }
    return AG_OK;
}

/* Bodies evaluated by this thread at its own time. */
struct ThreadBodies {
    const DevEphem& E;
    double t;
    PlanetState P;
    __device__ ThreadBodies(const DevEphem& e, double tt) : E(e), t(tt) {}
    __device__ int init(const ForceCfg& c) {
        int nv = (c.forces & AG_F_EIH) ? c.gr_eih_sources : 0;
        if (c.geocentric) nv = nv > AG_EAR + 1 ? nv : AG_EAR + 1;
        return ag_planets_at(E, t, nv, c.geocentric == 1, P);
    }
    __device__ const PlanetState& planets() const { return P; }
    __device__ void eih(int j, double* aj, double* t1) const { ag_eih_source(E, P, j, aj, t1); }
    __device__ int asteroid(int m, double* p) const {
        double h[3];
        int st = ag_asteroid_pos(E, m, t, h);
        p[0] = h[0] + P.x[AG_SUN]; p[1] = h[1] + P.y[AG_SUN]; p[2] = h[2] + P.z[AG_SUN];
        return st;
    }
};

/* Bodies from a table evaluated once for the time shared by every particle
 * (layout of AgTable below, typically staged in shared memory). */
struct AgTable {
    PlanetState P;
    double ast[AG_MAX_AST][3];       /* barycentric asteroid positions */
    double eih_a[AG_NPL][3];         /* per-source Newtonian acceleration */
    double eih_t1[AG_NPL];           /* per-source sum GM_k / r_jk */
    int status;
};
struct TableBodies {
    const AgTable& T;
    __device__ TableBodies(const AgTable& t) : T(t) {}
    __device__ int init(const ForceCfg&) { return T.status; }
    __device__ const PlanetState& planets() const { return T.P; }
    __device__ void eih(int j, double* aj, double* t1) const {
        aj[0] = T.eih_a[j][0]; aj[1] = T.eih_a[j][1]; aj[2] = T.eih_a[j][2]; *t1 = T.eih_t1[j];
    }
    __device__ int asteroid(int m, double* p) const { p[0] = T.ast[m][0]; p[1] = T.ast[m][1]; p[2] = T.ast[m][2]; return AG_OK; }
};

/* Fill a table for time t (called by one thread per body slot; thread 0 also
 * does the per-source EIH sums after a __syncthreads by the caller). */
__device__ inline int ag_table_planets(const DevEphem& E, const ForceCfg& c, double t, AgTable& T) {
    int nv = (c.forces & AG_F_EIH) ? c.gr_eih_sources : 0;
    if (c.geocentric) nv = nv > AG_EAR + 1 ? nv : AG_EAR + 1;
    return ag_planets_at(E, t, nv, c.geocentric == 1, T.P);
}

/* Harmonic partials helper: rotate v into the pole frame (x' = -x sa + y ca, ...). */
__device__ __forceinline__ void ag_rot_in(double sa, double ca, double sd, double cd, double x, double y, double z,
                                          double* o) {
    o[0] = -x * sa + y * ca;
    o[1] = -x * ca * sd - y * sa * sd + z * cd;
    o[2] = x * ca * cd + y * sa * cd + z * sd;
}
__device__ __forceinline__ void ag_rot_out(double sa, double ca, double sd, double cd, double x, double y, double z,
                                           double* o) {
    o[0] = -x * sa - y * ca * sd + z * ca * cd;
    o[1] = x * ca - y * sa * sd + z * sa * cd;
    o[2] = y * cd + z * sd;
}
/* J (pole frame, symmetric M) -> original frame: R^T M R with R the rotation above. */
__device__ __forceinline__ void ag_rot_sym_add(double sa, double ca, double sd, double cd, const double M[3][3],
                                               double J[3][6]) {
    double R[3][3] = {{-sa, ca, 0.0}, {-ca * sd, -sa * sd, cd}, {ca * cd, sa * cd, sd}};
    double MR[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) MR[a][b] = M[a][0] * R[0][b] + M[a][1] * R[1][b] + M[a][2] * R[2][b];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) J[a][b] += R[0][a] * MR[0][b] + R[1][a] * MR[1][b] + R[2][a] * MR[2][b];
}

/* ------------------------------------------------------------------ terms
 * Each term adds to (ax, ay, az) and, with JAC, to the 3x6 Jacobian J.
 * ag_forces calls them in ASSIST's order; the block-cooperative IAS15 kernel
 * calls subsets of them from different warps. */

/* Separation of the particle from planet k and its inverse length. */
__device__ __forceinline__ void ag_sep(const PlanetState& P, const double* x, const double* xo, int k, double& dx,
                                       double& dy, double& dz, double& ri) {
    dx = x[0] + (xo[0] - P.x[k]);
    dy = x[1] + (xo[1] - P.y[k]);
    dz = x[2] + (xo[2] - P.z[k]);
    ri = rsqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
}

/* Marsden non-gravitational acceleration (radial, transverse, normal);
 * d, rinv: heliocentric separation; dv: heliocentric velocity. */
template <bool JAC>
__device__ __forceinline__ void ag_term_nongrav(const ForceCfg& c, const double* d, double rinv, const double* dv,
                                                const double* A, double& ax, double& ay, double& az, double (*J)[6],
                                                double (*JA)[3], bool* has_ng) {
    const double r = 1.0 / rinv;
    double g, dgdr;
    if (c.nongrav_rm2) {
        /* g = alpha (r0 / r)^2: no division (the reference's pow(r/r0, -2)
         * and this product agree to a few units in the last place) */
        const double q = c.r0 * rinv;
        g = c.alpha * q * q;
        dgdr = -2.0 * g * rinv;
    } else {
        const double rr0 = r / c.r0;
        const double pn = pow(rr0, c.nn);
        g = c.alpha * pow(rr0, -c.nm) * pow(1.0 + pn, -c.nk);
        dgdr = (c.alpha / c.r0) * (-c.nm * pow(rr0, -c.nm - 1) * pow(1.0 + pn, -c.nk)
                + pow(rr0, -c.nm) * (-c.nk * c.nn) * pow(rr0, c.nn - 1) * pow(1.0 + pn, -c.nk - 1));
    }
    const double h[3] = {d[1] * dv[2] - d[2] * dv[1], d[2] * dv[0] - d[0] * dv[2], d[0] * dv[1] - d[1] * dv[0]};
    const double hinv = rsqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
    const double tv[3] = {h[1] * d[2] - h[2] * d[1], h[2] * d[0] - h[0] * d[2], h[0] * d[1] - h[1] * d[0]};
    const double tinv = rsqrt(tv[0] * tv[0] + tv[1] * tv[1] + tv[2] * tv[2]);
    const double ga1 = A[0] * g * rinv, ga2 = A[1] * g * tinv, ga3 = A[2] * g * hinv;
    ax += ga1 * d[0] + ga2 * tv[0] + ga3 * h[0];
    ay += ga1 * d[1] + ga2 * tv[1] + ga3 * h[1];
    az += ga1 * d[2] + ga2 * tv[2] + ga3 * h[2];
    if (JAC) {
        *has_ng = true;
        const double r2 = r * r;
        const double r3inv = rinv * rinv * rinv;
        const double v2 = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
        const double rdv = d[0] * dv[0] + d[1] * dv[1] + d[2] * dv[2];
        const double vdt = dv[0] * tv[0] + dv[1] * tv[1] + dv[2] * tv[2];
        const double dg[3] = {dgdr * d[0] * rinv, dgdr * d[1] * rinv, dgdr * d[2] * rinv};
        const double h3 = hinv * hinv * hinv, t3 = tinv * tinv * tinv;
        for (int a = 0; a < 3; a++) {
            JA[a][0] = g * d[a] * rinv; JA[a][1] = g * tv[a] * tinv; JA[a][2] = g * h[a] * hinv;
        }
        for (int a = 0; a < 3; a++) {
            for (int b = 0; b < 3; b++) {
                const int cc = 3 - a - b;       /* the third axis when a != b */
                const double eps = (b == (a + 1) % 3) ? 1.0 : -1.0;
                double jx, jv;
                if (a == b) {
                    jx = A[0] * (dg[a] * d[a] * rinv + g * (rinv - d[a] * d[a] * r3inv))
                       + A[1] * (dg[a] * tv[a] * tinv + g * ((d[a] * dv[a] - rdv) * tinv - tv[a] * t3 * (2.0 * d[a] * vdt - rdv * tv[a])))
                       + A[2] * (dg[a] * h[a] * hinv - g * h[a] * h3 * (v2 * d[a] - rdv * dv[a]));
                    const double ss = r2 - d[a] * d[a];
                    jv = A[1] * g * (ss * tinv - tv[a] * t3 * r2 * tv[a])
                       + A[2] * g * (-h[a] * h3 * (r2 * dv[a] - d[a] * rdv));
                } else {
                    jx = A[0] * (dg[b] * d[a] * rinv - g * d[a] * d[b] * r3inv)
                       + A[1] * (dg[b] * tv[a] * tinv + g * ((2.0 * d[b] * dv[a] - d[a] * dv[b]) * tinv - tv[a] * t3 * (2.0 * d[b] * vdt - rdv * tv[b])))
                       + A[2] * (dg[b] * h[a] * hinv + g * (eps * dv[cc] * hinv - h[a] * h3 * (v2 * d[b] - rdv * dv[b])));
                    jv = A[1] * g * (-d[b] * d[a] * tinv - tv[b] * t3 * r2 * tv[a])
                       + A[2] * g * (-eps * d[cc] * hinv - h[a] * h3 * (r2 * dv[b] - d[b] * rdv));
                }
                J[a][b] += jx;
                J[a][3 + b] += jv;
            }
        }
    }
}

/* Earth J2, J3, J4 in the equatorial frame of the J2000 pole; (dx, dy, dz),
 * rinv: geocentric separation. */
template <bool JAC>
__device__ __forceinline__ void ag_term_earth_h(const DevEphem& E, const ForceCfg& c, double dx, double dy, double dz,
                                                double rinv, double& ax, double& ay, double& az, double (*J)[6]) {
    const double GMe = E.gm[AG_EAR];
    const double r2i = rinv * rinv;
    double p[3];
    ag_rot_in(c.e_sa, c.e_ca, c.e_sd, c.e_cd, dx, dy, dz, p);
    const double Re2 = E.Re_eq * E.Re_eq;
    const double c2 = p[2] * p[2] * r2i;
    const double r5i = r2i * r2i * rinv;
    const double p2 = 1.5 * E.J2E * Re2 * r5i;
    const double f2 = 5.0 * c2 - 1.0;
    const double p3 = 2.5 * E.J3E * Re2 * E.Re_eq * r5i;
    const double f3 = 3.0 - 7.0 * c2;
    const double p4 = 0.625 * E.J4E * Re2 * Re2 * r5i * r2i;
    const double f4 = (63.0 * c2 - 42.0) * c2 + 3.0;
    double res[3];
    const double k2 = GMe * p2, k3 = GMe * p3, k4 = GMe * p4;
    res[0] = k2 * f2 * p[0] - k3 * r2i * f3 * p[0] * p[2] + k4 * f4 * p[0];
    res[1] = k2 * f2 * p[1] - k3 * r2i * f3 * p[1] * p[2] + k4 * f4 * p[1];
    res[2] = k2 * (f2 - 2.0) * p[2] - k3 * ((6.0 - 7.0 * c2) * c2 - 0.6) + k4 * (f4 + 12.0 - 28.0 * c2) * p[2];
    double o[3];
    ag_rot_out(c.e_sa, c.e_ca, c.e_sd, c.e_cd, res[0], res[1], res[2], o);
    ax += o[0]; ay += o[1]; az += o[2];
    if (JAC) {
        const double g2 = 7.0 * c2 - 1.0, g3 = (35.0 * c2 - 30.0) * c2 + 3.0;
        const double ct = p[2] * rinv;
        const double h2 = 21.0 * (1.0 - 3.0 * c2) * r2i;
        const double h3 = 3.0 * ((-21.0 * c2 + 14.0) * c2 - 1.0) * r2i;
        const double h4 = ((-63.0 * c2 + 70.0) * c2 - 15.0) * ct * rinv;
        const double q2 = (33.0 * c2 - 18.0) * c2 + 1.0, q3 = (33.0 * c2 - 30.0) * c2 + 5.0;
        const double q4 = ((231.0 * c2 - 315.0) * c2 + 105.0) * c2 - 5.0;
        double M[3][3];
        for (int a = 0; a < 2; a++) {
            M[a][a] = k2 * (f2 - 5.0 * g2 * p[a] * p[a] * r2i) + k3 * ct * (h2 * p[a] * p[a] - f3) * rinv
                      + k4 * (f4 - 21.0 * q2 * p[a] * p[a] * r2i);
            M[a][2] = M[2][a] = -5.0 * k2 * (g2 - 2.0) * p[a] * p[2] * r2i + k3 * h3 * p[a]
                                - 21.0 * k4 * q3 * p[a] * p[2] * r2i;
        }
        M[0][1] = M[1][0] = -5.0 * k2 * g2 * p[0] * p[1] * r2i + k3 * h2 * ct * p[0] * p[1] * rinv
                            - 21.0 * k4 * q2 * p[0] * p[1] * r2i;
        M[2][2] = -k2 * g3 + k3 * h4 - 3.0 * k4 * q4;
        ag_rot_sym_add(c.e_sa, c.e_ca, c.e_sd, c.e_cd, M, J);
    }
}

/* Sun J2 about the solar pole; (dx, dy, dz), rinv: heliocentric separation. */
template <bool JAC>
__device__ __forceinline__ void ag_term_sun_h(const DevEphem& E, const ForceCfg& c, double dx, double dy, double dz,
                                              double rinv, double& ax, double& ay, double& az, double (*J)[6]) {
    const double GMs = E.gm[AG_SUN];
    const double r2i = rinv * rinv;
    double p[3];
    ag_rot_in(c.s_sa, c.s_ca, c.s_sd, c.s_cd, dx, dy, dz, p);
    const double c2 = p[2] * p[2] * r2i;
    const double k2 = GMs * 1.5 * E.J2SUN * E.Rs_eq * E.Rs_eq * r2i * r2i * rinv;
    const double f2 = 5.0 * c2 - 1.0;
    double o[3];
    ag_rot_out(c.s_sa, c.s_ca, c.s_sd, c.s_cd, k2 * f2 * p[0], k2 * f2 * p[1], k2 * (f2 - 2.0) * p[2], o);
    ax += o[0]; ay += o[1]; az += o[2];
    if (JAC) {
        const double g2 = 7.0 * c2 - 1.0, g3 = (35.0 * c2 - 30.0) * c2 + 3.0;
        double M[3][3];
        M[0][0] = k2 * (f2 - 5.0 * g2 * p[0] * p[0] * r2i);
        M[1][1] = k2 * (f2 - 5.0 * g2 * p[1] * p[1] * r2i);
        M[2][2] = -k2 * g3;
        M[0][1] = M[1][0] = -5.0 * k2 * g2 * p[0] * p[1] * r2i;
        M[1][2] = M[2][1] = -5.0 * k2 * (g2 - 2.0) * p[1] * p[2] * r2i;
        M[0][2] = M[2][0] = -5.0 * k2 * (g2 - 2.0) * p[0] * p[2] * r2i;
        ag_rot_sym_add(c.s_sa, c.s_ca, c.s_sd, c.s_cd, M, J);
    }
}

/* EIH sums over all eleven planets that do not depend on the source:
 * sum_k GM_k / r_ik and (variational) sum_k GM_k d_ik / r_ik^3. */
template <bool JAC>
__device__ __forceinline__ void ag_eih_planet_sums(const DevEphem& E, const double* dx, const double* dy,
                                                   const double* dz, const double* ri, double& term0, double* g0) {
    term0 = 0.0;
    g0[0] = g0[1] = g0[2] = 0.0;
#pragma unroll
    for (int k = 0; k < AG_NPL; k++) {
        const double gri = E.gm[k] * ri[k];
        term0 += gri;
        if (JAC) {
            const double f = gri * ri[k] * ri[k];
            g0[0] = fma(f, dx[k], g0[0]); g0[1] = fma(f, dy[k], g0[1]); g0[2] = fma(f, dz[k], g0[2]);
        }
    }
}

/* Einstein-Infeld-Hoffmann (PPN, beta = gamma = 1) over the first
 * gr_eih_sources planets, given the planet sums above; sep(j, dj, rj) gives
 * the separation from source j and its inverse length. */
template <class Bodies, bool JAC, class Sep>
__device__ __forceinline__ void ag_term_eih_core(const Bodies& B, const DevEphem& E, const ForceCfg& c,
                                                 const PlanetState& P, double term0, const double* g0, Sep sep,
                                                 const double* v, const double* vo, const double* ao, double& ax,
                                                 double& ay, double& az, double (*J)[6]) {
    const double oc2 = E.over_c_squared;
    term0 *= -4.0 * oc2;
    const double vi2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double t7[3] = {0.0, 0.0, 0.0}, t8[3] = {0.0, 0.0, 0.0};
    const int nsrc = c.gr_eih_sources;
#pragma unroll 1
    for (int j = 0; j < nsrc; j++) {
        double dj[3], rj;
        sep(j, dj, rj);
        const double vjb[3] = {P.vx[j], P.vy[j], P.vz[j]};
        const double GMj = E.gm[j];
        const double pre = GMj * rj * rj * rj;
        const double vj[3] = {vjb[0] - vo[0], vjb[1] - vo[1], vjb[2] - vo[2]};
        double aj[3], t1;
        B.eih(j, aj, &t1);
        const double term1 = -oc2 * t1;
        const double term2 = oc2 * vi2;
        const double vj2 = vj[0] * vj[0] + vj[1] * vj[1] + vj[2] * vj[2];
        const double term3 = 2.0 * oc2 * vj2;
        const double vivj = v[0] * vj[0] + v[1] * vj[1] + v[2] * vj[2];
        const double term4 = -4.0 * oc2 * vivj;
        const double rdvj = dj[0] * vj[0] + dj[1] * vj[1] + dj[2] * vj[2];
        const double term5 = -1.5 * oc2 * (rdvj * rdvj) * (rj * rj);
        const double fv[3] = {4.0 * v[0] - 3.0 * vj[0], 4.0 * v[1] - 3.0 * vj[1], 4.0 * v[2] - 3.0 * vj[2]};
        const double f = dj[0] * fv[0] + dj[1] * fv[1] + dj[2] * fv[2];
        const double pf = pre * f;
        const double rel[3] = {v[0] - vj[0], v[1] - vj[1], v[2] - vj[2]};
        t7[0] = fma(pf, rel[0], t7[0]); t7[1] = fma(pf, rel[1], t7[1]); t7[2] = fma(pf, rel[2], t7[2]);
        const double rdaj = dj[0] * (aj[0] - ao[0]) + dj[1] * (aj[1] - ao[1]) + dj[2] * (aj[2] - ao[2]);
        const double term6 = -0.5 * oc2 * rdaj;
        const double t8f = GMj * rj * 3.5;
        t8[0] = fma(t8f, aj[0], t8[0]); t8[1] = fma(t8f, aj[1], t8[1]); t8[2] = fma(t8f, aj[2], t8[2]);
        const double factor = term0 + term1 + term2 + term3 + term4 + term5 + term6;
        ax += -pre * dj[0] * factor;
        ay += -pre * dj[1] * factor;
        az += -pre * dj[2] * factor;
        if (JAC) {
            const double r2i = rj * rj;
            const double dpre_s = -3.0 * pre * r2i;                 /* dpre_b = dpre_s * d_b */
            const double t5f = 3.0 * oc2 * rdvj * rj;
            double dfac[6];
            for (int a = 0; a < 3; a++) {
                const double dt0 = 4.0 * oc2 * g0[a];               /* -2(b+g)oc2 * (-sum GM d/r^3) */
                const double dt5 = -t5f * (vj[a] * rj - rdvj * dj[a] * rj * r2i);
                const double dt6 = -0.5 * oc2 * (aj[a] - ao[a]);
                dfac[a] = dt0 + dt5 + dt6;
                dfac[3 + a] = 2.0 * oc2 * v[a] - 4.0 * oc2 * vj[a];
            }
            const double t8d = -GMj * rj * r2i * 3.5;
            /* d acc_a / dx_b = -d_a (dpre_b factor + pre dfac_b) - pre factor delta_ab
             *                 + oc2 rel_a (dpre_b f + pre fv_b) + oc2 t8d aj_a d_b   (term 7 and term 8)
             * d acc_a / dv_b = -pre d_a dfac_(3+b) + oc2 (4 pre d_b rel_a + pf delta_ab)
             * as sums of outer products: the row factors d, rel, aj times the
             * column vectors u, w, y (position) and p, q (velocity). */
            const double sdu = -dpre_s * factor, swd = oc2 * dpre_s * f, swf = oc2 * pre, sy = oc2 * t8d,
                         sq = 4.0 * oc2 * pre;
            double u[3], w[3], y[3], p[3], q[3];
            for (int b = 0; b < 3; b++) {
                u[b] = fma(sdu, dj[b], -pre * dfac[b]);
                w[b] = fma(swd, dj[b], swf * fv[b]);
                y[b] = sy * dj[b];
                p[b] = -pre * dfac[3 + b];
                q[b] = sq * dj[b];
            }
            const double diag_x = pre * factor, diag_v = oc2 * pf;
            for (int a = 0; a < 3; a++) {
                for (int b = 0; b < 3; b++) {
                    double s = fma(dj[a], u[b], fma(rel[a], w[b], fma(aj[a], y[b], J[a][b])));
                    if (a == b) s -= diag_x;
                    J[a][b] = s;
                    double sv = fma(dj[a], p[b], fma(rel[a], q[b], J[a][3 + b]));
                    if (a == b) sv += diag_v;
                    J[a][3 + b] = sv;
                }
            }
        }
    }
    ax += t7[0] * oc2 + t8[0] * oc2;
    ay += t7[1] * oc2 + t8[1] * oc2;
    az += t7[2] * oc2 + t8[2] * oc2;
}

/* EIH with the separations from all eleven planets in arrays. */
template <class Bodies, bool JAC>
__device__ __forceinline__ void ag_term_eih(const Bodies& B, const DevEphem& E, const ForceCfg& c,
                                            const PlanetState& P, const double* dx, const double* dy, const double* dz,
                                            const double* ri, const double* v, const double* vo, const double* ao,
                                            double& ax, double& ay, double& az, double (*J)[6]) {
    double term0, g0[3];
    ag_eih_planet_sums<JAC>(E, dx, dy, dz, ri, term0, g0);
    auto sep = [&](int j, double* dj, double& rj) {
        /* select source j's data with static indices (keeps arrays in registers) */
        dj[0] = dj[1] = dj[2] = 0.0;
        rj = 0.0;
#pragma unroll
        for (int k = 0; k < AG_NPL; k++)
            if (k == j) { dj[0] = dx[k]; dj[1] = dy[k]; dj[2] = dz[k]; rj = ri[k]; }
    };
    ag_term_eih_core<Bodies, JAC>(B, E, c, P, term0, g0, sep, v, vo, ao, ax, ay, az, J);
}

/* GR potential (Nobili & Roxburgh); p, rinv: heliocentric separation. */
template <bool JAC>
__device__ __forceinline__ void ag_term_gr_pot(const DevEphem& E, const double* p, double rinv, double& ax, double& ay,
                                               double& az, double (*J)[6]) {
    const double GMs = E.gm[AG_SUN];
    const double r2i = rinv * rinv;
    const double pre = -6.0 * GMs * GMs * E.over_c_squared * r2i * r2i;
    ax += pre * p[0]; ay += pre * p[1]; az += pre * p[2];
    if (JAC)
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) J[a][b] += (a == b ? pre : 0.0) - 4.0 * pre * p[a] * p[b] * r2i;
}

/* GR simple (Damour & Deruelle); p, rinv, pv: heliocentric separation and velocity. */
template <bool JAC>
__device__ __forceinline__ void ag_term_gr_simple(const DevEphem& E, const double* p, double rinv, const double* pv,
                                                  double& ax, double& ay, double& az, double (*J)[6]) {
    const double GMs = E.gm[AG_SUN];
    const double v2 = pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2];
    const double Aq = 4.0 * GMs * rinv - v2;
    const double Bq = 4.0 * (p[0] * pv[0] + p[1] * pv[1] + p[2] * pv[2]);
    const double pre = GMs * rinv * rinv * rinv * E.over_c_squared;
    ax += pre * (Aq * p[0] + Bq * pv[0]);
    ay += pre * (Aq * p[1] + Bq * pv[1]);
    az += pre * (Aq * p[2] + Bq * pv[2]);
    if (JAC) {
        const double dpdr = -3.0 * pre * rinv;
        for (int a = 0; a < 3; a++) {
            const double base_a = Aq * p[a] + Bq * pv[a];
            for (int b = 0; b < 3; b++) {
                double bx = -p[a] * p[b] * rinv * 4.0 * GMs * rinv * rinv + 4.0 * pv[b] * pv[a];
                if (a == b) bx += Aq;
                J[a][b] += dpdr * p[b] * rinv * base_a + pre * bx;
                double bv = -2.0 * pv[b] * p[a] + 4.0 * p[b] * pv[a];
                if (a == b) bv += Bq;
                J[a][3 + b] += pre * bv;
            }
        }
    }
}

/* The direct terms' Jacobian (src/forces.c: 3 GM d d^T / r^5 - GM I / r^3 per
 * body) accumulated apart from the other terms': its symmetric part s (xx,
 * xy, xz, yy, yz, zz) and the sum g of GM / r^3, so that a body costs six
 * fused multiply-adds and one addition instead of nine and three;
 * ag_symjac_add then puts s - g I into the Jacobian once. */
struct AgSymJac {
    double s[6];
    double g;
};
__device__ __forceinline__ void ag_symjac_term(AgSymJac& Y, double gr3, double rk, double d0, double d1, double d2) {
    const double g5 = 3.0 * gr3 * rk * rk;
    const double e0 = g5 * d0, e1 = g5 * d1, e2 = g5 * d2;
    Y.s[0] = fma(e0, d0, Y.s[0]); Y.s[1] = fma(e0, d1, Y.s[1]); Y.s[2] = fma(e0, d2, Y.s[2]);
    Y.s[3] = fma(e1, d1, Y.s[3]); Y.s[4] = fma(e1, d2, Y.s[4]); Y.s[5] = fma(e2, d2, Y.s[5]);
    Y.g += gr3;
}
__device__ __forceinline__ void ag_symjac_add(const AgSymJac& Y, double (*J)[6]) {
    J[0][0] += Y.s[0] - Y.g; J[0][1] += Y.s[1]; J[0][2] += Y.s[2];
    J[1][0] += Y.s[1]; J[1][1] += Y.s[3] - Y.g; J[1][2] += Y.s[4];
    J[2][0] += Y.s[2]; J[2][1] += Y.s[4]; J[2][2] += Y.s[5] - Y.g;
}

/* Direct gravity of asteroids m0..m1-1 (their positions from the Bodies
 * policy); on_ast false keeps only the Jacobian (ASSIST's variational
 * equations include the asteroids even when their force is off). */
template <class Bodies, bool JAC>
__device__ __forceinline__ int ag_term_asteroids(const Bodies& B, const DevEphem& E, bool on_ast, const double* x,
                                                 const double* xo, int m0, int m1, double& ax, double& ay, double& az,
                                                 AgSymJac* Y) {
#pragma unroll 1
    for (int m = m0; m < m1; m++) {
        double pa[3];
        const int st = B.asteroid(m, pa);
        if (st != AG_OK) return st;
        const double ddx = x[0] + (xo[0] - pa[0]), ddy = x[1] + (xo[1] - pa[1]), ddz = x[2] + (xo[2] - pa[2]);
        const double rinv = rsqrt(fma(ddx, ddx, fma(ddy, ddy, ddz * ddz)));
        const double gr3 = E.ast_gm[m] * rinv * rinv * rinv;
        if (on_ast) { ax = fma(-gr3, ddx, ax); ay = fma(-gr3, ddy, ay); az = fma(-gr3, ddz, az); }
        if (JAC) ag_symjac_term(*Y, gr3, rinv, ddx, ddy, ddz);
    }
    return AG_OK;
}

/* Direct gravity of one planet k; on: its force flag. */
template <bool JAC>
__device__ __forceinline__ void ag_term_planet(const DevEphem& E, bool on, int k, double dk0, double dk1, double dk2,
                                               double rk, double& ax, double& ay, double& az, AgSymJac* Y) {
    const double gr3 = E.gm[k] * rk * rk * rk;
    if (on) { ax = fma(-gr3, dk0, ax); ay = fma(-gr3, dk1, ay); az = fma(-gr3, dk2, az); }
    if (JAC) ag_symjac_term(*Y, gr3, rk, dk0, dk1, dk2);
}

/* direct-sum order of the planets, src/forces.c:281-293 */
__device__ __forceinline__ int ag_planet_order(int q) {
    constexpr int order[AG_NPL] = {AG_PLU, AG_MOO, AG_MAR, AG_MER, AG_NEP, AG_URA, AG_EAR, AG_VEN, AG_SAT, AG_JUP, AG_SUN};
    return order[q];
}

/* Origin of the frame: the Earth for geocentric integrations, else the barycentre. */
__device__ __forceinline__ void ag_origin(const ForceCfg& c, const PlanetState& P, double* xo, double* vo, double* ao) {
    xo[0] = xo[1] = xo[2] = vo[0] = vo[1] = vo[2] = ao[0] = ao[1] = ao[2] = 0.0;
    if (c.geocentric == 1) {
        xo[0] = P.x[AG_EAR]; xo[1] = P.y[AG_EAR]; xo[2] = P.z[AG_EAR];
        vo[0] = P.vx[AG_EAR]; vo[1] = P.vy[AG_EAR]; vo[2] = P.vz[AG_EAR];
        ao[0] = P.ex_a[0]; ao[1] = P.ex_a[1]; ao[2] = P.ex_a[2];
    }
}

/*
 * Acceleration of one real particle at (x, v) and time t.
 *   A     : Marsden A1..A3 (zeros skip the term, as ASSIST does)
 *   acc   : out, AU/day^2
 *   J, JA : out if JAC: d acc / d(x, v) (3x6) and d acc / dA (3x3; valid when
 *           *has_ng is set by the call)
 * Returns AG_OK or an ASSIST status (coverage).
 */
template <class Bodies, bool JAC>
__device__ __forceinline__ int ag_forces(Bodies& B, const DevEphem& E, const ForceCfg& c, const double* x,
                                         const double* v, const double* A, double* acc, double (*J)[6],
                                         double (*JA)[3], bool* has_ng) {
    int st = B.init(c);
    if (st != AG_OK) return st;
    const PlanetState& P = B.planets();
    double xo[3], vo[3], ao[3];
    ag_origin(c, P, xo, vo, ao);
    /* particle-planet separations and inverse distances, shared by all terms */
    double dx[AG_NPL], dy[AG_NPL], dz[AG_NPL], ri[AG_NPL];
#pragma unroll
    for (int k = 0; k < AG_NPL; k++) ag_sep(P, x, xo, k, dx[k], dy[k], dz[k], ri[k]);
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (JAC) {
        for (int a = 0; a < 3; a++) {
            for (int b = 0; b < 6; b++) J[a][b] = 0.0;
            for (int b = 0; b < 3; b++) JA[a][b] = 0.0;
        }
        *has_ng = false;
    }
    if ((c.forces & AG_F_NONGRAV) && A != nullptr && (A[0] != 0.0 || A[1] != 0.0 || A[2] != 0.0)) {
        const double d[3] = {dx[AG_SUN], dy[AG_SUN], dz[AG_SUN]};
        const double dv[3] = {v[0] + (vo[0] - P.vx[AG_SUN]), v[1] + (vo[1] - P.vy[AG_SUN]), v[2] + (vo[2] - P.vz[AG_SUN])};
        ag_term_nongrav<JAC>(c, d, ri[AG_SUN], dv, A, ax, ay, az, J, JA, has_ng);
    }
    if (c.forces & AG_F_EARTH_H)
        ag_term_earth_h<JAC>(E, c, dx[AG_EAR], dy[AG_EAR], dz[AG_EAR], ri[AG_EAR], ax, ay, az, J);
    if (c.forces & AG_F_SUN_H)
        ag_term_sun_h<JAC>(E, c, dx[AG_SUN], dy[AG_SUN], dz[AG_SUN], ri[AG_SUN], ax, ay, az, J);
    if (c.forces & AG_F_EIH)
        ag_term_eih<Bodies, JAC>(B, E, c, P, dx, dy, dz, ri, v, vo, ao, ax, ay, az, J);
    if (c.forces & AG_F_GR_POT) {
        const double p[3] = {dx[AG_SUN], dy[AG_SUN], dz[AG_SUN]};
        ag_term_gr_pot<JAC>(E, p, ri[AG_SUN], ax, ay, az, J);
    }
    if (c.forces & AG_F_GR_SIMPLE) {
        const double p[3] = {dx[AG_SUN], dy[AG_SUN], dz[AG_SUN]};
        const double pv[3] = {v[0] + (vo[0] - P.vx[AG_SUN]), v[1] + (vo[1] - P.vy[AG_SUN]), v[2] + (vo[2] - P.vz[AG_SUN])};
        ag_term_gr_simple<JAC>(E, p, ri[AG_SUN], pv, ax, ay, az, J);
    }
    /* direct Newtonian gravity: asteroids, then planets in ASSIST's order */
    if (c.forces & (AG_F_SUN | AG_F_PLANETS | AG_F_AST)) {
        const bool on_ast = (c.forces & AG_F_AST) != 0;
        AgSymJac Y = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, 0.0};
        if (on_ast || JAC) {
            st = ag_term_asteroids<Bodies, JAC>(B, E, on_ast, x, xo, 0, E.n_ast, ax, ay, az, &Y);
            if (st != AG_OK) return st;
        }
#pragma unroll
        for (int q = 0; q < AG_NPL; q++) {
            const int k = ag_planet_order(q);
            const bool on = (k == AG_SUN) ? (c.forces & AG_F_SUN) : (c.forces & AG_F_PLANETS);
            ag_term_planet<JAC>(E, on, k, dx[k], dy[k], dz[k], ri[k], ax, ay, az, &Y);
        }
        if (JAC) ag_symjac_add(Y, J);
    }
    if (c.geocentric == 1) { ax -= ao[0]; ay -= ao[1]; az -= ao[2]; }
    acc[0] = ax; acc[1] = ay; acc[2] = az;
    return AG_OK;
}

#endif
