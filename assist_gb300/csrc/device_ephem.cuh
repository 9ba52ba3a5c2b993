/*
 * device_ephem.cuh -- Chebyshev ephemeris evaluation on sm_103a.
 *
 * Planets come from the .440 records (ASSIST src/ascii_ephem.c:27-65,
 * 275-384): one 32-day record holds every body's coefficients; a body's
 * column is split into `niv` sub-intervals of `ncf` coefficients per
 * component.  Asteroids come from SPK type-2 segments (src/spk.c:405-481):
 * records [MID, RADIUS, X(P), Y(P), Z(P)] in km, heliocentric.
 *
 * The file images live in device memory unchanged.  Time arithmetic on
 * Julian dates (~2.45e6, where one ulp is 4.7e-10 day) is done with the same
 * operations in the same order as ASSIST so the selected record and the
 * normalised time agree bit for bit; only the Chebyshev sums (FMA, reciprocal
 * scale factors) differ from the reference at the rounding level.
 */
#ifndef ASSIST_GB300_DEVICE_EPHEM_CUH
#define ASSIST_GB300_DEVICE_EPHEM_CUH

#include <cstdint>

#define AG_NPL 11
#define AG_MAX_AST 32
#define AG_MAX_BODIES (AG_NPL + AG_MAX_AST)
#define AG_MAX_NCF 24
#define AG_MAX_SPK_P 32

enum { AG_OK = 0, AG_ERR_EPHEM_FILE = 1, AG_ERR_AST_FILE = 2, AG_ERR_NAST = 3, AG_ERR_NEPHEM = 4, AG_ERR_COVERAGE = 5 };
enum { AG_SUN = 0, AG_MER, AG_VEN, AG_EAR, AG_MOO, AG_MAR, AG_JUP, AG_SAT, AG_URA, AG_NEP, AG_PLU };
/* .440 column indices */
enum { AG_C_MER = 0, AG_C_VEN, AG_C_EMB, AG_C_MAR, AG_C_JUP, AG_C_SAT, AG_C_URA, AG_C_NEP, AG_C_PLU, AG_C_LUN, AG_C_SUN };

/* One SPK type-2 segment, with the Julian-date conversions ASSIST performs per
 * call (src/spk.c:432-445) done once on the host with the same operations. */
struct AgSpkSeg {
    double init_jd;              /* 2451545 + INIT/86400 */
    double intlen_days;          /* INTLEN/86400 */
    double inv_intlen_days;      /* 86400/INTLEN */
    long long data_off;          /* 0-based index of the first record's MID in the file */
    int nrec, R, P;
    int meta_off;                /* index of the first record in rec_meta */
};

/* Per SPK record: x = MID as a Julian date, y = RADIUS/86400 (days),
 * z = 86400/RADIUS, w unused (32-byte aligned for one vector load). */
struct __align__(32) AgRecMeta {
    double x, y, z, w;
};

/* Everything a kernel needs to evaluate bodies; passed by value. */
struct DevEphem {
    double jd_ref;
    /* planets (.440) */
    const double* pl_data;       /* the whole file as doubles; record k at pl_data + k*pl_rec_len */
    long long pl_ndbl;           /* doubles in the file */
    int pl_nrec;                 /* records in the file (header and constants included) */
    int pl_rec_len;              /* doubles per record */
    double pl_beg, pl_end, pl_inc, pl_cau, pl_cem;
    int col_off[13], col_ncf[13], col_niv[13];   /* 0-based offsets within a record */
    double gm[AG_NPL];
    double inv_cau;              /* 1/AU[km] */
    double cau_per_day;          /* AU[km]/86400 (velocity divisor of the exact path) */
    double f_earth, f_moon;      /* -1/(1+EMRAT), EMRAT/(1+EMRAT) */
    double col_vscale[13];       /* (2*niv/inc/86400) * 86400/AU: d/dtau -> AU/day */
    int pl_inc_pow2;             /* record length is a power of two: divide by multiplying */
    double pl_inv_inc;
    /* asteroids (SPK type 2) */
    int n_ast;
    const double* spk;           /* the whole SPK file as doubles */
    long long spk_ndbl;
    double ast_beg[AG_MAX_AST], ast_end[AG_MAX_AST], ast_res[AG_MAX_AST], ast_gm[AG_MAX_AST];
    float ast_gm_hi[AG_MAX_AST], ast_gm_lo[AG_MAX_AST];   /* ast_gm as a float pair hi + lo */
    int ast_nseg[AG_MAX_AST], ast_seg0[AG_MAX_AST];
    const struct AgSpkSeg* segs; /* per segment, see AgSpkSeg */
    const AgRecMeta* rec_meta;     /* per SPK record: (MID as JD, RADIUS/86400, 86400/RADIUS, 0) */
    /* planets from an SPK file (pl_spk = 1) instead of the .440 record:
     * segments of the eleven bodies' targets (Sun 10, Mercury 1, Venus 2,
     * Earth 399, Moon 301, Mars 4 .. Pluto 9) and, in slot 11, the Earth-Moon
     * barycentre 3 that Earth and Moon are stored about */
    int pl_spk;
    const double* pspk;          /* the whole planets SPK file as doubles */
    const struct AgSpkSeg* psegs;
    const AgRecMeta* pmeta;
    int ps_seg0[AG_NPL + 1], ps_nseg[AG_NPL + 1];
    double ps_beg[AG_NPL + 1], ps_end[AG_NPL + 1], ps_res[AG_NPL + 1];
    double au_km;                /* the file's AU (km) */
    /* constants (ASSIST src/assist.c:296-309) */
    double J2E, J3E, J4E, J2SUN, Re_eq, Rs_eq, c_squared, over_c_squared;
    /* device copy of this view: kernels read the ephemeris through it (a
     * by-value kernel parameter indexed with run-time indices would be
     * copied into every thread's local memory) */
    const struct DevEphem* self_dev;
};

/* isnormal() for a non-negative argument (the IAS15 error measures take
 * maxima of |a| and |b|): at least the smallest normal double and finite;
 * false for 0, subnormals, Inf and NaN. */
__device__ __forceinline__ bool ag_isnormal_pos(double a) {
    /* a >= DBL_MIN && a <= DBL_MAX, on the high word (an integer compare
     * rather than two FP64 ones): sign clear and exponent field 1..2046 */
    return (unsigned)__double2hiint(a) - 0x00100000u <= 0x7FEFFFFFu - 0x00100000u;
}
/* The larger of two non-negative doubles (or zero and a normal value): their
 * bit patterns order as integers do, compared on the integer pipes. */
__device__ __forceinline__ double ag_max_nonneg(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    return __longlong_as_double(ia > ib ? ia : ib);
}

/* Sub-interval b of tt = record fraction x niv and the integer part fl with
 * tau = 2 (tt - fl) - 1, as src/ascii_ephem.c:35-39 takes them: b = (int)tt
 * and fmod(tt, 1) = tt - trunc(tt) (exact).  A time a rounding below a record
 * boundary gives a tiny negative tt: b = 0, tau just below -1, the record's
 * start.  At tt == niv exactly the reference reads one sub-interval past the
 * column; here b stays in the last sub-interval, at its end (tau = +1). */
__device__ __forceinline__ int ag_subinterval(double tt, int niv, double* fl) {
    int b = (int)tt;
    double f = trunc(tt);
    if (b >= niv) { b = niv - 1; f = (double)(niv - 1); }
    *fl = f;
    return b;
}

/* Planet record selection shared by all eleven planets at one time
 * (src/ascii_ephem.c:294-300).  Returns AG_OK or AG_ERR_COVERAGE. */
__device__ __forceinline__ int ag_planet_record(const DevEphem& E, double t, const double** rec, double* tf) {
    const double jd = E.jd_ref + t;
    if (!(jd >= E.pl_beg && jd <= E.pl_end)) return AG_ERR_COVERAGE;   /* NaN too */
    const double num = E.jd_ref + t - E.pl_beg;
    const uint32_t blk = (uint32_t)(E.pl_inc_pow2 ? num * E.pl_inv_inc : num / E.pl_inc);
    if ((long long)blk + 2 >= (long long)E.pl_nrec) return AG_ERR_COVERAGE;
    *rec = E.pl_data + (size_t)(blk + 2) * (size_t)E.pl_rec_len;
    const double fr = (E.jd_ref - E.pl_beg - (double)blk * E.pl_inc) + t;
    *tf = E.pl_inc_pow2 ? fr * E.pl_inv_inc : fr / E.pl_inc;
    return AG_OK;
}

/* One .440 column: position in km (multiply by inv_cau for AU) and optionally
 * velocity already in AU/day.  tf is the record fraction in [0,1]. */
template <bool VEL>
__device__ __forceinline__ void ag_column(const DevEphem& E, const double* rec, int col, double tf,
                                          double* u, double* v) {
    const int ncf = E.col_ncf[col], niv = E.col_niv[col];
    const double tt = tf * (double)niv;
    double fl;
    const int b = ag_subinterval(tt, niv, &fl);
    const double tau = 2.0 * (tt - fl) - 1.0;
    const double two_tau = 2.0 * tau;
    const double* P = rec + E.col_off[col] + ncf * 3 * b;
    /* Chebyshev T_p(tau) and S_p = dT_p/dtau by their three-term recurrences */
    double T0 = 1.0, T1 = tau, S0 = 0.0, S1 = 1.0;
    double ux = P[0] + tau * P[1], uy = P[ncf] + tau * P[ncf + 1], uz = P[2 * ncf] + tau * P[2 * ncf + 1];
    double vx = 0.0, vy = 0.0, vz = 0.0;
    if (VEL) { vx = P[1]; vy = P[ncf + 1]; vz = P[2 * ncf + 1]; }
#pragma unroll 4
    for (int p = 2; p < ncf; p++) {
        const double T2 = fma(two_tau, T1, -T0);
        ux = fma(T2, P[p], ux);
        uy = fma(T2, P[ncf + p], uy);
        uz = fma(T2, P[2 * ncf + p], uz);
        if (VEL) {
            const double S2 = fma(two_tau, S1, fma(2.0, T1, -S0));
            vx = fma(S2, P[p], vx);
            vy = fma(S2, P[ncf + p], vy);
            vz = fma(S2, P[2 * ncf + p], vz);
            S0 = S1; S1 = S2;
        }
        T0 = T1; T1 = T2;
    }
    u[0] = ux; u[1] = uy; u[2] = uz;
    if (VEL) {
        const double c = E.col_vscale[col];
        v[0] = vx * c; v[1] = vy * c; v[2] = vz * c;
    }
}

/* Column of ASSIST body index (Earth and Moon are handled by the caller). */
__device__ __forceinline__ int ag_col_of(int body) {
    switch (body) {
        case AG_SUN: return AG_C_SUN;
        case AG_MER: return AG_C_MER;
        case AG_VEN: return AG_C_VEN;
        case AG_MAR: return AG_C_MAR;
        case AG_JUP: return AG_C_JUP;
        case AG_SAT: return AG_C_SAT;
        case AG_URA: return AG_C_URA;
        case AG_NEP: return AG_C_NEP;
        default: return AG_C_PLU;
    }
}

/* Full state of planet `body` (0..10): GM, position, velocity, acceleration
 * in AU and days, with the exact arithmetic of assist_ascii_calc
 * (defined after the exact column evaluator below). */
__device__ inline int ag_planet_full(const DevEphem& E, int body, double t, double* out);

/* Heliocentric asteroid position (AU) from its SPK type-2 segment
 * (src/spk.c:428-474): segment n from the target's epoch step, record b,
 * z = (t - MID)/RADIUS, sum of T_p(z) times the X/Y/Z coefficients, km -> AU
 * with ASSIST's fixed 149597870.7. */
__device__ __forceinline__ int ag_asteroid_pos(const DevEphem& E, int m, double t, double* p) {
    const double jd = E.jd_ref + t;
    if (!(jd >= E.ast_beg[m] && jd <= E.ast_end[m])) return AG_ERR_COVERAGE;   /* NaN too */
    int n = 0;
    if (E.ast_nseg[m] > 1) {
        n = (int)((E.jd_ref + t - E.ast_beg[m]) / E.ast_res[m]);
        if (n >= E.ast_nseg[m]) n = E.ast_nseg[m] - 1;
    }
    const AgSpkSeg sg = E.segs[E.ast_seg0[m] + n];
    int b = (int)(((E.jd_ref - sg.init_jd) + t) * sg.inv_intlen_days);
    if (b >= sg.nrec) b = sg.nrec - 1;
    if (b < 0) b = 0;
    const AgRecMeta meta = E.rec_meta[sg.meta_off + b];
    const double* X = E.spk + sg.data_off + (size_t)b * sg.R + 2;
    const int P = sg.P;
    const double z = ((E.jd_ref - meta.x) + t) * meta.z;
    const double two_z = 2.0 * z;
    double T0 = 1.0, T1 = z;
    double px = fma(z, X[1], X[0]), py = fma(z, X[P + 1], X[P]), pz = fma(z, X[2 * P + 1], X[2 * P]);
#pragma unroll 4
    for (int q = 2; q < P; q++) {
        const double T2 = fma(two_z, T1, -T0);
        px = fma(T2, X[q], px);
        py = fma(T2, X[P + q], py);
        pz = fma(T2, X[2 * P + q], pz);
        T0 = T1; T1 = T2;
    }
    const double s = 1.0 / 149597870.7;
    p[0] = px * s; p[1] = py * s; p[2] = pz * s;
    return AG_OK;
}

/* ---------------------------------------------------------------------------
 * Exact evaluators: ASSIST's arithmetic operation for operation (no FMA
 * contraction, the same association, true IEEE divisions), so body states
 * agree with the reference bit for bit.  Used wherever a body is evaluated
 * once for many particles (per-time tables); close approaches need it:
 * 1 ulp of the Earth's position (1e-16 AU) is a 1e-12 relative change of the
 * acceleration of a particle 1e-4 AU from the Earth.
 * ------------------------------------------------------------------------- */

/* .440 column in km and km/s (src/ascii_ephem.c:27-65). */
template <bool VEL>
__device__ __forceinline__ void ag_column_exact(const DevEphem& E, const double* rec, int col, double tf, double* u,
                                                double* v) {
    const int ncf = E.col_ncf[col], niv = E.col_niv[col];
    const double tt = __dmul_rn(tf, (double)niv);
    double fl;
    const int b = ag_subinterval(tt, niv, &fl);
    const double t0 = __dsub_rn(__dmul_rn(2.0, __dsub_rn(tt, fl)), 1.0);
    const double two_t0 = __dmul_rn(2.0, t0);
    const double* P = rec + E.col_off[col] + ncf * 3 * b;
    double ux = 0.0, uy = 0.0, uz = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
    double c = 0.0;
    if (VEL) c = __ddiv_rn(__ddiv_rn((double)(niv * 2), E.pl_inc), 86400.0);
    double T0 = 1.0, T1 = t0, S0 = 0.0, S1 = 1.0;
    for (int p = 0; p < ncf; p++) {
        double Tp, Sp;
        if (p == 0) { Tp = 1.0; Sp = 0.0; }
        else if (p == 1) { Tp = t0; Sp = 1.0; }
        else {
            Tp = __dsub_rn(__dmul_rn(two_t0, T1), T0);
            if (VEL) Sp = __dsub_rn(__dadd_rn(__dmul_rn(two_t0, S1), __dmul_rn(2.0, T1)), S0);
            T0 = T1; T1 = Tp;
            if (VEL) { S0 = S1; S1 = Sp; }
        }
        ux = __dadd_rn(ux, __dmul_rn(Tp, P[p]));
        uy = __dadd_rn(uy, __dmul_rn(Tp, P[ncf + p]));
        uz = __dadd_rn(uz, __dmul_rn(Tp, P[2 * ncf + p]));
        if (VEL) {
            vx = __dadd_rn(vx, __dmul_rn(__dmul_rn(Sp, P[p]), c));
            vy = __dadd_rn(vy, __dmul_rn(__dmul_rn(Sp, P[ncf + p]), c));
            vz = __dadd_rn(vz, __dmul_rn(__dmul_rn(Sp, P[2 * ncf + p]), c));
        }
    }
    u[0] = ux; u[1] = uy; u[2] = uz;
    if (VEL) { v[0] = vx; v[1] = vy; v[2] = vz; }
}

/* Planet `body` position (AU) and, if VEL, velocity (AU/day), exactly as
 * assist_ascii_calc forms them (src/ascii_ephem.c:302-380). */
template <bool VEL>
__device__ __forceinline__ void ag_planet_exact(const DevEphem& E, const double* rec, double tf, int body, double* x,
                                                double* v) {
    double u[3], w[3];
    if (body == AG_EAR || body == AG_MOO) {
        double eu[3], ev[3], lu[3], lv[3];
        ag_column_exact<VEL>(E, rec, AG_C_EMB, tf, eu, ev);
        ag_column_exact<VEL>(E, rec, AG_C_LUN, tf, lu, lv);
        const double f = body == AG_EAR ? E.f_earth : E.f_moon;
        for (int k = 0; k < 3; k++) {
            u[k] = __dadd_rn(eu[k], __dmul_rn(lu[k], f));
            if (VEL) w[k] = __dadd_rn(ev[k], __dmul_rn(lv[k], f));
        }
    } else {
        ag_column_exact<VEL>(E, rec, ag_col_of(body), tf, u, w);
    }
    for (int k = 0; k < 3; k++) {
        x[k] = __ddiv_rn(u[k], E.pl_cau);
        if (VEL) v[k] = __ddiv_rn(w[k], E.cau_per_day);
    }
}

/* .440 column position, velocity and acceleration (U = d2T/dtau2) with the
 * exact arithmetic of src/ascii_ephem.c:27-65 (km, km/s, km/s^2). */
__device__ __forceinline__ void ag_column_pva_exact(const DevEphem& E, const double* rec, int col, double tf, double* u,
                                                    double* v, double* w) {
    const int ncf = E.col_ncf[col], niv = E.col_niv[col];
    const double tt = __dmul_rn(tf, (double)niv);
    double fl;
    const int b = ag_subinterval(tt, niv, &fl);
    const double t0 = __dsub_rn(__dmul_rn(2.0, __dsub_rn(tt, fl)), 1.0);
    const double two_t0 = __dmul_rn(2.0, t0);
    const double c = __ddiv_rn(__ddiv_rn((double)(niv * 2), E.pl_inc), 86400.0);
    const double* P = rec + E.col_off[col] + ncf * 3 * b;
    double T[AG_MAX_NCF], S[AG_MAX_NCF], U[AG_MAX_NCF];
    T[0] = 1.0; T[1] = t0; S[0] = 0.0; S[1] = 1.0; U[0] = 0.0; U[1] = 0.0; U[2] = 4.0;
    for (int p = 2; p < ncf; p++) {
        T[p] = __dsub_rn(__dmul_rn(two_t0, T[p - 1]), T[p - 2]);
        S[p] = __dsub_rn(__dadd_rn(__dmul_rn(two_t0, S[p - 1]), __dmul_rn(2.0, T[p - 1])), S[p - 2]);
    }
    for (int p = 3; p < ncf; p++)
        U[p] = __dsub_rn(__dadd_rn(__dmul_rn(two_t0, U[p - 1]), __dmul_rn(4.0, S[p - 1])), U[p - 2]);
    for (int m = 0; m < 3; m++) {
        double su = 0.0, sv = 0.0, sw = 0.0;
        for (int p = 0; p < ncf; p++) {
            const double cf = P[m * ncf + p];
            su = __dadd_rn(su, __dmul_rn(T[p], cf));
            sv = __dadd_rn(sv, __dmul_rn(__dmul_rn(S[p], cf), c));
            sw = __dadd_rn(sw, __dmul_rn(__dmul_rn(__dmul_rn(U[p], cf), c), c));
        }
        u[m] = su; v[m] = sv; w[m] = sw;
    }
}

static __device__ __noinline__ int ag_spk_planet(const DevEphem& E, int body, double t, double* out);

__device__ inline int ag_planet_full(const DevEphem& E, int body, double t, double* out) {
    if (E.pl_spk) return ag_spk_planet(E, body, t, out);
    const double* rec;
    double tf;
    out[0] = E.gm[body];
    int st = ag_planet_record(E, t, &rec, &tf);
    if (st != AG_OK) return st;
    double u[3], v[3], w[3];
    if (body == AG_EAR || body == AG_MOO) {
        double eu[3], ev[3], ew[3], lu[3], lv[3], lw[3];
        ag_column_pva_exact(E, rec, AG_C_EMB, tf, eu, ev, ew);
        ag_column_pva_exact(E, rec, AG_C_LUN, tf, lu, lv, lw);
        const double f = body == AG_EAR ? E.f_earth : E.f_moon;
        for (int k = 0; k < 3; k++) {
            u[k] = __dadd_rn(eu[k], __dmul_rn(lu[k], f));
            v[k] = __dadd_rn(ev[k], __dmul_rn(lv[k], f));
            w[k] = __dadd_rn(ew[k], __dmul_rn(lw[k], f));
        }
    } else {
        ag_column_pva_exact(E, rec, ag_col_of(body), tf, u, v, w);
    }
    const double acc_div = E.pl_cau / (86400. * 86400.);
    for (int k = 0; k < 3; k++) {
        out[1 + k] = __ddiv_rn(u[k], E.pl_cau);
        out[4 + k] = __ddiv_rn(v[k], E.cau_per_day);
        out[7 + k] = __ddiv_rn(w[k], acc_div);
    }
    return AG_OK;
}

/* Position, velocity and acceleration sums (km, km/s, km/s^2) of planets-SPK
 * slot `slot` at time t, in the operations and order of
 * assist_spk_target_pos (src/spk.c:492-548): segment n from the target's
 * begin epoch and step, record b from the segment directory, z from the
 * record's MID and RADIUS, T/S/U recurrences, c = 1/RADIUS[s]. */
static __device__ __noinline__ void ag_spk_target_pva(const DevEphem& E, int slot, double t, double* u, double* v, double* w) {
    int n = (int)__ddiv_rn(__dsub_rn(__dadd_rn(E.jd_ref, t), E.ps_beg[slot]), E.ps_res[slot]);
    if (n >= E.ps_nseg[slot]) n = E.ps_nseg[slot] - 1;
    if (n < 0) n = 0;
    const AgSpkSeg sg = E.psegs[E.ps_seg0[slot] + n];
    int b = (int)(__ddiv_rn(__dadd_rn(__dsub_rn(E.jd_ref, sg.init_jd), t), sg.intlen_days));
    if (b >= sg.nrec) b = sg.nrec - 1;
    if (b < 0) b = 0;
    const AgRecMeta meta = E.pmeta[sg.meta_off + b];
    const double* val = E.pspk + sg.data_off + (size_t)b * sg.R;
    const int P = sg.P;
    const double z = __ddiv_rn(__dadd_rn(__dsub_rn(E.jd_ref, meta.x), t), meta.y);
    const double c = __ddiv_rn(1.0, val[1]);
    const double two_z = __dmul_rn(2.0, z);
    double T[AG_MAX_SPK_P], S[AG_MAX_SPK_P], U[AG_MAX_SPK_P];
    T[0] = 1.0; T[1] = z; S[0] = 0.0; S[1] = 1.0; U[0] = 0.0; U[1] = 0.0; U[2] = 4.0;
    for (int p = 2; p < P; p++) {
        T[p] = __dsub_rn(__dmul_rn(two_z, T[p - 1]), T[p - 2]);
        S[p] = __dsub_rn(__dadd_rn(__dmul_rn(two_z, S[p - 1]), __dmul_rn(2.0, T[p - 1])), S[p - 2]);
    }
    for (int p = 3; p < P; p++)
        U[p] = __dsub_rn(__dadd_rn(__dmul_rn(two_z, U[p - 1]), __dmul_rn(4.0, S[p - 1])), U[p - 2]);
    for (int k = 0; k < 3; k++) {
        const double* cf = val + 2 + k * P;
        double su = 0.0, sv = 0.0, sw = 0.0;
        for (int p = 0; p < P; p++) {
            su = __dadd_rn(su, __dmul_rn(cf[p], T[p]));
            sv = __dadd_rn(sv, __dmul_rn(__dmul_rn(cf[p], S[p]), c));
            sw = __dadd_rn(sw, __dmul_rn(__dmul_rn(__dmul_rn(cf[p], U[p]), c), c));
        }
        u[k] = su; v[k] = sv; w[k] = sw;
    }
}

/* Planet `body` from the planets SPK file as ASSIST's
 * assist_spk_calc_planets_from_target forms it (src/spk.c:550-608): Earth
 * and Moon plus the Earth-Moon barycentre, then km -> AU, AU/day, AU/day^2.
 * out: GM, x,y,z, vx,vy,vz, ax,ay,az. */
static __device__ __noinline__ int ag_spk_planet(const DevEphem& E, int body, double t, double* out) {
    const double jd = E.jd_ref + t;
    out[0] = E.gm[body];
    if (E.ps_nseg[body] <= 0) return AG_ERR_NEPHEM;
    if (!(jd >= E.ps_beg[body] && jd <= E.ps_end[body])) return AG_ERR_COVERAGE;   /* NaN too */
    double u[3], v[3], w[3];
    ag_spk_target_pva(E, body, t, u, v, w);
    if (body == AG_EAR || body == AG_MOO) {
        double eu[3], ev[3], ew[3];
        ag_spk_target_pva(E, AG_NPL, t, eu, ev, ew);
        for (int k = 0; k < 3; k++) { u[k] = __dadd_rn(u[k], eu[k]); v[k] = __dadd_rn(v[k], ev[k]); w[k] = __dadd_rn(w[k], ew[k]); }
    }
    const double vdiv = __ddiv_rn(E.au_km, 86400.);
    const double adiv = __ddiv_rn(E.au_km, __dmul_rn(86400., 86400.));
    for (int k = 0; k < 3; k++) {
        out[1 + k] = __ddiv_rn(u[k], E.au_km);
        out[4 + k] = __ddiv_rn(v[k], vdiv);
        out[7 + k] = __ddiv_rn(w[k], adiv);
    }
    return AG_OK;
}

/* Asteroid heliocentric position (AU), exactly as assist_spk_calc forms it
 * (src/spk.c:428-474). */
__device__ __forceinline__ int ag_asteroid_exact(const DevEphem& E, int m, double t, double* p) {
    const double jd = E.jd_ref + t;
    if (!(jd >= E.ast_beg[m] && jd <= E.ast_end[m])) return AG_ERR_COVERAGE;   /* NaN too */
    int n = 0;
    if (E.ast_nseg[m] > 1) {
        n = (int)((E.jd_ref + t - E.ast_beg[m]) / E.ast_res[m]);
        if (n >= E.ast_nseg[m]) n = E.ast_nseg[m] - 1;
    }
    const AgSpkSeg sg = E.segs[E.ast_seg0[m] + n];
    int b = (int)(__ddiv_rn(__dadd_rn(__dsub_rn(E.jd_ref, sg.init_jd), t), sg.intlen_days));
    if (b >= sg.nrec) b = sg.nrec - 1;
    if (b < 0) b = 0;
    const AgRecMeta meta = E.rec_meta[sg.meta_off + b];
    const double* X = E.spk + sg.data_off + (size_t)b * sg.R + 2;
    const int P = sg.P;
    const double z = __ddiv_rn(__dadd_rn(__dsub_rn(E.jd_ref, meta.x), t), meta.y);
    const double two_z = __dmul_rn(2.0, z);
    double px = 0.0, py = 0.0, pz = 0.0, T0 = 1.0, T1 = z;
    for (int q = 0; q < P; q++) {
        double Tq;
        if (q == 0) Tq = 1.0;
        else if (q == 1) Tq = z;
        else { Tq = __dsub_rn(__dmul_rn(two_z, T1), T0); T0 = T1; T1 = Tq; }
        px = __dadd_rn(px, __dmul_rn(X[q], Tq));
        py = __dadd_rn(py, __dmul_rn(X[P + q], Tq));
        pz = __dadd_rn(pz, __dmul_rn(X[2 * P + q], Tq));
    }
    p[0] = __ddiv_rn(px, 149597870.7); p[1] = __ddiv_rn(py, 149597870.7); p[2] = __ddiv_rn(pz, 149597870.7);
    return AG_OK;
}

#endif
