/*
 * warp_table.cuh -- the body table of one time, built by one warp with every
 * lane busy (used by the warp-synchronous batched IAS15).
 *
 * Work is split by column COMPONENT, not by body: each lane owns one
 * (column, x|y|z) pair and forms its Chebyshev sum in ASSIST's exact order
 * (src/ascii_ephem.c:54-63), so the table is bit-identical to the
 * reference's body states while the critical path is the longest single
 * column (14 coefficients) instead of a whole body.  Then one lane per
 * (planet, component) converts km to AU and forms Earth/Moon from the
 * Earth-Moon barycentre; one lane per (asteroid, component) sums the SPK
 * record (src/spk.c:428-474); the EIH source sums over the other planets are
 * a lane-parallel reduction.
 */
#ifndef ASSIST_GB300_WARP_TABLE_CUH
#define ASSIST_GB300_WARP_TABLE_CUH

#include "device_forces.cuh"

/* Raw column sums of one time (km, km/s) in shared memory. */
struct AgWarpScratch {
    double col[11][3];       /* columns MER VEN EMB MAR JUP SAT URA NEP PLU LUN SUN */
    double sun_v[3];         /* Sun velocity sums */
};

/* One component sum of a .440 column with the exact arithmetic; VEL also
 * forms the velocity sum (S recurrence, times c per term). */
template <bool VEL>
__device__ __forceinline__ double ag_colcomp_exact(const DevEphem& E, const double* rec, int col, int comp, double tf,
                                                   double* vsum) {
    const int ncf = E.col_ncf[col], niv = E.col_niv[col];
    const double tt = __dmul_rn(tf, (double)niv);
    double fl;
    const int b = ag_subinterval(tt, niv, &fl);
    const double t0 = __dsub_rn(__dmul_rn(2.0, __dsub_rn(tt, fl)), 1.0);
    const double two_t0 = __dmul_rn(2.0, t0);
    const double* P = rec + E.col_off[col] + ncf * (3 * b + comp);
    double c = 0.0;
    if (VEL) c = __ddiv_rn(__ddiv_rn((double)(niv * 2), E.pl_inc), 86400.0);
    double u = 0.0, v = 0.0, T0 = 1.0, T1 = t0, S0 = 0.0, S1 = 1.0;
    for (int p = 0; p < ncf; p++) {
        double Tp, Sp = 0.0;
        if (p == 0) { Tp = 1.0; Sp = 0.0; }
        else if (p == 1) { Tp = t0; Sp = 1.0; }
        else {
            Tp = __dsub_rn(__dmul_rn(two_t0, T1), T0);
            if (VEL) { Sp = __dsub_rn(__dadd_rn(__dmul_rn(two_t0, S1), __dmul_rn(2.0, T1)), S0); S0 = S1; S1 = Sp; }
            T0 = T1; T1 = Tp;
        }
        u = __dadd_rn(u, __dmul_rn(Tp, P[p]));
        if (VEL) v = __dadd_rn(v, __dmul_rn(__dmul_rn(Sp, P[p]), c));
    }
    if (VEL) *vsum = v;
    return u;
}

/* Per-component asteroid position (AU, heliocentric), exact arithmetic. */
__device__ __forceinline__ int ag_astcomp_exact(const DevEphem& E, int m, int comp, double t, double* out) {
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
    const int P = sg.P;
    const double* X = E.spk + sg.data_off + (size_t)b * sg.R + 2 + comp * P;
    const double z = __ddiv_rn(__dadd_rn(__dsub_rn(E.jd_ref, meta.x), t), meta.y);
    const double two_z = __dmul_rn(2.0, z);
    double s = 0.0, T0 = 1.0, T1 = z;
    for (int q = 0; q < P; q++) {
        double Tq;
        if (q == 0) Tq = 1.0;
        else if (q == 1) Tq = z;
        else { Tq = __dsub_rn(__dmul_rn(two_z, T1), T0); T0 = T1; T1 = Tq; }
        s = __dadd_rn(s, __dmul_rn(X[q], Tq));
    }
    *out = __ddiv_rn(s, 149597870.7);
    return AG_OK;
}

/* Velocity of a further EIH source, or of the geocentric Earth (rare
 * configurations; kept out of line). */
static __device__ __noinline__ void ag_table_velocity(const DevEphem& E, const double* rec, double tf, int body, AgTable& T) {
    double u[3], v[3];
    ag_planet_exact<true>(E, rec, tf, body, u, v);
    T.P.vx[body] = v[0]; T.P.vy[body] = v[1]; T.P.vz[body] = v[2];
}

/* Earth's barycentric acceleration for the geocentric frame. */
static __device__ __noinline__ void ag_table_earth_acc(const DevEphem& E, double t, AgTable& T) {
    double e_[10];
    ag_planet_full(E, AG_EAR, t, e_);
    T.P.ex_a[0] = e_[7]; T.P.ex_a[1] = e_[8]; T.P.ex_a[2] = e_[9];
}

/* Asteroids (barycentric, from the table's Sun) and the EIH per-source sums
 * of a table whose planets are in place; warp-uniform status. */
__device__ __forceinline__ int ag_warp_table_rest(const DevEphem& E, const ForceCfg& c, double t, AgTable& T, int lane) {
    /* ---- phase C: asteroid components (3 lanes per asteroid) */
    int ast_st = AG_OK;
    for (int task = lane; task < 3 * E.n_ast; task += 32) {
        const int m = task / 3, comp = task % 3;
        double h;
        const int s2 = ag_astcomp_exact(E, m, comp, t, &h);
        if (s2 != AG_OK) ast_st = s2;
        const double sun = comp == 0 ? T.P.x[AG_SUN] : (comp == 1 ? T.P.y[AG_SUN] : T.P.z[AG_SUN]);
        T.ast[m][comp] = __dadd_rn(h, sun);
    }
    __syncwarp();
    /* ---- phase D: per-source EIH sums, one lane per other planet */
    if (c.forces & AG_F_EIH) {
        for (int j = 0; j < c.gr_eih_sources && j < AG_NPL; j++) {
            double ax = 0.0, ay = 0.0, az = 0.0, s1 = 0.0;
            if (lane < AG_NPL && lane != j) {
                const int k = lane;
                const double dx = T.P.x[j] - T.P.x[k], dy = T.P.y[j] - T.P.y[k], dz = T.P.z[j] - T.P.z[k];
                const double ri = rsqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
                const double gri = E.gm[k] * ri;
                s1 = gri;
                const double f = gri * ri * ri;
                ax = -f * dx; ay = -f * dy; az = -f * dz;
            }
            for (int o = 8; o > 0; o >>= 1) {
                ax += __shfl_down_sync(0xffffffffu, ax, o, 16);
                ay += __shfl_down_sync(0xffffffffu, ay, o, 16);
                az += __shfl_down_sync(0xffffffffu, az, o, 16);
                s1 += __shfl_down_sync(0xffffffffu, s1, o, 16);
            }
            if (lane == 0) { T.eih_a[j][0] = ax; T.eih_a[j][1] = ay; T.eih_a[j][2] = az; T.eih_t1[j] = s1; }
        }
    }
    if (!(c.forces & (AG_F_SUN | AG_F_PLANETS | AG_F_AST))) ast_st = AG_OK;
    __syncwarp();
    const unsigned bad = __ballot_sync(0xffffffffu, ast_st != AG_OK);
    if (lane == 0) T.status = AG_OK;
    __syncwarp();
    return bad ? AG_ERR_COVERAGE : AG_OK;
}

/* The planets of the table from a planets SPK file: one lane per body, full
 * state (src/spk.c:550-608).  Returns a warp-uniform status. */
static __device__ __noinline__ int ag_warp_planets_spk(const DevEphem& E, const ForceCfg& c, double t, AgTable& T, int lane) {
    int st = AG_OK;
    if (lane < AG_NPL) {
        double o[10];
        st = ag_spk_planet(E, lane, t, o);
        T.P.x[lane] = o[1]; T.P.y[lane] = o[2]; T.P.z[lane] = o[3];
        T.P.vx[lane] = o[4]; T.P.vy[lane] = o[5]; T.P.vz[lane] = o[6];
        if (lane == AG_EAR && c.geocentric == 1) { T.P.ex_a[0] = o[7]; T.P.ex_a[1] = o[8]; T.P.ex_a[2] = o[9]; }
    }
    __syncwarp();
    return __any_sync(0xffffffffu, st != AG_OK) ? AG_ERR_COVERAGE : AG_OK;
}

/* Build the table of time t with the whole warp.  Returns a warp-uniform
 * status.  Falls back to body-per-lane velocities when more EIH sources than
 * the Sun need velocities (rare configuration). */
static __device__ __noinline__ int ag_warp_table_fast(const DevEphem& E, const ForceCfg& c, double t, AgTable& T, AgWarpScratch& S,
                                  int lane) {
    if (E.pl_spk) {
        const int sp = ag_warp_planets_spk(E, c, t, T, lane);
        if (sp != AG_OK) return sp;
        return ag_warp_table_rest(E, c, t, T, lane);
    }
    const double* rec = nullptr;
    double tf = 0.0;
    int st = ag_planet_record(E, t, &rec, &tf);
    if (st != AG_OK) return st;
    int nv = (c.forces & AG_F_EIH) ? c.gr_eih_sources : 0;
    if (c.geocentric) nv = nv > AG_EAR + 1 ? nv : AG_EAR + 1;
    /* ---- phase A: 33 column components (+3 Sun velocity sums) over 32 lanes.
     * Lanes 0..2: Sun x,y,z with velocity; lanes 3..32 the other 10 columns;
     * the 33rd task (Pluto z) rides on lane 31 after its own. */
    {
        int task = lane;                       /* 0..31 */
        for (int pass = 0; pass < 2; pass++) {
            if (pass == 1) { if (lane != 31) break; task = 32; }
            /* task 0..2: Sun; 3..32: columns MER..LUN (indices 0..9) */
            const int col = task < 3 ? AG_C_SUN : (task - 3) / 3;
            const int comp = task < 3 ? task : (task - 3) % 3;
            if (col == AG_C_SUN) {
                double vs;
                S.col[col][comp] = ag_colcomp_exact<true>(E, rec, col, comp, tf, &vs);
                S.sun_v[comp] = vs;
            } else {
                S.col[col][comp] = ag_colcomp_exact<false>(E, rec, col, comp, tf, nullptr);
            }
        }
    }
    __syncwarp();
    /* ---- phase B: km -> AU, Earth/Moon from EMB and Moon; Sun velocity */
    for (int task = lane; task < 36; task += 32) {
        if (task < 33) {
            const int b = task / 3, comp = task % 3;
            double u;
            if (b == AG_EAR) u = __dadd_rn(S.col[AG_C_EMB][comp], __dmul_rn(S.col[AG_C_LUN][comp], E.f_earth));
            else if (b == AG_MOO) u = __dadd_rn(S.col[AG_C_EMB][comp], __dmul_rn(S.col[AG_C_LUN][comp], E.f_moon));
            else u = S.col[ag_col_of(b)][comp];
            const double x = __ddiv_rn(u, E.pl_cau);
            if (comp == 0) T.P.x[b] = x; else if (comp == 1) T.P.y[b] = x; else T.P.z[b] = x;
        } else {
            const int comp = task - 33;
            const double v = __ddiv_rn(S.sun_v[comp], E.cau_per_day);
            if (comp == 0) T.P.vx[AG_SUN] = v; else if (comp == 1) T.P.vy[AG_SUN] = v; else T.P.vz[AG_SUN] = v;
        }
    }
    __syncwarp();
    if (nv > 1 && lane > 0 && lane < nv && lane < AG_NPL) ag_table_velocity(E, rec, tf, lane, T);
    if (c.geocentric == 1 && lane == AG_EAR) ag_table_earth_acc(E, t, T);
    return ag_warp_table_rest(E, c, t, T, lane);
}

#endif
