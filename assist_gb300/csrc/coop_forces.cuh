/*
 * coop_forces.cuh -- block-cooperative body tables and force evaluation:
 * the body table of one time built by a 128-thread block (column components
 * of the .440 record and asteroid components on different threads, optionally
 * from the record staged in shared memory by a bulk copy), and the force on a
 * particle split into four warp shares (warp 0: planets' direct gravity,
 * non-gravitational term, Earth J2-J4; warp 1: EIH/PPN relativity and the GR
 * terms; warps 2 and 3: the asteroids, Earth J2-J4 with Jacobians, Sun J2)
 * whose partial sums the caller adds ((w3 + w2) + w1) + w0.  Used by the
 * block-cooperative batched kernel (ias15_coop.cuh) and by the shared-step
 * step kernel (kernels_shared.cu).
 */
#ifndef ASSIST_GB300_COOP_FORCES_CUH
#define ASSIST_GB300_COOP_FORCES_CUH

#include "device_forces.cuh"
#include "ieee_convert.cuh"
#include "warp_table.cuh"

#ifndef AG_FULL
#define AG_FULL 0xffffffffu
#endif

/* Raw sums of one substep time, shared by the block. */
struct AgCoopScratch {
    double col[11][3];              /* .440 column position sums (km) */
    double sun_v[3];                /* Sun velocity sums (km/s) */
    double ast_h[AG_MAX_AST][3];    /* heliocentric asteroid positions (AU) */
};

/* The block's body tables are formed with fused multiply-adds and
 * multiplications by reciprocals: within an ulp or two of the reference's
 * operations (a 1e-16 relative change of a body position, far below the
 * 1e-14 acceleration bar; the drop-in callback, the per-evaluation kernels
 * and the independent-step kernel keep the reference's exact arithmetic).
 * The tables are rebuilt for every step's eight node times and are a large
 * share of a step's FP64 work: the exact sums take a multiply and an add per
 * term and the reference's divisions expand to many FP64 instructions. */

/* One component of a .440 column (km): the position sum and, with VEL, the
 * velocity sum (km/s). */
template <bool VEL>
__device__ __forceinline__ double ag_colcomp_fused(const DevEphem& E, const double* rec, int col, int comp, double tf,
                                                   double* vsum) {
    const int ncf = E.col_ncf[col], niv = E.col_niv[col];
    const double tt = tf * (double)niv;
    double fl;
    const int b = ag_subinterval(tt, niv, &fl);
    const double t0 = fma(2.0, tt - fl, -1.0);
    const double two_t0 = 2.0 * t0;
    const double* P = rec + E.col_off[col] + ncf * (3 * b + comp);
    double u = fma(t0, P[1], P[0]), v = P[1];
    double T0 = 1.0, T1 = t0, S0 = 0.0, S1 = 1.0;
    for (int p = 2; p < ncf; p++) {
        const double Tp = fma(two_t0, T1, -T0);
        u = fma(Tp, P[p], u);
        if (VEL) {
            const double Sp = fma(two_t0, S1, fma(2.0, T1, -S0));
            v = fma(Sp, P[p], v);
            S0 = S1; S1 = Sp;
        }
        T0 = T1; T1 = Tp;
    }
    if (VEL) *vsum = v * ((double)(niv * 2) / E.pl_inc / 86400.0);
    return u;
}

/* One component of an asteroid's heliocentric position (AU) from its SPK
 * record, with the record's precomputed 1/RADIUS and the segment's
 * 1/INTLEN. */
__device__ __forceinline__ int ag_astcomp_fused(const DevEphem& E, int m, int comp, double t, double* out) {
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
    const int P = sg.P;
    const double* X = E.spk + sg.data_off + (size_t)b * sg.R + 2 + comp * P;
    const double z = ((E.jd_ref - meta.x) + t) * meta.z;
    const double two_z = 2.0 * z;
    double s = P > 1 ? fma(X[1], z, X[0]) : X[0], T0 = 1.0, T1 = z;
    for (int q = 2; q < P; q++) {
        const double Tq = fma(two_z, T1, -T0);
        s = fma(X[q], Tq, s);
        T0 = T1; T1 = Tq;
    }
    *out = s * (1.0 / 149597870.7);
    return AG_OK;
}

/* A value as the unevaluated sum hi + lo of two floats ("double-float",
 * about 48 significant bits), for arithmetic on the FP32 pipes, which on
 * GB300 retire 64 lanes for every lane of FP64 work. */
struct AgF2 {
    float h, l;
};

/* A body table of one substep time and, per body, the origin minus the body's
 * position: the particle-independent half of every separation
 * x + (xo - x_body) (src/forces.c), formed once per table rather than once
 * per particle: the eleven planets in FP64, the asteroids as float pairs (their
 * FP64 positions stay in T.ast). */
struct AgCoopTab {
    AgTable T;
    double rel[AG_NPL][3];
    AgF2 arel[AG_MAX_AST][3];
};

/* Double-float operations: Knuth's two-sum and Dekker's fast two-sum for
 * the addition, the product's rounding error from one fused multiply-add,
 * each result renormalised (the methods of Dekker 1971 and of the
 * double-double libraries built on them), written with round-to-nearest
 * intrinsics so that no operation is contracted or reordered. */
__device__ __forceinline__ AgF2 ag_f2_fast(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ AgF2 ag_f2_add(AgF2 a, AgF2 b) {
    const float s = __fadd_rn(a.h, b.h);
    const float bb = __fsub_rn(s, a.h);
    const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    return ag_f2_fast(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ AgF2 ag_f2_mul(AgF2 a, AgF2 b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return ag_f2_fast(p, e);
}
__device__ __forceinline__ AgF2 ag_f2_neg(AgF2 a) { return {-a.h, -a.l}; }
/* The split of a double and the sum back, their conversions on the integer
 * pipes (bit for bit the hardware's, which would occupy the FP64 pipe). */
__device__ __forceinline__ AgF2 ag_f2_of(double x) {
    const float h = ag_d2f_int(x);
    return {h, ag_d2f_int(x - ag_f2d_int(h))};
}
__device__ __forceinline__ double ag_f2_to(AgF2 a) { return ag_f2d_int(a.h) + ag_f2d_int(a.l); }
/* 1/sqrt(x): the FP32 estimate y0, then one Newton step in double-float,
 * y = y0 + y0 (1 - x y0^2) / 2 (relative error about 1.5 e0^2, a few 1e-14). */
__device__ __forceinline__ AgF2 ag_f2_rsqrt(AgF2 x) {
    const float y0 = rsqrtf(x.h);
    const AgF2 y = {y0, 0.0f};
    const AgF2 t = ag_f2_mul(x, ag_f2_mul(y, y));
    const AgF2 e = ag_f2_add({1.0f, 0.0f}, ag_f2_neg(t));
    return ag_f2_add(y, ag_f2_mul(e, {0.5f * y0, 0.0f}));
}

/* ---- The active .440 record staged in shared memory by a bulk (TMA) copy.
 *
 * One thread issues cp.async.bulk of the record (1,018 doubles, 8,144 bytes
 * for DE440's layout) from the device image into the block's buffer, with an
 * mbarrier counting the bytes; every thread waits on the barrier's phase.
 * Records are 32 days long, so a block re-stages only when its group's time
 * crosses into the next record: the eight node tables of a step and the
 * steps and groups after it read their Chebyshev coefficients from shared
 * memory.  The copy starts at the record's address rounded down to 16 bytes
 * and covers the record rounded up to 16 bytes (the device image carries 64
 * bytes of padding), as the bulk copy requires. */
#define AG_STAGE_BYTES 8192
#define AG_STAGE_MAX_REC ((AG_STAGE_BYTES - 16) / 8)     /* largest record (doubles) that fits with its offset */
#define AG_STAGE_WAIT_LIMIT (1 << 22)                    /* try_wait polls before a copy counts as lost */

struct AgRecStage {
    double buf[AG_STAGE_BYTES / 8];
    unsigned long long bar;        /* mbarrier: one arrival (the issuing thread) + the copied bytes */
};

/* Per-thread view of the staging state: the record held (identical in every
 * thread of the block) and the barrier phase to wait for next. */
struct AgStageCursor {
    const double* src = nullptr;
    unsigned phase = 0;
};

__device__ __forceinline__ void ag_mbar_init(unsigned long long* bar) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

/* Bounded wait for the barrier's phase `parity`; false when it did not
 * complete within AG_STAGE_WAIT_LIMIT polls. */
__device__ __forceinline__ bool ag_mbar_wait(unsigned long long* bar, unsigned parity) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    for (int it = 0; it < AG_STAGE_WAIT_LIMIT; it++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

/* Record `rec` (global) in the block's buffer: a bulk copy when it is not
 * the record already held.  Every thread of the block calls it with the same
 * rec.  Returns the record's first coefficient in shared memory; sets
 * *fail when the copy did not complete. */
__device__ __forceinline__ const double* ag_stage_record(const DevEphem& E, const double* rec, AgRecStage& R, int tid,
                                                         AgStageCursor& cur, int* fail) {
    const unsigned long long a = reinterpret_cast<unsigned long long>(rec);
    const unsigned long long al = a & ~15ull;
    const unsigned delta = (unsigned)(a - al);
    if (rec != cur.src) {
        const unsigned bytes = (delta + 8u * (unsigned)E.pl_rec_len + 15u) & ~15u;
        if (tid == 0) {
            const unsigned b = (unsigned)__cvta_generic_to_shared(&R.bar);
            const unsigned d = (unsigned)__cvta_generic_to_shared(R.buf);
            /* the buffer's previous contents were read by generic loads before
             * the caller's last barrier; order them before the async write */
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         ::"r"(d), "l"(al), "r"(bytes), "r"(b)
                         : "memory");
        }
        if (!ag_mbar_wait(&R.bar, cur.phase)) {
            *fail = 1;
            cur.src = nullptr;
        } else {
            cur.src = rec;
        }
        cur.phase ^= 1u;
    }
    return reinterpret_cast<const double*>(reinterpret_cast<const char*>(R.buf) + delta);
}

/* Table pass 1: column and asteroid component sums.  Returns this thread's
 * coverage status (combined by the caller's barrier).  STAGE: the .440
 * coefficients come from the record staged in shared memory (R, cur); a lost
 * copy sets *stage_fail. */
template <bool STAGE>
__device__ __forceinline__ int ag_coop_table_pass1(const DevEphem& E, const ForceCfg& c, double t, AgCoopScratch& S,
                                                   AgCoopTab& CT, int tid, AgRecStage* R, AgStageCursor& cur,
                                                   int* stage_fail) {
    AgTable& T = CT.T;
    int bad = 0;
    const double* srec = nullptr;    /* staged record (STAGE) */
    double stf = 0.0;
    if (STAGE && !E.pl_spk && E.pl_rec_len <= AG_STAGE_MAX_REC) {
        const double* grec = nullptr;
        if (ag_planet_record(E, t, &grec, &stf) == AG_OK) srec = ag_stage_record(E, grec, *R, tid, cur, stage_fail);
    }
    if (E.pl_spk) {
        /* planets from an SPK file: one thread of warp 1 per body, full state
         * straight into the table (src/spk.c:550-608) */
        if (tid >= 32 && tid < 32 + AG_NPL) {
            const int b = tid - 32;
            double o[10];
            if (ag_spk_planet(E, b, t, o) != AG_OK) bad = 1;
            T.P.x[b] = o[1]; T.P.y[b] = o[2]; T.P.z[b] = o[3];
            T.P.vx[b] = o[4]; T.P.vy[b] = o[5]; T.P.vz[b] = o[6];
            if (c.geocentric != 1) { CT.rel[b][0] = 0.0 - o[1]; CT.rel[b][1] = 0.0 - o[2]; CT.rel[b][2] = 0.0 - o[3]; }
            if (b == AG_EAR && c.geocentric == 1) { T.P.ex_a[0] = o[7]; T.P.ex_a[1] = o[8]; T.P.ex_a[2] = o[9]; }
        }
    } else if (tid < 64) {
        const int lane = tid & 31;
        const bool w0 = tid < 32;
        if ((w0 && lane < 30) || (!w0 && lane < 3)) {
            const double* rec = srec;
            double tf = stf;
            if (!rec && ag_planet_record(E, t, &rec, &tf) != AG_OK) {
                bad = 1;
            } else if (w0) {
                /* MER..LUN (columns 0..9), component lane % 3 */
                S.col[lane / 3][lane % 3] = ag_colcomp_fused<false>(E, rec, lane / 3, lane % 3, tf, nullptr);
            } else {
                double vs;
                S.col[AG_C_SUN][lane] = ag_colcomp_fused<true>(E, rec, AG_C_SUN, lane, tf, &vs);
                S.sun_v[lane] = vs;
            }
        }
    }
    if (tid >= 64) {
        /* asteroid components (both planets formats) */
        const bool need = (c.forces & (AG_F_SUN | AG_F_PLANETS | AG_F_AST)) != 0;
        for (int task = tid - 64; task < 3 * E.n_ast; task += 64) {
            double h = 0.0;
            if (ag_astcomp_fused(E, task / 3, task % 3, t, &h) != AG_OK && need) bad = 1;
            S.ast_h[task / 3][task % 3] = h;
        }
    }
    return bad;
}

/* Table pass 2: bodies in AU (Earth and Moon from the Earth-Moon barycentre),
 * the Sun's velocity, barycentric asteroids, further EIH velocities and the
 * geocentric Earth acceleration. */
__device__ __forceinline__ void ag_coop_table_pass2(const DevEphem& E, const ForceCfg& c, double t, AgCoopTab& CT,
                                                    const AgCoopScratch& S, int tid) {
    AgTable& T = CT.T;
    const bool bary = c.geocentric != 1;     /* origin at zero: rel = 0 - x_body */
    if (E.pl_spk) {
        /* planets are in place: only the barycentric asteroids */
        if (tid >= 64)
            for (int q = tid - 64; q < 3 * E.n_ast; q += 64) {
                const int comp = q % 3;
                const double sun = comp == 0 ? T.P.x[AG_SUN] : (comp == 1 ? T.P.y[AG_SUN] : T.P.z[AG_SUN]);
                const double xa = S.ast_h[q / 3][comp] + sun;
                T.ast[q / 3][comp] = xa;
                if (bary) CT.arel[q / 3][comp] = ag_f2_of(0.0 - xa);
            }
        return;
    }
    if (tid < 33) {
        const int b = tid / 3, comp = tid % 3;
        double u;
        if (b == AG_EAR) u = fma(S.col[AG_C_LUN][comp], E.f_earth, S.col[AG_C_EMB][comp]);
        else if (b == AG_MOO) u = fma(S.col[AG_C_LUN][comp], E.f_moon, S.col[AG_C_EMB][comp]);
        else u = S.col[ag_col_of(b)][comp];
        const double x = u * E.inv_cau;
        if (comp == 0) T.P.x[b] = x; else if (comp == 1) T.P.y[b] = x; else T.P.z[b] = x;
        if (bary) CT.rel[b][comp] = 0.0 - x;
    } else if (tid < 36) {
        const int comp = tid - 33;
        const double v = S.sun_v[comp] * (86400.0 * E.inv_cau);
        if (comp == 0) T.P.vx[AG_SUN] = v; else if (comp == 1) T.P.vy[AG_SUN] = v; else T.P.vz[AG_SUN] = v;
    } else if (tid >= 64) {
        for (int task = tid - 64; task < 3 * E.n_ast; task += 64) {
            const int comp = task % 3;
            const double sun = S.col[AG_C_SUN][comp] * E.inv_cau;
            const double xa = S.ast_h[task / 3][comp] + sun;
            T.ast[task / 3][comp] = xa;
            if (bary) CT.arel[task / 3][comp] = ag_f2_of(0.0 - xa);
        }
        int nv = (c.forces & AG_F_EIH) ? c.gr_eih_sources : 0;
        if (c.geocentric) nv = nv > AG_EAR + 1 ? nv : AG_EAR + 1;
        const int j = tid - 96;                 /* warp 3: one lane per further source */
        if (nv > 1 && j > 0 && j < nv && j < AG_NPL) {
            const double* rec = nullptr;
            double tf = 0.0;
            if (ag_planet_record(E, t, &rec, &tf) == AG_OK) ag_table_velocity(E, rec, tf, j, T);
        }
        if (c.geocentric == 1 && tid == 127) ag_table_earth_acc(E, t, T);
    }
}

/* Geocentric origin: rel = x_Earth - x_body, after pass 2 (the caller
 * synchronises the block before and after). */
__device__ __forceinline__ void ag_coop_rel_geo(const DevEphem& E, AgCoopTab& CT, int tid) {
    const PlanetState& P = CT.T.P;
    for (int q = tid; q < 3 * (AG_NPL + E.n_ast); q += 128) {
        const int k = q / 3, comp = q % 3;
        const double xo = comp == 0 ? P.x[AG_EAR] : (comp == 1 ? P.y[AG_EAR] : P.z[AG_EAR]);
        if (k < AG_NPL) CT.rel[k][comp] = xo - (comp == 0 ? P.x[k] : (comp == 1 ? P.y[k] : P.z[k]));
        else CT.arel[k - AG_NPL][comp] = ag_f2_of(xo - CT.T.ast[k - AG_NPL][comp]);
    }
}

/* Separation of the particle at x from body row k and its inverse length. */
__device__ __forceinline__ void ag_coop_sep(const AgCoopTab& CT, const double* x, int k, double& dx, double& dy,
                                            double& dz, double& ri) {
    dx = x[0] + CT.rel[k][0];
    dy = x[1] + CT.rel[k][1];
    dz = x[2] + CT.rel[k][2];
    ri = rsqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
}

/* Origin minus asteroid m in FP64 (x + this is the separation of
 * src/forces.c's direct term), from the table's positions. */
__device__ __forceinline__ void ag_coop_ast_rel(const AgCoopTab& CT, bool geo, int m, double* r) {
    const AgTable& T = CT.T;
    if (geo) {
        r[0] = T.P.x[AG_EAR] - T.ast[m][0]; r[1] = T.P.y[AG_EAR] - T.ast[m][1]; r[2] = T.P.z[AG_EAR] - T.ast[m][2];
    } else {
        r[0] = 0.0 - T.ast[m][0]; r[1] = 0.0 - T.ast[m][1]; r[2] = 0.0 - T.ast[m][2];
    }
}

/* An asteroid closer than this (AU, squared) to the particle has its term in
 * FP64: there the float-pair separation's absolute error (about 2^-48 of the
 * heliocentric distances, 1e-14 AU) would no longer be small against the
 * separation.  Beyond it the pair term's relative error (a few 1e-13) times the
 * term's share of the acceleration (below 1.3e-5 for the heaviest asteroid at
 * 0.02 AU from a main-belt particle) stays below 1e-17. */
#define AG_AST_NEAR2 4.0e-4f

/* Direct gravity of asteroids m0..m1-1 (src/forces.c, the asteroid loop of
 * the direct term).  Without the Jacobian each term is computed in
 * double-float arithmetic on the FP32 pipes (the asteroids' terms are below
 * 1e-4 of the acceleration), except for an asteroid within 0.02 AU of this
 * particle, and the terms' sum joins the FP64 acceleration at the end; with
 * the Jacobian, or with F2 off, every term is FP64 (the learned-warm-start
 * builds: beside the network's registers the float-pair chains made that
 * kernel 1.8x slower). */
template <bool JAC, bool F2 = true>
__device__ __forceinline__ void ag_coop_asteroids(const DevEphem& E, const AgCoopTab& CT, bool geo, bool on_ast,
                                                  const double* x, int m0, int m1, double& ax, double& ay, double& az,
                                                  double (*J)[6], const AgF2* xf_in = nullptr) {
    if (JAC || !F2) {
        AgSymJac Y = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, 0.0};
#pragma unroll 1
        for (int m = m0; m < m1; m++) {
            double r[3];
            ag_coop_ast_rel(CT, geo, m, r);
            const double ddx = x[0] + r[0], ddy = x[1] + r[1], ddz = x[2] + r[2];
            const double rinv = rsqrt(fma(ddx, ddx, fma(ddy, ddy, ddz * ddz)));
            const double gr3 = E.ast_gm[m] * rinv * rinv * rinv;
            if (on_ast) { ax = fma(-gr3, ddx, ax); ay = fma(-gr3, ddy, ay); az = fma(-gr3, ddz, az); }
            if (JAC) ag_symjac_term(Y, gr3, rinv, ddx, ddy, ddz);
        }
        if (JAC) ag_symjac_add(Y, J);
        return;
    }
    if (!on_ast) return;
    /* the position as float pairs: from the caller (split once by the
     * warp that predicted it) or here */
    const AgF2 xf[3] = {xf_in ? xf_in[0] : ag_f2_of(x[0]), xf_in ? xf_in[1] : ag_f2_of(x[1]),
                        xf_in ? xf_in[2] : ag_f2_of(x[2])};
    AgF2 sx = {0.0f, 0.0f}, sy = {0.0f, 0.0f}, sz = {0.0f, 0.0f};
#pragma unroll 1
    for (int m = m0; m < m1; m++) {
        const AgF2 rx = CT.arel[m][0], ry = CT.arel[m][1], rz = CT.arel[m][2];
        const float ex = xf[0].h + rx.h, ey = xf[1].h + ry.h, ez = xf[2].h + rz.h;
        if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < AG_AST_NEAR2) {
            double r[3];
            ag_coop_ast_rel(CT, geo, m, r);
            const double ddx = x[0] + r[0], ddy = x[1] + r[1], ddz = x[2] + r[2];
            const double rinv = rsqrt(fma(ddx, ddx, fma(ddy, ddy, ddz * ddz)));
            const double gr3 = E.ast_gm[m] * rinv * rinv * rinv;
            ax = fma(-gr3, ddx, ax); ay = fma(-gr3, ddy, ay); az = fma(-gr3, ddz, az);
            continue;
        }
        const AgF2 dx = ag_f2_add(xf[0], rx), dy = ag_f2_add(xf[1], ry), dz = ag_f2_add(xf[2], rz);
        const AgF2 r2 = ag_f2_add(ag_f2_mul(dx, dx), ag_f2_add(ag_f2_mul(dy, dy), ag_f2_mul(dz, dz)));
        const AgF2 ri = ag_f2_rsqrt(r2);
        const AgF2 g = ag_f2_neg(ag_f2_mul({E.ast_gm_hi[m], E.ast_gm_lo[m]}, ag_f2_mul(ri, ag_f2_mul(ri, ri))));
        sx = ag_f2_add(sx, ag_f2_mul(g, dx));
        sy = ag_f2_add(sy, ag_f2_mul(g, dy));
        sz = ag_f2_add(sz, ag_f2_mul(g, dz));
    }
    ax += ag_f2_to(sx); ay += ag_f2_to(sy); az += ag_f2_to(sz);
}

/* EIH per-source sums (Newtonian acceleration of source j by the other
 * planets, sum GM_k / r_jk), one lane per other planet, by one warp. */
__device__ __forceinline__ void ag_coop_eih_sources(const DevEphem& E, const ForceCfg& c, AgTable& T, int lane) {
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
            ax += __shfl_down_sync(AG_FULL, ax, o, 16);
            ay += __shfl_down_sync(AG_FULL, ay, o, 16);
            az += __shfl_down_sync(AG_FULL, az, o, 16);
            s1 += __shfl_down_sync(AG_FULL, s1, o, 16);
        }
        if (lane == 0) { T.eih_a[j][0] = ax; T.eih_a[j][1] = ay; T.eih_a[j][2] = az; T.eih_t1[j] = s1; }
    }
    __syncwarp();
}

/* The GR potential / simple models (off in ASSIST's default force set), out of
 * line so that their code stays out of the hot instruction stream. */
static __device__ __noinline__ void ag_coop_gr_cold(const DevEphem& E, const ForceCfg& c, const double* p, double ri,
                                                    const double* pv, double* a) {
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (c.forces & AG_F_GR_POT) ag_term_gr_pot<false>(E, p, ri, ax, ay, az, nullptr);
    if (c.forces & AG_F_GR_SIMPLE) ag_term_gr_simple<false>(E, p, ri, pv, ax, ay, az, nullptr);
    a[0] += ax; a[1] += ay; a[2] += az;
}

/* Warp w's share of the force evaluation at (x, v): partial acceleration and,
 * with JAC, partial 3x6 Jacobian; JA_out / ng_out (warp 0, optional) receive
 * the derivative of the non-gravitational term by A1..A3 and whether the term
 * applies. */
template <bool JAC, bool F2 = true>
__device__ __forceinline__ int ag_coop_force_part(int w, const AgCoopTab& CT, const DevEphem& E, const ForceCfg& c,
                                                  const double* x, const double* v, const double* A, double* acc,
                                                  double (*J)[6], double (*JA_out)[3] = nullptr,
                                                  bool* ng_out = nullptr, const AgF2* xf = nullptr) {
    const AgTable& T = CT.T;
    const TableBodies B(T);
    const PlanetState& P = T.P;
    double xo[3], vo[3], ao[3];
    ag_origin(c, P, xo, vo, ao);
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (JAC)
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 6; b++) J[a][b] = 0.0;
    const bool direct = (c.forces & (AG_F_SUN | AG_F_PLANETS | AG_F_AST)) != 0;
    int st = AG_OK;
    if (JAC && ng_out) *ng_out = false;
    if (w == 0) {
        double dx[AG_NPL], dy[AG_NPL], dz[AG_NPL], ri[AG_NPL];
#pragma unroll
        for (int k = 0; k < AG_NPL; k++) ag_coop_sep(CT, x, k, dx[k], dy[k], dz[k], ri[k]);
        if ((c.forces & AG_F_NONGRAV) && A != nullptr && (A[0] != 0.0 || A[1] != 0.0 || A[2] != 0.0)) {
            const double d[3] = {dx[AG_SUN], dy[AG_SUN], dz[AG_SUN]};
            const double dv[3] = {v[0] + (vo[0] - P.vx[AG_SUN]), v[1] + (vo[1] - P.vy[AG_SUN]), v[2] + (vo[2] - P.vz[AG_SUN])};
            double JA[3][3];
            bool has_ng;
            ag_term_nongrav<JAC>(c, d, ri[AG_SUN], dv, A, ax, ay, az, J, JA, &has_ng);
            if (JAC && JA_out) {
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) JA_out[a][b] = JA[a][b];
                *ng_out = has_ng;
            }
        }
        if (direct) {
            AgSymJac Y = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, 0.0};
#pragma unroll
            for (int q = 0; q < AG_NPL; q++) {
                const int k = ag_planet_order(q);
                const bool on = (k == AG_SUN) ? (c.forces & AG_F_SUN) : (c.forces & AG_F_PLANETS);
                ag_term_planet<JAC>(E, on, k, dx[k], dy[k], dz[k], ri[k], ax, ay, az, &Y);
            }
            if (JAC) ag_symjac_add(Y, J);
        }
        if (c.geocentric == 1) { ax -= ao[0]; ay -= ao[1]; az -= ao[2]; }
    } else if (w == 1) {
        if (c.forces & AG_F_EIH) {
            double dx[AG_NPL], dy[AG_NPL], dz[AG_NPL], ri[AG_NPL];
#pragma unroll
            for (int k = 0; k < AG_NPL; k++) ag_coop_sep(CT, x, k, dx[k], dy[k], dz[k], ri[k]);
            ag_term_eih<TableBodies, JAC>(B, E, c, P, dx, dy, dz, ri, v, vo, ao, ax, ay, az, J);
        }
        if (c.forces & (AG_F_GR_POT | AG_F_GR_SIMPLE)) {
            double p[3], ri;
            ag_coop_sep(CT, x, AG_SUN, p[0], p[1], p[2], ri);
            if (c.forces & AG_F_GR_POT) ag_term_gr_pot<JAC>(E, p, ri, ax, ay, az, J);
            if (c.forces & AG_F_GR_SIMPLE) {
                const double pv[3] = {v[0] + (vo[0] - P.vx[AG_SUN]), v[1] + (vo[1] - P.vy[AG_SUN]), v[2] + (vo[2] - P.vz[AG_SUN])};
                ag_term_gr_simple<JAC>(E, p, ri, pv, ax, ay, az, J);
            }
        }
    } else {
        const bool on_ast = (c.forces & AG_F_AST) != 0;
        const int h = (E.n_ast + 1) / 2;
        if (direct && (on_ast || JAC))
            ag_coop_asteroids<JAC, F2>(E, CT, c.geocentric == 1, on_ast, x, w == 2 ? 0 : h, w == 2 ? h : E.n_ast, ax,
                                       ay, az, J, xf);
        if (w == 2 && (c.forces & AG_F_EARTH_H)) {
            double dx, dy, dz, ri;
            ag_coop_sep(CT, x, AG_EAR, dx, dy, dz, ri);
            ag_term_earth_h<JAC>(E, c, dx, dy, dz, ri, ax, ay, az, J);
        }
        if (w == 3 && (c.forces & AG_F_SUN_H)) {
            double dx, dy, dz, ri;
            ag_coop_sep(CT, x, AG_SUN, dx, dy, dz, ri);
            ag_term_sun_h<JAC>(E, c, dx, dy, dz, ri, ax, ay, az, J);
        }
    }
    acc[0] = ax; acc[1] = ay; acc[2] = az;
    return st;
}

/* Particle-planet separations split between warps 0 and 1 (bodies 0..5 and
 * 6..10), exchanged through shared memory at named barrier 1 (64 threads:
 * both warps wait there once per evaluation). */
struct AgCoopSeps {
    double d[AG_NPL][3][32];
    double ri[AG_NPL][32];
};

/* The no-Jacobian force share of warps 0 and 1 with the separations split
 * (every lane of both warps calls it; `active` lanes compute). */
__device__ __forceinline__ void ag_coop_force_split01(int w, bool active, AgCoopSeps& SH, int lane, const AgCoopTab& CT,
                                                      const DevEphem& E, const ForceCfg& c, const double* x,
                                                      const double* v, const double* A, double* acc) {
    const AgTable& T = CT.T;
    const TableBodies B(T);
    const PlanetState& P = T.P;
    double xo[3], vo[3], ao[3];
    ag_origin(c, P, xo, vo, ao);
    double ax = 0.0, ay = 0.0, az = 0.0;
    const int k0 = w == 0 ? 0 : 6, k1 = w == 0 ? 6 : AG_NPL;
    if (active)
        for (int k = k0; k < k1; k++) {
            double dx, dy, dz, ri;
            ag_coop_sep(CT, x, k, dx, dy, dz, ri);
            SH.d[k][0][lane] = dx; SH.d[k][1][lane] = dy; SH.d[k][2][lane] = dz; SH.ri[k][lane] = ri;
        }
    __syncwarp();
    asm volatile("bar.sync 1, 64;" ::: "memory");
    if (active) {
        double dx[AG_NPL], dy[AG_NPL], dz[AG_NPL], ri[AG_NPL];
#pragma unroll
        for (int k = 0; k < AG_NPL; k++) { dx[k] = SH.d[k][0][lane]; dy[k] = SH.d[k][1][lane]; dz[k] = SH.d[k][2][lane]; ri[k] = SH.ri[k][lane]; }
        if (w == 0) {
            if ((c.forces & AG_F_NONGRAV) && A != nullptr && (A[0] != 0.0 || A[1] != 0.0 || A[2] != 0.0)) {
                const double d[3] = {dx[AG_SUN], dy[AG_SUN], dz[AG_SUN]};
                const double dv[3] = {v[0] + (vo[0] - P.vx[AG_SUN]), v[1] + (vo[1] - P.vy[AG_SUN]), v[2] + (vo[2] - P.vz[AG_SUN])};
                double JA[3][3];
                bool has_ng;
                ag_term_nongrav<false>(c, d, ri[AG_SUN], dv, A, ax, ay, az, nullptr, JA, &has_ng);
            }
            if (c.forces & (AG_F_SUN | AG_F_PLANETS | AG_F_AST)) {
#pragma unroll
                for (int q = 0; q < AG_NPL; q++) {
                    const int k = ag_planet_order(q);
                    const bool on = (k == AG_SUN) ? (c.forces & AG_F_SUN) : (c.forces & AG_F_PLANETS);
                    ag_term_planet<false>(E, on, k, dx[k], dy[k], dz[k], ri[k], ax, ay, az, nullptr);
                }
            }
            if (c.geocentric == 1) { ax -= ao[0]; ay -= ao[1]; az -= ao[2]; }
        } else {
            if (c.forces & AG_F_EIH) ag_term_eih<TableBodies, false>(B, E, c, P, dx, dy, dz, ri, v, vo, ao, ax, ay, az, nullptr);
            if (c.forces & (AG_F_GR_POT | AG_F_GR_SIMPLE)) {
                const double p[3] = {dx[AG_SUN], dy[AG_SUN], dz[AG_SUN]};
                const double pv[3] = {v[0] + (vo[0] - P.vx[AG_SUN]), v[1] + (vo[1] - P.vy[AG_SUN]), v[2] + (vo[2] - P.vz[AG_SUN])};
                double a[3] = {ax, ay, az};
                ag_coop_gr_cold(E, c, p, ri[AG_SUN], pv, a);
                ax = a[0]; ay = a[1]; az = a[2];
            }
        }
    }
    acc[0] = ax; acc[1] = ay; acc[2] = az;
}

#endif
