/*
 * table_forces.cuh -- the force evaluation of every particle at ONE shared
 * time (the REBOUND callback assist_additional_forces, src/forces.c:49-173),
 * as block-level device functions: the block builds the body table of that
 * time in shared memory, then each thread evaluates particles.  Used by the
 * one-launch force kernel (kernels_forces.cu); the shared-step IAS15 kernel
 * (kernels_shared.cu) uses its Jacobian application for variational
 * particles.
 */
#ifndef ASSIST_GB300_TABLE_FORCES_CUH
#define ASSIST_GB300_TABLE_FORCES_CUH

#include "device_forces.cuh"
#include "internal.h"

/* ------------------------------------------------------------------ table */

/* Cooperative body table for time t, executed by a whole block. */
static __device__ void ag_block_table(const DevEphem& E, const ForceCfg& c, double t, AgTable& T) {
    const int tid = threadIdx.x;
    __shared__ int s_st;
    __shared__ const double* s_rec;
    __shared__ double s_tf;
    if (tid == 0) {
        const double* rec = nullptr;
        double tf = 0.0;
        s_st = E.pl_spk ? AG_OK : ag_planet_record(E, t, &rec, &tf);
        s_rec = rec;
        s_tf = tf;
    }
    __syncthreads();
    int nv = (c.forces & AG_F_EIH) ? c.gr_eih_sources : 0;
    if (c.geocentric) nv = nv > AG_EAR + 1 ? nv : AG_EAR + 1;
    if (E.pl_spk) {
        /* planets from an SPK file: one thread per body, full state */
        if (tid < AG_NPL) {
            double o[10];
            const int st = ag_spk_planet(E, tid, t, o);
            if (st != AG_OK) atomicMax(&s_st, st);
            T.P.x[tid] = o[1]; T.P.y[tid] = o[2]; T.P.z[tid] = o[3];
            T.P.vx[tid] = o[4]; T.P.vy[tid] = o[5]; T.P.vz[tid] = o[6];
            if (tid == AG_EAR && c.geocentric == 1) { T.P.ex_a[0] = o[7]; T.P.ex_a[1] = o[8]; T.P.ex_a[2] = o[9]; }
        }
        __syncthreads();
    } else if (s_st == AG_OK && tid < AG_NPL) {
        const int b = tid;
        double u[3], v[3] = {0.0, 0.0, 0.0};
        if ((b == AG_SUN) || (b < nv)) ag_planet_exact<true>(E, s_rec, s_tf, b, u, v);
        else ag_planet_exact<false>(E, s_rec, s_tf, b, u, v);
        T.P.x[b] = u[0]; T.P.y[b] = u[1]; T.P.z[b] = u[2];
        T.P.vx[b] = v[0]; T.P.vy[b] = v[1]; T.P.vz[b] = v[2];
        if (b == AG_EAR && c.geocentric == 1) {
            double e_[10];
            ag_planet_full(E, AG_EAR, t, e_);
            T.P.ex_a[0] = e_[7]; T.P.ex_a[1] = e_[8]; T.P.ex_a[2] = e_[9];
        }
    }
    if (tid == 0) T.status = s_st;
    __syncthreads();
    if (s_st == AG_OK) {
        if (tid >= 32 && tid - 32 < E.n_ast) {
            const int m = tid - 32;
            double h[3];
            int st = ag_asteroid_exact(E, m, t, h);
            T.ast[m][0] = __dadd_rn(h[0], T.P.x[AG_SUN]); T.ast[m][1] = __dadd_rn(h[1], T.P.y[AG_SUN]);
            T.ast[m][2] = __dadd_rn(h[2], T.P.z[AG_SUN]);
            if (st != AG_OK && (c.forces & (AG_F_SUN | AG_F_PLANETS | AG_F_AST))) atomicMax(&T.status, st);
        }
        if ((c.forces & AG_F_EIH) && tid < c.gr_eih_sources && tid < AG_NPL) {
            double aj[3], t1;
            ag_eih_source(E, T.P, tid, aj, &t1);
            T.eih_a[tid][0] = aj[0]; T.eih_a[tid][1] = aj[1]; T.eih_a[tid][2] = aj[2]; T.eih_t1[tid] = t1;
        }
    }
    __syncthreads();
}

/* Apply a real particle's Jacobian to one variational particle. */
static __device__ __forceinline__ void ag_apply_jac(const double (*J)[6], const double (*JA)[3], bool has_ng, const double* dx,
                                             const double* dv, const double* dA, double* out) {
    for (int a = 0; a < 3; a++) {
        double s = J[a][0] * dx[0];
        s = fma(J[a][1], dx[1], s); s = fma(J[a][2], dx[2], s);
        s = fma(J[a][3], dv[0], s); s = fma(J[a][4], dv[1], s); s = fma(J[a][5], dv[2], s);
        if (has_ng && dA) { s = fma(JA[a][0], dA[0], s); s = fma(JA[a][1], dA[1], s); s = fma(JA[a][2], dA[2], s); }
        out[a] = s;
    }
}

/* The acceleration of real particle i (and of its variational particles,
 * from its Jacobian) at the table's time; io's arrays are SoA (x[3][stride]). */
static __device__ __forceinline__ void ag_table_force_particle(const DevEphem& E, const ForceCfg& c, const AgTable& T,
                                                             const AgForceIO& io, int i) {
    if (T.status != AG_OK) {
        if (i == 0 && io.status) *io.status = T.status;
        return;
    }
    const double x[3] = {io.x[i], io.x[io.stride + i], io.x[2 * io.stride + i]};
    const double v[3] = {io.v[i], io.v[io.stride + i], io.v[2 * io.stride + i]};
    const double* A = nullptr;
    double Ab[3];
    if (io.params) { Ab[0] = io.params[3 * i]; Ab[1] = io.params[3 * i + 1]; Ab[2] = io.params[3 * i + 2]; A = Ab; }
    double acc[3];
    TableBodies B(T);
    const int v0 = io.var_start ? io.var_start[i] : 0, v1 = io.var_start ? io.var_start[i + 1] : 0;
    int st;
    if (v1 > v0) {
        double J[3][6], JA[3][3];
        bool has_ng;
        st = ag_forces<TableBodies, true>(B, E, c, x, v, A, acc, J, JA, &has_ng);
        for (int q = v0; q < v1; q++) {
            const int p = io.var_index[q];        /* particle slot of the variational particle */
            const int cfg = io.var_cfg ? io.var_cfg[q] : -1;
            const double dx[3] = {io.x[p], io.x[io.stride + p], io.x[2 * io.stride + p]};
            const double dv[3] = {io.v[p], io.v[io.stride + p], io.v[2 * io.stride + p]};
            double dA[3] = {0.0, 0.0, 0.0};
            if (io.params && cfg >= 0) {
                const size_t r = 3 * (size_t)(io.n_real + cfg);
                dA[0] = io.params[r]; dA[1] = io.params[r + 1]; dA[2] = io.params[r + 2];
            }
            double out[3];
            ag_apply_jac(J, JA, has_ng, dx, dv, dA, out);
            io.a[p] = out[0]; io.a[io.stride + p] = out[1]; io.a[2 * io.stride + p] = out[2];
        }
    } else {
        st = ag_forces<TableBodies, false>(B, E, c, x, v, A, acc, nullptr, nullptr, nullptr);
    }
    io.a[i] = acc[0]; io.a[io.stride + i] = acc[1]; io.a[2 * io.stride + i] = acc[2];
    if (st != AG_OK && io.status) atomicMax(io.status, st);
}

#endif
