/*
 * kernels_forces.cu -- ephemeris and force kernels (K1, K2) and their launchers.
 *
 *   ag_k_bodies       : full body states (GM, x, v, a) at n times, one thread per
 *                       (time, body); the device side of assist_all_ephem /
 *                       assist_get_particle (src/forces.c:175-263).
 *   ag_k_forces_table : every particle at ONE shared time (the REBOUND callback
 *                       assist_additional_forces, src/forces.c:49-173).  Each block
 *                       evaluates the body table for that time into shared
 *                       memory (11 planet threads, one thread per asteroid, one
 *                       per EIH source), then one thread per real particle
 *                       computes its acceleration and, if it has variational
 *                       particles, their accelerations from its Jacobian.
 *   ag_k_forces_each  : every particle at its OWN time (batched API); bodies are
 *                       evaluated per thread.
 */
#include <cuda_runtime.h>
#include <cstdio>

#include "device_forces.cuh"
#include "internal.h"

/* ------------------------------------------------------------------ table */

/* Cooperative body table for time t, executed by a whole block. */
__device__ void ag_block_table(const DevEphem& E, const ForceCfg& c, double t, AgTable& T) {
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
__device__ __forceinline__ void ag_apply_jac(const double (*J)[6], const double (*JA)[3], bool has_ng, const double* dx,
                                             const double* dv, const double* dA, double* out) {
    for (int a = 0; a < 3; a++) {
        double s = J[a][0] * dx[0];
        s = fma(J[a][1], dx[1], s); s = fma(J[a][2], dx[2], s);
        s = fma(J[a][3], dv[0], s); s = fma(J[a][4], dv[1], s); s = fma(J[a][5], dv[2], s);
        if (has_ng && dA) { s = fma(JA[a][0], dA[0], s); s = fma(JA[a][1], dA[1], s); s = fma(JA[a][2], dA[2], s); }
        out[a] = s;
    }
}

/* All particles at one time.  Particle arrays are SoA (x[3][n]). */
__global__ void __launch_bounds__(128) ag_k_forces_table(const DevEphem* __restrict__ Ep, ForceCfg c, double t, AgForceIO io) {
    const DevEphem& E = *Ep;
    __shared__ AgTable T;
    ag_block_table(E, c, t, T);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= io.n_real) return;
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

/* Every particle at its own time; nv (0 or 6) variational particles per real
 * particle stored right after it: state arrays are [n][6], var [n][nv][6]. */
template <int NV>
__global__ void __launch_bounds__(128) ag_k_forces_each(const DevEphem* __restrict__ Ep, ForceCfg c, int n, const double* __restrict__ t,
                                                        const double* __restrict__ state, const double* __restrict__ params,
                                                        const double* __restrict__ var_state, double* __restrict__ acc,
                                                        double* __restrict__ var_acc, int* __restrict__ status) {
    const DevEphem& E = *Ep;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x[3] = {state[6 * (size_t)i], state[6 * (size_t)i + 1], state[6 * (size_t)i + 2]};
    const double v[3] = {state[6 * (size_t)i + 3], state[6 * (size_t)i + 4], state[6 * (size_t)i + 5]};
    double Ab[3] = {0.0, 0.0, 0.0};
    const double* A = nullptr;
    if (params) { Ab[0] = params[3 * (size_t)i]; Ab[1] = params[3 * (size_t)i + 1]; Ab[2] = params[3 * (size_t)i + 2]; A = Ab; }
    ThreadBodies B(E, t[i]);
    double a[3];
    int st;
    if (NV > 0) {
        double J[3][6], JA[3][3];
        bool has_ng;
        st = ag_forces<ThreadBodies, true>(B, E, c, x, v, A, a, J, JA, &has_ng);
#pragma unroll 1
        for (int q = 0; q < NV; q++) {
            const double* vs = var_state + ((size_t)i * NV + q) * 6;
            double out[3];
            ag_apply_jac(J, JA, has_ng, vs, vs + 3, nullptr, out);
            double* va = var_acc + ((size_t)i * NV + q) * 3;
            va[0] = out[0]; va[1] = out[1]; va[2] = out[2];
        }
    } else {
        st = ag_forces<ThreadBodies, false>(B, E, c, x, v, A, a, nullptr, nullptr, nullptr);
    }
    acc[3 * (size_t)i] = a[0]; acc[3 * (size_t)i + 1] = a[1]; acc[3 * (size_t)i + 2] = a[2];
    if (status) status[i] = st;
}

/* Full body states: out[(ti * nb + b) * 10 + ...] = GM, x, y, z, vx, vy, vz, ax, ay, az. */
__global__ void ag_k_bodies(const DevEphem* __restrict__ Ep, int n, const double* __restrict__ t, double* __restrict__ out,
                            int* __restrict__ status) {
    const DevEphem& E = *Ep;
    const int nb = AG_NPL + E.n_ast;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n * nb) return;
    const int ti = g / nb, b = g % nb;
    double* o = out + (size_t)g * 10;
    int st;
    if (b < AG_NPL) {
        st = ag_planet_full(E, b, t[ti], o);
    } else {
        const int m = b - AG_NPL;
        double h[3], sun[10];
        o[0] = E.ast_gm[m];
        st = ag_asteroid_exact(E, m, t[ti], h);
        if (st == AG_OK) st = ag_planet_full(E, AG_SUN, t[ti], sun);
        o[1] = __dadd_rn(h[0], sun[1]); o[2] = __dadd_rn(h[1], sun[2]); o[3] = __dadd_rn(h[2], sun[3]);
        for (int k = 4; k < 10; k++) o[k] = __longlong_as_double(0x7ff8000000000000LL);
    }
    if (status) atomicMax(&status[ti], st);
}

/* ------------------------------------------------------------------ launchers */

int ag_launch_forces_table(const DevEphem& E, const ForceCfg& c, double t, const AgForceIO& io, cudaStream_t s) {
    if (io.n_real <= 0) return 0;
    const int tpb = 128;
    const int blocks = (io.n_real + tpb - 1) / tpb;
    ag_k_forces_table<<<blocks, tpb, 0, s>>>(E.self_dev, c, t, io);
    return (int)cudaGetLastError();
}

int ag_launch_forces_each(const DevEphem& E, const ForceCfg& c, int n, const double* t, const double* state,
                          const double* params, int nv, const double* var_state, double* acc, double* var_acc,
                          int* status, cudaStream_t s) {
    if (n <= 0) return 0;
    const int tpb = 128;
    const int blocks = (n + tpb - 1) / tpb;
    if (nv == 6) ag_k_forces_each<6><<<blocks, tpb, 0, s>>>(E.self_dev, c, n, t, state, params, var_state, acc, var_acc, status);
    else ag_k_forces_each<0><<<blocks, tpb, 0, s>>>(E.self_dev, c, n, t, state, params, var_state, acc, var_acc, status);
    return (int)cudaGetLastError();
}

int ag_launch_bodies(const DevEphem& E, int n, const double* t, double* out, int* status, cudaStream_t s) {
    const int nb = AG_NPL + E.n_ast;
    const int total = n * nb;
    if (total <= 0) return 0;
    ag_k_bodies<<<(total + 127) / 128, 128, 0, s>>>(E.self_dev, n, t, out, status);
    return (int)cudaGetLastError();
}
