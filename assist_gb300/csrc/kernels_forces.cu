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
#include "table_forces.cuh"

/* All particles at one time.  Particle arrays are SoA (x[3][n]). */
__global__ void __launch_bounds__(128) ag_k_forces_table(const DevEphem* __restrict__ Ep, ForceCfg c, double t, AgForceIO io) {
    const DevEphem& E = *Ep;
    __shared__ AgTable T;
    ag_block_table(E, c, t, T);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= io.n_real) return;
    ag_table_force_particle(E, c, T, io, i);
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
