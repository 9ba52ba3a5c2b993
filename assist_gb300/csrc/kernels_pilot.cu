/*
 * kernels_pilot.cu -- expected close-encounter cost of each particle, used
 * only to order the grouped batched kernels' work queue.
 *
 * A group of particles steps at the smallest step any member needs, and a
 * member passing close to a planet needs many small steps: such a group runs
 * several times longer than its orbit class suggests.  Queued late, it is
 * still running after every other block has gone idle.  This pilot
 * estimates, per particle, the extra steps of its encounters from a
 * two-body (heliocentric Kepler) propagation sampled on a time grid against
 * the planets' ephemeris positions.  With the local dynamical rate
 * w = sqrt(GM / d^3) of the Sun (heliocentric distance) and of each planet
 * (distance to it),
 *     base  = sum over samples of w_sun,
 *     extra = sum over samples of max(0, max_k w_k - w_sun),
 * and the result is extra / base: the fraction of steps the encounters add.
 * The grouping multiplies a particle's cost estimate by (1 + extra / base).
 * Integration results do not depend on the queue order; only the time the
 * batch takes does.  The arithmetic is FP32 (a ranking, not a trajectory);
 * the orbital elements are formed in FP64.
 */
#include <cuda_runtime.h>

#include "device_ephem.cuh"
#include "internal.h"

/* Bodies sampled on the grid: the Sun (barycentric, to make the particles
 * heliocentric) and the planets except the Moon (its pull is a 1/81 share of
 * the Earth's, at the same place). */
#define AG_PILOT_NB 10
__constant__ int ag_pilot_body[AG_PILOT_NB] = {AG_SUN, AG_MER, AG_VEN, AG_EAR, AG_MAR,
                                               AG_JUP, AG_SAT, AG_URA, AG_NEP, AG_PLU};

/* grid[i * NB + b]: body b at time tmin + i * dtg; the Sun barycentric
 * (x, y, z, and vx in w; vy, vz follow in sunv), planets heliocentric. */
__global__ void ag_k_pilot_grid(const DevEphem* __restrict__ Ep, double tmin, double dtg, int G, float4* grid,
                                float2* sunv) {
    const DevEphem& E = *Ep;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G) return;
    const double t = tmin + dtg * q;
    double s[10] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, o[10];
    const bool ok = ag_planet_full(E, AG_SUN, t, s) == AG_OK;
    grid[(size_t)q * AG_PILOT_NB] = make_float4((float)s[1], (float)s[2], (float)s[3], (float)s[4]);
    sunv[q] = make_float2((float)s[5], (float)s[6]);
    for (int b = 1; b < AG_PILOT_NB; b++) {
        float4 p = make_float4(1e30f, 1e30f, 1e30f, 0.0f);       /* off the ephemeris: far away */
        if (ok && ag_planet_full(E, ag_pilot_body[b], t, o) == AG_OK)
            p = make_float4((float)(o[1] - s[1]), (float)(o[2] - s[2]), (float)(o[3] - s[3]), 0.0f);
        grid[(size_t)q * AG_PILOT_NB + b] = p;
    }
}

__global__ void ag_k_pilot(const DevEphem* __restrict__ Ep, int n, const double* __restrict__ t0,
                           const double* __restrict__ te, const double* __restrict__ state, const float4* __restrict__ grid,
                           const float2* __restrict__ sunv, int G, double tmin, double dtg, float* ratio) {
    const DevEphem& E = *Ep;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ratio[i] = 0.0f;
    if (G < 2) return;
    const double ta = t0[i], tb = te[i];
    /* the Sun at t0, linear between grid points */
    double f = (ta - tmin) / dtg;
    int g0 = (int)floor(f);
    g0 = g0 < 0 ? 0 : (g0 > G - 2 ? G - 2 : g0);
    f -= g0;
    const float4 sa = grid[(size_t)g0 * AG_PILOT_NB], sb = grid[(size_t)(g0 + 1) * AG_PILOT_NB];
    const float2 va = sunv[g0], vb = sunv[g0 + 1];
    const double sx = sa.x + f * (sb.x - sa.x), sy = sa.y + f * (sb.y - sa.y), sz = sa.z + f * (sb.z - sa.z);
    const double svx = sa.w + f * (sb.w - sa.w), svy = va.x + f * (vb.x - va.x), svz = va.y + f * (vb.y - va.y);
    const double* s0 = state + 6 * (size_t)i;
    const double r[3] = {s0[0] - sx, s0[1] - sy, s0[2] - sz};
    const double v[3] = {s0[3] - svx, s0[4] - svy, s0[5] - svz};
    const double mu = E.gm[AG_SUN];
    /* elliptic elements; other orbits keep the plain estimate */
    const double rn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    const double inv_a = 2.0 / rn - v2 / mu;
    if (!(inv_a > 0.0) || !(rn > 0.0)) return;
    const double a = 1.0 / inv_a;
    double ev[3];
    for (int k = 0; k < 3; k++) ev[k] = ((v2 - mu / rn) * r[k] - rv * v[k]) / mu;
    const double e = sqrt(ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2]);
    if (!(e < 0.98)) return;
    const double h[3] = {r[1] * v[2] - r[2] * v[1], r[2] * v[0] - r[0] * v[2], r[0] * v[1] - r[1] * v[0]};
    const double hn = sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
    if (!(hn > 0.0)) return;
    /* perifocal frame: P toward pericentre (toward r for a circular orbit), Q = h x P / |h| */
    double P[3];
    if (e > 1e-8) { for (int k = 0; k < 3; k++) P[k] = ev[k] / e; }
    else { for (int k = 0; k < 3; k++) P[k] = r[k] / rn; }
    const double Q[3] = {(h[1] * P[2] - h[2] * P[1]) / hn, (h[2] * P[0] - h[0] * P[2]) / hn,
                         (h[0] * P[1] - h[1] * P[0]) / hn};
    /* eccentric and mean anomaly at t0 (from the perifocal coordinates of r) */
    const double xp = r[0] * P[0] + r[1] * P[1] + r[2] * P[2], yp = r[0] * Q[0] + r[1] * Q[1] + r[2] * Q[2];
    const double be = sqrt(1.0 - e * e);
    const double E0 = atan2(yp / (a * be), xp / a + e);
    const double M0 = E0 - e * sin(E0);
    const double nmot = sqrt(mu * inv_a) * inv_a;
    /* grid samples inside the integration interval */
    const double lo = fmin(ta, tb), hi = fmax(ta, tb);
    int i0 = (int)ceil((lo - tmin) / dtg), i1 = (int)floor((hi - tmin) / dtg);
    i0 = i0 < 0 ? 0 : i0;
    i1 = i1 > G - 1 ? G - 1 : i1;
    if (i1 < i0) return;
    const float fa = (float)a, fe = (float)e, fb = (float)(a * be);
    const float Pf[3] = {(float)P[0], (float)P[1], (float)P[2]}, Qf[3] = {(float)Q[0], (float)Q[1], (float)Q[2]};
    const float musun = (float)mu;
    float gmk[AG_PILOT_NB];
    for (int b = 1; b < AG_PILOT_NB; b++) gmk[b] = (float)E.gm[ag_pilot_body[b]];
    float base = 0.0f, extra = 0.0f;
    /* mean anomaly at the first sample in FP64, then FP32 increments (the
     * loop stays off the FP64 pipe) */
    const double twopi = 6.283185307179586;
    double Ms = M0 + nmot * ((tmin + dtg * i0) - ta);
    Ms -= twopi * floor(Ms / twopi);
    const float Mstart = (float)Ms, dM = (float)(nmot * dtg), tpf = 6.2831853f, itpf = 1.0f / 6.2831853f;
    for (int q = i0; q <= i1; q++) {
        float Mf = fmaf((float)(q - i0), dM, Mstart);
        Mf -= tpf * floorf(Mf * itpf);
        float Ea = Mf + fe * __sinf(Mf);
        for (int it = 0; it < 6; it++) {
            float sE, cE;
            __sincosf(Ea, &sE, &cE);
            Ea -= (Ea - fe * sE - Mf) / (1.0f - fe * cE);
        }
        float sE, cE;
        __sincosf(Ea, &sE, &cE);
        const float xo = fa * (cE - fe), yo = fb * sE;
        const float px = xo * Pf[0] + yo * Qf[0], py = xo * Pf[1] + yo * Qf[1], pz = xo * Pf[2] + yo * Qf[2];
        const float r2 = px * px + py * py + pz * pz;
        const float wsun = sqrtf(musun / (r2 * sqrtf(r2)));
        float wmax = 0.0f;
        const float4* gq = grid + (size_t)q * AG_PILOT_NB;
#pragma unroll
        for (int b = 1; b < AG_PILOT_NB; b++) {
            const float4 pb = gq[b];
            const float dx = px - pb.x, dy = py - pb.y, dz = pz - pb.z;
            const float d2 = fmaxf(dx * dx + dy * dy + dz * dz, 1e-16f);
            wmax = fmaxf(wmax, sqrtf(gmk[b] / (d2 * sqrtf(d2))));
        }
        base += wsun;
        extra += fmaxf(0.0f, wmax - wsun);
    }
    if (base > 0.0f && isfinite(extra)) ratio[i] = extra / base;
}

int ag_pilot_encounters(const DevEphem& E, int n, const double* d_t0, const double* d_te, const double* d_state,
                        double tmin, double tmax, float* d_ratio, float4* d_grid, float2* d_sunv, int G,
                        cudaStream_t s) {
    if (n <= 0) return 0;
    const double dtg = G > 1 ? (tmax - tmin) / (G - 1) : 1.0;
    if (!(dtg > 0.0)) return (int)cudaMemsetAsync(d_ratio, 0, sizeof(float) * (size_t)n, s);
    ag_k_pilot_grid<<<(G + 127) / 128, 128, 0, s>>>(E.self_dev, tmin, dtg, G, d_grid, d_sunv);
    ag_k_pilot<<<(n + 127) / 128, 128, 0, s>>>(E.self_dev, n, d_t0, d_te, d_state, d_grid, d_sunv, G, tmin, dtg,
                                               d_ratio);
    return (int)cudaGetLastError();
}
