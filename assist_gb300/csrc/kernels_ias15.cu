/*
 * kernels_ias15.cu -- K4: batched, persistent IAS15 with a device work queue.
 *
 * Every thread owns one slot.  It takes particle indices from an atomic queue
 * (ordered longest integration first by the host), integrates that particle
 * (and its NV first-order variational particles) from t0 to t_end with its own
 * adaptive IAS15 step, writes the end state back and takes the next index.
 * The loop body is ONE force evaluation: a per-slot state machine decides
 * where that evaluation is (the step's start, node n of predictor-corrector
 * iteration k) and what to do with the result, so the expensive part (the
 * ephemeris + force model, ~2k FP64 instructions) runs converged across the
 * warp while the cheap bookkeeping diverges.
 *
 * IAS15 (Rein & Spiegel 2015, MNRAS 446, 1424), as ASSIST runs it through
 * REBOUND with adaptive_mode = 1 (src/assist.c:446):
 *   - Gauss-Radau nodes h_1..h_7, acceleration a(h) = a0 + sum_k b_k h^(k+1);
 *   - predictor-corrector iterations until the change of b_6 relative to the
 *     largest acceleration drops below 1e-16, stops decreasing (after 2
 *     iterations), or 12 iterations ran;
 *   - step-size control dt_new = dt (epsilon / (max|b_6| / max|a|))^(1/7),
 *     rejection when dt_new < dt/4, growth capped at 4x, optional min_dt;
 *   - the next step's b predicted from this step's by the polynomial shift
 *     with the step-size ratio (skipped above ratio 20);
 *   - compensated summation of position, velocity and time.
 * Variational particles are integrated with the same coefficients and never
 * enter the error measures.
 *
 * Per-component state lives in a slot-major workspace in HBM/L2
 * ([field][component][slot], coalesced); per-slot scalars live in registers.
 * A clock64 watchdog bounds the kernel's run time: a slot whose budget is
 * spent writes its particle back with ASSIST_GB300_TIMEOUT-like status and exits.
 */
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>

#include <type_traits>

#include "device_forces.cuh"
#include "ias15_common.cuh"
#include "internal.h"
#include "warp_table.cuh"
#include "mlp.cuh"

size_t ag_batch_ws_doubles(int nslots, int nv) { return (size_t)W_NF * 3 * (1 + nv) * (size_t)nslots; }

template <int NV>
__global__ void __launch_bounds__(128) ag_k_batch(const DevEphem* __restrict__ Ep, ForceCfg cf, AgBatchArgs A) {
    const DevEphem& E = *Ep;
    constexpr int C = 3 * (1 + NV);
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= A.nslots) return;
    const Ws<C> W{A.ws, A.nslots, slot};
    const long long clk0 = clock64();
    unsigned long long n_acc = 0, n_rej = 0, n_ev = 0, n_it = 0;

    int pid = -1;
    double t = 0, tc = 0, dt = 0, dtls = 0, tend = 0, hstep = 0, pc_err = 0, pc_last = 0;
    double prm[3] = {0.0, 0.0, 0.0};
    bool has_prm = false;
    int phase = 0, iters = 0, sub = 0, last = 0, pstat = 0;
    long long steps = 0;
    bool stop = false;

    while (true) {
        if (pid < 0) {
            const int qpos = atomicAdd(A.queue, 1);
            if (qpos >= A.n) break;
            pid = A.order[qpos];
            if (stop) {
                /* run-time budget spent: the particles still queued are not
                 * integrated (state untouched) and say so */
                if (A.status) A.status[pid] = AG_ST_TIMEOUT;
                pid = -1;
                continue;
            }
            const double* s0 = A.state + 6 * (size_t)pid;
            for (int k = 0; k < 3; k++) {
                W(W_X0, k) = s0[k]; W(W_V0, k) = s0[3 + k]; W(W_XC, k) = 0.0; W(W_VC, k) = 0.0;
            }
            for (int q = 0; q < NV; q++) {
                const double* vs = A.var_state + ((size_t)pid * NV + q) * 6;
                for (int k = 0; k < 3; k++) {
                    W(W_X0, 3 + 3 * q + k) = vs[k]; W(W_V0, 3 + 3 * q + k) = vs[3 + k];
                    W(W_XC, 3 + 3 * q + k) = 0.0; W(W_VC, 3 + 3 * q + k) = 0.0;
                }
            }
            for (int comp = 0; comp < C; comp++)
                for (int k = 0; k < 7; k++) {
                    W(W_B + k, comp) = 0.0; W(W_E + k, comp) = 0.0; W(W_BR + k, comp) = 0.0; W(W_ER + k, comp) = 0.0;
                }
            has_prm = false;
            if (A.params) {
                prm[0] = A.params[3 * (size_t)pid]; prm[1] = A.params[3 * (size_t)pid + 1]; prm[2] = A.params[3 * (size_t)pid + 2];
                has_prm = true;
            }
            t = A.t0[pid]; tend = A.t_end[pid]; tc = 0.0; dtls = 0.0;
            dt = (tend >= t ? 1.0 : -1.0) * fabs(A.dt0);
            steps = 0; pstat = AG_ST_OK; phase = 0;
            if (t == tend) phase = 3;     /* nothing to integrate */
            if (phase == 0) {
                const double rem = (tend - t) - tc;
                if (fabs(dt) >= fabs(rem)) { hstep = rem; last = 1; } else { hstep = dt; last = 0; }
            }
        }
        if (phase != 3 && A.watchdog_cycles > 0 && clock64() - clk0 > A.watchdog_cycles) {
            pstat = AG_ST_TIMEOUT;
            phase = 3;
            stop = true;
        }
        if (phase != 3) {
            /* ---- evaluation point: the step start (node 0) or node `sub` */
            const double hn = phase == 0 ? 0.0 : ag_ias.h[sub];
            const double tn = phase == 0 ? t : t + (tc + hstep * hn);
            double sx[9], sv[8];
            if (phase == 1) {
                sx[0] = hstep * hn;
                sx[1] = sx[0] * sx[0] * 0.5;
#pragma unroll
                for (int k = 2; k < 9; k++) sx[k] = sx[k - 1] * ag_ias.fx[sub][k];
                sv[0] = hstep * hn;
#pragma unroll
                for (int k = 1; k < 8; k++) sv[k] = sv[k - 1] * ag_ias.fv[sub][k];
            }
            double xp[3], vp[3];
            for (int k = 0; k < 3; k++) {
                if (phase == 0) { xp[k] = W(W_X0, k); vp[k] = W(W_V0, k); }
                else {
                    double px = sx[8] * W(W_B + 6, k);
#pragma unroll
                    for (int j = 5; j >= 0; j--) px = fma(sx[j + 2], W(W_B + j, k), px);
                    px = fma(sx[1], W(W_A0, k), px);
                    px = fma(sx[0], W(W_V0, k), px);
                    xp[k] = W(W_X0, k) + (px + W(W_XC, k));
                    double pv = sv[7] * W(W_B + 6, k);
#pragma unroll
                    for (int j = 5; j >= 0; j--) pv = fma(sv[j + 1], W(W_B + j, k), pv);
                    pv = fma(sv[0], W(W_A0, k), pv);
                    vp[k] = W(W_V0, k) + (pv + W(W_VC, k));
                }
            }
            /* ---- ephemeris + force model at (tn, xp, vp) */
            ThreadBodies B(E, tn);
            double at[C];
            int st;
            if (NV > 0) {
                double J[3][6], JA[3][3];
                bool has_ng;
                st = ag_forces<ThreadBodies, true>(B, E, cf, xp, vp, has_prm ? prm : nullptr, at, J, JA, &has_ng);
#pragma unroll 1
                for (int q = 0; q < NV; q++) {
                    double dxq[3], dvq[3];
                    for (int k = 0; k < 3; k++) {
                        const int comp = 3 + 3 * q + k;
                        if (phase == 0) { dxq[k] = W(W_X0, comp); dvq[k] = W(W_V0, comp); }
                        else {
                            double px = sx[8] * W(W_B + 6, comp);
                            for (int j = 5; j >= 0; j--) px = fma(sx[j + 2], W(W_B + j, comp), px);
                            px = fma(sx[1], W(W_A0, comp), px);
                            px = fma(sx[0], W(W_V0, comp), px);
                            dxq[k] = W(W_X0, comp) + (px + W(W_XC, comp));
                            double pv = sv[7] * W(W_B + 6, comp);
                            for (int j = 5; j >= 0; j--) pv = fma(sv[j + 1], W(W_B + j, comp), pv);
                            pv = fma(sv[0], W(W_A0, comp), pv);
                            dvq[k] = W(W_V0, comp) + (pv + W(W_VC, comp));
                        }
                    }
                    for (int a = 0; a < 3; a++) {
                        double s = J[a][0] * dxq[0];
                        s = fma(J[a][1], dxq[1], s); s = fma(J[a][2], dxq[2], s);
                        s = fma(J[a][3], dvq[0], s); s = fma(J[a][4], dvq[1], s); s = fma(J[a][5], dvq[2], s);
                        at[3 + 3 * q + a] = s;
                    }
                }
            } else {
                st = ag_forces<ThreadBodies, false>(B, E, cf, xp, vp, has_prm ? prm : nullptr, at, nullptr, nullptr, nullptr);
            }
            n_ev++;
            if (st != AG_OK) {
                pstat = AG_ST_COVERAGE;
                phase = 3;
            } else if (phase == 0) {
                /* ---- step start: a0 and g from the predicted b */
                for (int comp = 0; comp < C; comp++) {
                    W(W_A0, comp) = at[comp];
                    double b[7];
#pragma unroll
                    for (int k = 0; k < 7; k++) b[k] = W(W_B + k, comp);
#pragma unroll
                    for (int j = 0; j < 7; j++) {
                        double s = b[j];
#pragma unroll
                        for (int k = j + 1; k < 7; k++) s = fma(b[k], ag_ias.d[j][k], s);
                        W(W_G + j, comp) = s;
                    }
                }
                phase = 1; iters = 1; sub = 1; pc_last = 1e300; pc_err = 0.0;
            } else {
                /* ---- node `sub`: divided difference g_(n-1), then b */
                const int n = sub;
                double maxa = 0.0, maxdb = 0.0;
                for (int comp = 0; comp < C; comp++) {
                    double gn = (at[comp] - W(W_A0, comp)) * ag_ias.rrinv[n][0];
                    for (int j = 1; j < n; j++) gn = (gn - W(W_G + j - 1, comp)) * ag_ias.rrinv[n][j];
                    const double delta = gn - W(W_G + n - 1, comp);
                    W(W_G + n - 1, comp) = gn;
                    for (int k = 0; k < n - 1; k++) W(W_B + k, comp) = fma(delta, ag_ias.c[n - 1][k], W(W_B + k, comp));
                    W(W_B + n - 1, comp) += delta;
                    if (n == 7 && comp < 3) {
                        const double aa = fabs(at[comp]);
                        if (ag_isnormal_pos(aa) && aa > maxa) maxa = aa;
                        const double db = fabs(delta);
                        if (ag_isnormal_pos(db) && db > maxdb) maxdb = db;
                    }
                }
                if (n < 7) {
                    sub = n + 1;
                } else {
                    pc_err = maxdb / maxa;
                    const bool conv = (pc_err < 1e-16) || (iters > 2 && pc_last <= pc_err) || (iters >= 12);
                    if (!conv) {
                        pc_last = pc_err; iters++; sub = 1;
                    } else {
                        n_it += (unsigned long long)iters;
                        /* ---- step-size control */
                        double dt_new = hstep;
                        bool reject = false;
                        if (A.epsilon > 0.0) {
                            double ma = 0.0, mb = 0.0;
                            for (int k = 0; k < 3; k++) {
                                const double aa = fabs(at[k]);
                                if (ag_isnormal_pos(aa) && aa > ma) ma = aa;
                                const double bb = fabs(W(W_B + 6, k));
                                if (ag_isnormal_pos(bb) && bb > mb) mb = bb;
                            }
                            const double err = mb / ma;
                            const double safety = 0.25;
                            if (ag_isnormal_pos(err)) dt_new = pow(A.epsilon / err, 1.0 / 7.0) * hstep;
                            else dt_new = hstep / safety;
                            if (fabs(dt_new) < A.min_dt) dt_new = copysign(A.min_dt, dt_new);
                            const double ratio = dt_new / hstep;
                            if (fabs(ratio) < safety) reject = true;
                            else if (fabs(ratio) > 1.0 / safety) dt_new = hstep / safety;
                        }
                        if (!last && A.dt_floor > 0.0 && fabs(dt_new) < A.dt_floor) {
                            /* step underflow: the particle is hitting a body (not
                             * tested on a step cut short to land on t_end, whose
                             * proposal scales with the short step) */
                            pstat = AG_ST_UNDERFLOW;
                            phase = 3;
                        } else if (reject) {
                            n_rej++;
                            if (dtls != 0.0) ag_predict_next<C>(W, dt_new / dtls);
                            else
                                for (int comp = 0; comp < C; comp++)
                                    for (int k = 0; k < 7; k++) { W(W_B + k, comp) = 0.0; W(W_E + k, comp) = 0.0; }
                            dt = dt_new;
                        } else {
                            n_acc++;
                            /* ---- accept: advance x0, v0, t with compensated sums */
                            const double h2 = hstep * hstep;
                            for (int comp = 0; comp < C; comp++) {
                                double b[7];
#pragma unroll
                                for (int k = 0; k < 7; k++) b[k] = W(W_B + k, comp);
                                const double a0 = W(W_A0, comp);
                                double ix = b[6] / 72. + b[5] / 56. + b[4] / 42. + b[3] / 30. + b[2] / 20. + b[1] / 12. + b[0] / 6. + a0 / 2.;
                                ix = fma(ix, h2, W(W_V0, comp) * hstep);
                                double y = ix + W(W_XC, comp);
                                double x0 = W(W_X0, comp);
                                double s = x0 + y;
                                W(W_XC, comp) = y - (s - x0);
                                W(W_X0, comp) = s;
                                double iv = b[6] / 8. + b[5] / 7. + b[4] / 6. + b[3] / 5. + b[2] / 4. + b[1] / 3. + b[0] / 2. + a0;
                                iv = iv * hstep;
                                y = iv + W(W_VC, comp);
                                const double v0 = W(W_V0, comp);
                                s = v0 + y;
                                W(W_VC, comp) = y - (s - v0);
                                W(W_V0, comp) = s;
#pragma unroll
                                for (int k = 0; k < 7; k++) { W(W_ER + k, comp) = W(W_E + k, comp); W(W_BR + k, comp) = b[k]; }
                            }
                            {
                                const double y = hstep + tc;
                                const double s = t + y;
                                tc = y - (s - t);
                                t = s;
                            }
                            dtls = hstep;
                            ag_predict_next<C>(W, dt_new / hstep);
                            dt = dt_new;
                            steps++;
                            if (last) { t = tend; tc = 0.0; phase = 3; }
                            else if (A.max_steps > 0 && steps >= A.max_steps) { pstat = AG_ST_BUDGET; phase = 3; }
                        }
                        if (phase != 3) {
                            phase = 0;
                            const double rem = (tend - t) - tc;
                            if (fabs(dt) >= fabs(rem)) { hstep = rem; last = 1; } else { hstep = dt; last = 0; }
                        }
                    }
                }
            }
        }
        if (phase == 3) {
            /* ---- particle finished: write back and free the slot */
            double* s0 = A.state + 6 * (size_t)pid;
            bool finite = true;
            for (int k = 0; k < 3; k++) {
                s0[k] = W(W_X0, k) + W(W_XC, k);
                s0[3 + k] = W(W_V0, k) + W(W_VC, k);
                finite = finite && isfinite(s0[k]) && isfinite(s0[3 + k]);
            }
            for (int q = 0; q < NV; q++) {
                double* vs = A.var_state + ((size_t)pid * NV + q) * 6;
                for (int k = 0; k < 3; k++) {
                    vs[k] = W(W_X0, 3 + 3 * q + k) + W(W_XC, 3 + 3 * q + k);
                    vs[3 + k] = W(W_V0, 3 + 3 * q + k) + W(W_VC, 3 + 3 * q + k);
                }
            }
            if (pstat == AG_ST_OK && !finite) pstat = AG_ST_NONFINITE;
            if (A.status) A.status[pid] = pstat;
            pid = -1;
        }
    }
    atomicAdd(&A.counters[0], n_acc);
    atomicAdd(&A.counters[1], n_rej);
    atomicAdd(&A.counters[2], n_ev);
    atomicAdd(&A.counters[3], n_it);
    atomicAdd(&A.counters[6], n_ev);     /* every evaluation evaluates its own bodies */
}

/* The IAS15 tables of this unit's kernels on the current device, ahead of a
 * stream capture. */
int ag_batch_ready(void) { return ag_ias_tables_init(); }

int ag_batch_max_slots(int nv, int tpb) {
    int dev = 0, sms = 0, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (nv == 6) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ag_k_batch<6>, tpb, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ag_k_batch<0>, tpb, 0);
    if (bps < 1) bps = 1;
    return sms * bps * tpb;
}

int ag_launch_batch(const DevEphem& E, const ForceCfg& c, const AgBatchArgs& a, int nv, int tpb, cudaStream_t s) {
    int e = ag_ias_tables_init();
    if (e) return e;
    if (tpb > 128) tpb = 128;
    const int blocks = (a.nslots + tpb - 1) / tpb;
    if (nv == 6) ag_k_batch<6><<<blocks, tpb, 0, s>>>(E.self_dev, c, a);
    else ag_k_batch<0><<<blocks, tpb, 0, s>>>(E.self_dev, c, a);
    return (int)cudaGetLastError();
}

/* FP64 FMA throughput of this device (GFLOP/s), measured with independent FMA
 * chains; the roofline denominator of the FP64-bound kernels. */
__global__ void ag_k_dfma_probe(double* out, int iters, double a, double b) {
    double acc[8];
#pragma unroll
    for (int c = 0; c < 8; c++) acc[c] = (double)(threadIdx.x + c) * 1e-3;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < 8; c++) acc[c] = fma(acc[c], a, b);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) s += acc[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

double ag_fp64_probe_gflops(void) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256, blocks = sms * 8, iters = 4096;
    double* d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * threads * blocks) != cudaSuccess) return 0.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    ag_k_dfma_probe<<<blocks, threads>>>(d, 64, 1.0000001, 1e-9);
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(e0);
        ag_k_dfma_probe<<<blocks, threads>>>(d, iters, 1.0000001, 1e-9);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    cudaFree(d);
    return 2.0 * 8 * (double)iters * threads * blocks / (best * 1e-3) / 1e9;
}

/* Copy of the device IAS15 tables (diagnostics: compared with the generated
 * header by the tests). out: 306 doubles in IasTables order. */
extern "C" int ag_debug_ias_tables(double* out) {
    int e = ag_ias_tables_init();
    if (e) return e;
    return (int)cudaMemcpyFromSymbol(out, ag_ias, sizeof(IasTables));
}

/* =========================================================================
 * K4g: warp-synchronous groups.
 *
 * A warp integrates a group of up to 32 particles that start at the same t0
 * (the host groups particles by start time, direction, orbital timescale
 * q^1.5 and integration length).  The group shares t and the adaptive step:
 * each lane runs IAS15's own error control for its particle and the group
 * takes the most restrictive step (dt = min over lanes, rejection when any
 * lane rejects); predictor-corrector iterations continue until every lane has
 * converged (a converged lane keeps its b).  Sharing the time lets the warp
 * evaluate every body ONCE per node, one lane per planet / asteroid, with the
 * reference's exact arithmetic, into a per-warp table in shared memory that
 * all 32 lanes read; per-lane FP64 work is then the force model alone.  A
 * lane whose particle reaches its own t_end writes it back and idles until
 * the group is done; the warp then takes the next group from the queue
 * (groups ordered longest first).
 * ========================================================================= */


template <int NV>
__global__ void __launch_bounds__(128) ag_k_group(const DevEphem* __restrict__ Ep, ForceCfg cf, AgBatchArgs A) {
    constexpr int C = 3 * (1 + NV);
    const DevEphem& E = *Ep;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    __shared__ AgTable tabs[4];
    __shared__ AgWarpScratch scr[4];
    AgTable& Tab = tabs[wib];
    AgWarpScratch& Scr = scr[wib];
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    const Ws<C> W{A.ws, A.nslots, slot};
    const long long clk0 = clock64();
    unsigned long long n_acc = 0, n_rej = 0, n_ev = 0, n_it = 0, n_tab = 0;
    bool stop = false;     /* warp-uniform */

    while (true) {
        int g = 0;
        if (lane == 0) g = atomicAdd(A.queue, 1);
        g = __shfl_sync(AG_FULL, g, 0);
        if (g >= A.n_groups) break;
        const int gs = A.grp_size[g], g0 = A.grp_start[g];
        if (stop) {
            /* run-time budget spent: groups still queued are not integrated */
            if (lane < gs && A.status) A.status[A.order[g0 + lane]] = AG_ST_TIMEOUT;
            continue;
        }
        const int pid = lane < gs ? A.order[g0 + lane] : -1;
        double t = A.t0[A.order[g0]], tc = 0.0, dtls = 0.0;
        const double tend = pid >= 0 ? A.t_end[pid] : t;
        double dir = 0.0;
        {
            double d = pid >= 0 ? (tend - t) : 0.0;
            const unsigned fwd = __ballot_sync(AG_FULL, d > 0.0), bwd = __ballot_sync(AG_FULL, d < 0.0);
            dir = fwd ? 1.0 : (bwd ? -1.0 : 1.0);
        }
        double dt = dir * fabs(A.dt0);
        double prm[3] = {0.0, 0.0, 0.0};
        bool has_prm = false;
        int pstat = AG_ST_OK;
        bool live = pid >= 0;
        if (live) {
            const double* s0 = A.state + 6 * (size_t)pid;
            for (int k = 0; k < 3; k++) { W(W_X0, k) = s0[k]; W(W_V0, k) = s0[3 + k]; W(W_XC, k) = 0.0; W(W_VC, k) = 0.0; }
            for (int q = 0; q < NV; q++) {
                const double* vs = A.var_state + ((size_t)pid * NV + q) * 6;
                for (int k = 0; k < 3; k++) {
                    W(W_X0, 3 + 3 * q + k) = vs[k]; W(W_V0, 3 + 3 * q + k) = vs[3 + k];
                    W(W_XC, 3 + 3 * q + k) = 0.0; W(W_VC, 3 + 3 * q + k) = 0.0;
                }
            }
            for (int comp = 0; comp < C; comp++)
                for (int k = 0; k < 7; k++) {
                    W(W_B + k, comp) = 0.0; W(W_E + k, comp) = 0.0; W(W_BR + k, comp) = 0.0; W(W_ER + k, comp) = 0.0;
                }
            if (A.params) {
                prm[0] = A.params[3 * (size_t)pid]; prm[1] = A.params[3 * (size_t)pid + 1]; prm[2] = A.params[3 * (size_t)pid + 2];
                has_prm = true;
            }
        }
        bool finish_now = live && (tend == t);
        long long steps = 0;
        while (true) {
            /* ---- retire lanes whose particle is complete */
            if (finish_now) {
                double* s0 = A.state + 6 * (size_t)pid;
                bool finite = true;
                for (int k = 0; k < 3; k++) {
                    s0[k] = W(W_X0, k) + W(W_XC, k);
                    s0[3 + k] = W(W_V0, k) + W(W_VC, k);
                    finite = finite && isfinite(s0[k]) && isfinite(s0[3 + k]);
                }
                for (int q = 0; q < NV; q++) {
                    double* vs = A.var_state + ((size_t)pid * NV + q) * 6;
                    for (int k = 0; k < 3; k++) {
                        vs[k] = W(W_X0, 3 + 3 * q + k) + W(W_XC, 3 + 3 * q + k);
                        vs[3 + k] = W(W_V0, 3 + 3 * q + k) + W(W_VC, 3 + 3 * q + k);
                    }
                }
                if (pstat == AG_ST_OK && !finite) pstat = AG_ST_NONFINITE;
                if (A.status) A.status[pid] = pstat;
                live = false;
                finish_now = false;
            }
            if (!__any_sync(AG_FULL, live)) break;
            if (__any_sync(AG_FULL, A.watchdog_cycles > 0 && clock64() - clk0 > A.watchdog_cycles)) {
                pstat = AG_ST_TIMEOUT;
                finish_now = live;
                stop = true;
                continue;
            }
            /* ---- step size: no further than the nearest unfinished end */
            const double rem = live ? fabs((tend - t) - tc) : 1e300;
            const double rem_min = warp_min(rem);
            double hstep;
            bool last_group = false;
            if (fabs(dt) >= rem_min) { hstep = dir * rem_min; last_group = true; }
            else hstep = dt;
            const bool last = live && last_group && rem == rem_min;
            /* ---- node 0: accelerations at the step start, g from the predicted b */
            int st = ag_warp_table_fast(E, cf, t, Tab, Scr, lane);
            n_tab++;
            if (st != AG_OK) { pstat = AG_ST_COVERAGE; finish_now = live; continue; }
            if (live) {
                double at[C];
                double xp[3] = {W(W_X0, 0), W(W_X0, 1), W(W_X0, 2)}, vp[3] = {W(W_V0, 0), W(W_V0, 1), W(W_V0, 2)};
                TableBodies B(Tab);
                if (NV > 0) {
                    double J[3][6], JA[3][3];
                    bool has_ng;
                    st = ag_forces<TableBodies, true>(B, E, cf, xp, vp, has_prm ? prm : nullptr, at, J, JA, &has_ng);
                    for (int q = 0; q < NV; q++)
                        for (int a = 0; a < 3; a++) {
                            double s = 0.0;
                            for (int b = 0; b < 3; b++) {
                                s = fma(J[a][b], W(W_X0, 3 + 3 * q + b), s);
                                s = fma(J[a][3 + b], W(W_V0, 3 + 3 * q + b), s);
                            }
                            at[3 + 3 * q + a] = s;
                        }
                } else {
                    st = ag_forces<TableBodies, false>(B, E, cf, xp, vp, has_prm ? prm : nullptr, at, nullptr, nullptr, nullptr);
                }
                n_ev++;
                for (int comp = 0; comp < C; comp++) {
                    W(W_A0, comp) = at[comp];
                    double b[7];
#pragma unroll
                    for (int k = 0; k < 7; k++) b[k] = W(W_B + k, comp);
#pragma unroll
                    for (int j = 0; j < 7; j++) {
                        double s = b[j];
#pragma unroll
                        for (int k = j + 1; k < 7; k++) s = fma(b[k], ag_ias.d[j][k], s);
                        W(W_G + j, comp) = s;
                    }
                }
            }
            /* ---- predictor-corrector iterations */
            int iters = 1;
            double pc_last = 1e300, ma7 = 0.0;
            bool conv = !live;
            while (true) {
                for (int n = 1; n < 8; n++) {
                    const double hn = ag_ias.h[n];
                    const double tn = t + (tc + hstep * hn);
                    st = ag_warp_table_fast(E, cf, tn, Tab, Scr, lane);
                    n_tab++;
                    if (st != AG_OK) break;
                    if (!conv) {
                        double sx[9], sv[8];
                        sx[0] = hstep * hn;
                        sx[1] = sx[0] * sx[0] * 0.5;
#pragma unroll
                        for (int k = 2; k < 9; k++) sx[k] = sx[k - 1] * ag_ias.fx[n][k];
                        sv[0] = hstep * hn;
#pragma unroll
                        for (int k = 1; k < 8; k++) sv[k] = sv[k - 1] * ag_ias.fv[n][k];
                        double xp[C], vp[C];
                        for (int comp = 0; comp < C; comp++) {
                            double px = sx[8] * W(W_B + 6, comp);
#pragma unroll
                            for (int j = 5; j >= 0; j--) px = fma(sx[j + 2], W(W_B + j, comp), px);
                            px = fma(sx[1], W(W_A0, comp), px);
                            px = fma(sx[0], W(W_V0, comp), px);
                            xp[comp] = W(W_X0, comp) + (px + W(W_XC, comp));
                            double pv = sv[7] * W(W_B + 6, comp);
#pragma unroll
                            for (int j = 5; j >= 0; j--) pv = fma(sv[j + 1], W(W_B + j, comp), pv);
                            pv = fma(sv[0], W(W_A0, comp), pv);
                            vp[comp] = W(W_V0, comp) + (pv + W(W_VC, comp));
                        }
                        double at[C];
                        TableBodies B(Tab);
                        if (NV > 0) {
                            double J[3][6], JA[3][3];
                            bool has_ng;
                            ag_forces<TableBodies, true>(B, E, cf, xp, vp, has_prm ? prm : nullptr, at, J, JA, &has_ng);
                            for (int q = 0; q < NV; q++)
                                for (int a = 0; a < 3; a++) {
                                    double s = 0.0;
                                    for (int b = 0; b < 3; b++) {
                                        s = fma(J[a][b], xp[3 + 3 * q + b], s);
                                        s = fma(J[a][3 + b], vp[3 + 3 * q + b], s);
                                    }
                                    at[3 + 3 * q + a] = s;
                                }
                        } else {
                            ag_forces<TableBodies, false>(B, E, cf, xp, vp, has_prm ? prm : nullptr, at, nullptr, nullptr, nullptr);
                        }
                        n_ev++;
                        double maxa = 0.0, maxdb = 0.0;
                        for (int comp = 0; comp < C; comp++) {
                            double gn = (at[comp] - W(W_A0, comp)) * ag_ias.rrinv[n][0];
                            for (int j = 1; j < n; j++) gn = (gn - W(W_G + j - 1, comp)) * ag_ias.rrinv[n][j];
                            const double delta = gn - W(W_G + n - 1, comp);
                            W(W_G + n - 1, comp) = gn;
                            for (int k = 0; k < n - 1; k++) W(W_B + k, comp) = fma(delta, ag_ias.c[n - 1][k], W(W_B + k, comp));
                            W(W_B + n - 1, comp) += delta;
                            if (n == 7 && comp < 3) {
                                const double aa = fabs(at[comp]);
                                if (ag_isnormal_pos(aa) && aa > maxa) maxa = aa;
                                const double db = fabs(delta);
                                if (ag_isnormal_pos(db) && db > maxdb) maxdb = db;
                            }
                        }
                        if (n == 7) {
                            ma7 = maxa;
                            const double pc_err = maxdb / maxa;
                            conv = (pc_err < 1e-16) || (iters > 2 && pc_last <= pc_err) || (iters >= 12);
                            if (conv) n_it += (unsigned long long)iters;
                            else pc_last = pc_err;
                        }
                    }
                }
                if (st != AG_OK) break;
                if (__all_sync(AG_FULL, conv)) break;
                iters++;
            }
            if (st != AG_OK) { pstat = AG_ST_COVERAGE; finish_now = live; continue; }
            /* ---- step-size control: each lane's choice, the group takes the smallest */
            double dt_new_l = 1e300, dt_nocap_l = 1e300;
            bool rej_l = false;
            if (A.epsilon > 0.0 && live) {
                double mb = 0.0;
                for (int k = 0; k < 3; k++) {
                    const double bb = fabs(W(W_B + 6, k));
                    if (ag_isnormal_pos(bb) && bb > mb) mb = bb;
                }
                const double err = mb / ma7;
                const double safety = 0.25;
                double dn;
                if (ag_isnormal_pos(err)) dn = pow(A.epsilon / err, 1.0 / 7.0) * hstep;
                else dn = hstep / safety;
                if (fabs(dn) < A.min_dt) dn = copysign(A.min_dt, dn);
                dt_nocap_l = fabs(dn);
                const double ratio = dn / hstep;
                if (fabs(ratio) < safety) rej_l = true;
                else if (fabs(ratio) > 1.0 / safety) dn = hstep / safety;
                dt_new_l = fabs(dn);
            }
            if (live && !last_group && A.epsilon > 0.0 && A.dt_floor > 0.0 && dt_nocap_l < A.dt_floor) {
                /* step underflow: this lane's particle is hitting a body; it stops
                 * (state of the step start) and the group goes on without it.  Not
                 * tested on a step cut short to land on a member's t_end: the
                 * proposals scale with that short step */
                pstat = AG_ST_UNDERFLOW;
                finish_now = true;
                rej_l = false;
                dt_new_l = 1e300;
                dt_nocap_l = 1e300;
            }
            if (__any_sync(AG_FULL, finish_now && pstat == AG_ST_UNDERFLOW)) {
                if (!__any_sync(AG_FULL, live && !finish_now)) continue;   /* only underflowing lanes left */
            }
            double dt_new;
            if (A.epsilon > 0.0) {
                dt_new = dir * warp_min(dt_new_l);
                /* a step shortened to land on a lane's t_end does not shrink the
                 * group's step beyond what the error control asks for */
                if (last_group) dt_new = dir * fmin(fabs(dt), fmax(fabs(dt_new), warp_min(dt_nocap_l)));
            } else {
                dt_new = dt;            /* fixed step */
            }
            const bool reject = __any_sync(AG_FULL, rej_l);
            if (reject) {
                n_rej += live ? 1 : 0;
                if (live) {
                    if (dtls != 0.0) ag_predict_next<C>(W, dt_new / dtls);
                    else
                        for (int comp = 0; comp < C; comp++)
                            for (int k = 0; k < 7; k++) { W(W_B + k, comp) = 0.0; W(W_E + k, comp) = 0.0; }
                }
                dt = dt_new;
                continue;
            }
            /* ---- accept */
            if (live) {
                n_acc++;
                const double h2 = hstep * hstep;
                for (int comp = 0; comp < C; comp++) {
                    double b[7];
#pragma unroll
                    for (int k = 0; k < 7; k++) b[k] = W(W_B + k, comp);
                    const double a0 = W(W_A0, comp);
                    double ix = b[6] / 72. + b[5] / 56. + b[4] / 42. + b[3] / 30. + b[2] / 20. + b[1] / 12. + b[0] / 6. + a0 / 2.;
                    ix = fma(ix, h2, W(W_V0, comp) * hstep);
                    double y = ix + W(W_XC, comp);
                    const double x0 = W(W_X0, comp);
                    double s = x0 + y;
                    W(W_XC, comp) = y - (s - x0);
                    W(W_X0, comp) = s;
                    double iv = b[6] / 8. + b[5] / 7. + b[4] / 6. + b[3] / 5. + b[2] / 4. + b[1] / 3. + b[0] / 2. + a0;
                    iv = iv * hstep;
                    y = iv + W(W_VC, comp);
                    const double v0 = W(W_V0, comp);
                    s = v0 + y;
                    W(W_VC, comp) = y - (s - v0);
                    W(W_V0, comp) = s;
#pragma unroll
                    for (int k = 0; k < 7; k++) { W(W_ER + k, comp) = W(W_E + k, comp); W(W_BR + k, comp) = b[k]; }
                }
                ag_predict_next<C>(W, dt_new / hstep);
            }
            {
                const double y = hstep + tc;
                const double s = t + y;
                tc = y - (s - t);
                t = s;
            }
            dtls = hstep;
            dt = dt_new;
            steps++;
            if (last) finish_now = true;
            if (last_group && live && !last && fabs((tend - t) - tc) == 0.0) finish_now = true;
            if (A.max_steps > 0 && steps >= A.max_steps && live && !finish_now) { pstat = AG_ST_BUDGET; finish_now = true; }
        }
    }
    atomicAdd(&A.counters[0], n_acc);
    atomicAdd(&A.counters[1], n_rej);
    atomicAdd(&A.counters[2], n_ev);
    atomicAdd(&A.counters[3], n_it);
    if (lane == 0) atomicAdd(&A.counters[6], n_tab);   /* body tables, one per warp and node time */
}

int ag_group_max_slots(int nv) {
    int dev = 0, sms = 0, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (nv == 6) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ag_k_group<6>, 128, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ag_k_group<0>, 128, 0);
    if (bps < 1) bps = 1;
    return sms * bps * 128;
}

int ag_launch_group(const DevEphem& E, const ForceCfg& c, const AgBatchArgs& a, int nv, cudaStream_t s) {
    int e = ag_ias_tables_init();
    if (e) return e;
    const int blocks = (a.nslots + 127) / 128;
    if (nv == 6) ag_k_group<6><<<blocks, 128, 0, s>>>(E.self_dev, c, a);
    else ag_k_group<0><<<blocks, 128, 0, s>>>(E.self_dev, c, a);
    return (int)cudaGetLastError();
}

