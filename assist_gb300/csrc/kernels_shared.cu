/*
 * kernels_shared.cu -- K3: IAS15 for ONE simulation whose particles share the
 * step (REBOUND's reb_simulation_integrate with ASSIST attached: the drop-in
 * path of the CPU reference, src/assist.c:440-446 selects IAS15 with
 * adaptive_mode = 1).
 *
 * All per-particle state stays on the device between steps.  A step is
 * a start evaluation (node 0) and predictor-corrector iterations of 7 node
 * evaluations; each node is predict -> forces -> update, all inside one
 * kernel (sh_k_step) whose 128-thread blocks each own 32 real particles and
 * their variational particles and build the step's eight body tables once.
 * The update of node 7 also reduces max|delta b6|, max|a| and max|b6| over
 * the real particles (the global error measures of adaptive_mode = 1).  A
 * launch is the whole predictor-corrector loop of the step when the
 * simulation has one block (up to 32 real particles) or when all its blocks
 * fit on the device at once (a cooperative launch whose blocks meet at a
 * bounded grid barrier after each iteration); otherwise a launch is one
 * iteration and the host reads the three maxima back to decide convergence.
 * The host then decides acceptance and the next step size, with the same
 * rules as the batched kernel (kernels_ias15.cu).
 */
#include <cuda_runtime.h>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "device_forces.cuh"
#include "ias15_constants.h"
#include "internal.h"
#include "shared_sim.h"
#include "table_forces.cuh"
#include "coop_forces.cuh"

__constant__ double sh_h[8];
__constant__ double sh_rrinv[8][8];
__constant__ double sh_c[7][7];
__constant__ double sh_d[7][7];
__constant__ double sh_fx[8][9];
__constant__ double sh_fv[8][8];
static bool sh_ready[64];

static int sh_tables_init(void) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && sh_ready[dev]) return 0;
    const double h[8] = IAS15_H_INIT;
    const double rr[28] = IAS15_RR_INIT;
    const double cc[21] = IAS15_C_INIT;
    const double dd[21] = IAS15_D_INIT;
    double rrinv[8][8] = {{0}}, c[7][7] = {{0}}, d[7][7] = {{0}}, fx[8][9] = {{0}}, fv[8][8] = {{0}};
    int q = 0;
    for (int n = 1; n < 8; n++) for (int j = 0; j < n; j++) rrinv[n][j] = 1.0 / rr[q++];
    q = 0;
    for (int j = 1; j < 7; j++) for (int k = 0; k < j; k++) c[j][k] = cc[q++];
    q = 0;
    for (int j = 0; j < 6; j++) for (int k = j + 1; k < 7; k++) d[j][k] = dd[q++];
    for (int j = 0; j < 7; j++) { c[j][j] = 1.0; d[j][j] = 1.0; }
    for (int n = 0; n < 8; n++) {
        for (int k = 2; k < 9; k++) fx[n][k] = h[n] * (double)(k - 1) / (double)(k + 1);
        for (int k = 1; k < 8; k++) fv[n][k] = h[n] * (double)k / (double)(k + 1);
    }
    if (cudaMemcpyToSymbol(sh_h, h, sizeof(h)) != cudaSuccess) return 1;
    cudaMemcpyToSymbol(sh_rrinv, rrinv, sizeof(rrinv));
    cudaMemcpyToSymbol(sh_c, c, sizeof(c));
    cudaMemcpyToSymbol(sh_d, d, sizeof(d));
    cudaMemcpyToSymbol(sh_fx, fx, sizeof(fx));
    cudaMemcpyToSymbol(sh_fv, fv, sizeof(fv));
    if (dev >= 0 && dev < 64) sh_ready[dev] = true;
    return (int)cudaGetLastError();
}

/* field layout: f*(3*stride) + k*stride + i */
enum { S_X0 = 0, S_V0, S_A0, S_XC, S_VC, S_AT, S_XP, S_VP, S_B, S_G = S_B + 7, S_E = S_G + 7, S_BR = S_E + 7, S_ER = S_BR + 7,
       S_PX = S_ER + 7, S_PV, S_PA, S_NF };

struct ShView {
    double* w;
    int stride;
    __device__ __forceinline__ double& operator()(int f, int k, int i) const { return w[((size_t)f * 3 + k) * stride + i]; }
};

/* The predictor's coefficients of node `node` (1..7) of a step of size
 * hstep: sx[q] for x, sv[q] for v. */
__device__ __forceinline__ void sh_predict_coeffs(int node, double hstep, double* sx, double* sv) {
    const double hn = sh_h[node];
    sx[0] = hstep * hn;
    sx[1] = sx[0] * sx[0] * 0.5;
#pragma unroll
    for (int q = 2; q < 9; q++) sx[q] = sx[q - 1] * sh_fx[node][q];
    sv[0] = hstep * hn;
#pragma unroll
    for (int q = 1; q < 8; q++) sv[q] = sv[q - 1] * sh_fv[node][q];
}

/* Predictor of component k of particle i at node `node` with that node's
 * coefficients sx, sv (node 0: the start state). */
__device__ __forceinline__ void sh_predict(const ShView& W, int i, int k, int node, const double* sx, const double* sv) {
    if (node == 0) {
        W(S_XP, k, i) = W(S_X0, k, i);
        W(S_VP, k, i) = W(S_V0, k, i);
        return;
    }
    double px = sx[8] * W(S_B + 6, k, i);
#pragma unroll
    for (int j = 5; j >= 0; j--) px = fma(sx[j + 2], W(S_B + j, k, i), px);
    px = fma(sx[1], W(S_A0, k, i), px);
    px = fma(sx[0], W(S_V0, k, i), px);
    W(S_XP, k, i) = W(S_X0, k, i) + (px + W(S_XC, k, i));
    double pv = sv[7] * W(S_B + 6, k, i);
#pragma unroll
    for (int j = 5; j >= 0; j--) pv = fma(sv[j + 1], W(S_B + j, k, i), pv);
    pv = fma(sv[0], W(S_A0, k, i), pv);
    W(S_VP, k, i) = W(S_V0, k, i) + (pv + W(S_VC, k, i));
}

/* Start of a step for component k: a0 from the node-0 force, g from the
 * predicted b. */
__device__ __forceinline__ void sh_start(const ShView& W, int i, int k) {
    W(S_A0, k, i) = W(S_AT, k, i);
    double b[7];
#pragma unroll
    for (int q = 0; q < 7; q++) b[q] = W(S_B + q, k, i);
#pragma unroll
    for (int j = 0; j < 7; j++) {
        double s = b[j];
#pragma unroll
        for (int q = j + 1; q < 7; q++) s = fma(b[q], sh_d[j][q], s);
        W(S_G + j, k, i) = s;
    }
}

/* Corrector of component k of particle i at node `node`: g and b from the
 * node's force.  At node 7 the real particles' |delta b6|, |a| and |b6| enter
 * the running maxima (normal values only, as REBOUND's isnormal tests). */
__device__ __forceinline__ void sh_update(const ShView& W, int i, int k, int n_real, int node, double& mdb, double& ma,
                                          double& mb) {
    const double at = W(S_AT, k, i);
    double gn = (at - W(S_A0, k, i)) * sh_rrinv[node][0];
    for (int j = 1; j < node; j++) gn = (gn - W(S_G + j - 1, k, i)) * sh_rrinv[node][j];
    const double delta = gn - W(S_G + node - 1, k, i);
    W(S_G + node - 1, k, i) = gn;
    for (int q = 0; q < node - 1; q++) W(S_B + q, k, i) = fma(delta, sh_c[node - 1][q], W(S_B + q, k, i));
    W(S_B + node - 1, k, i) += delta;
    if (node == 7 && i < n_real) {
        const double aa = fabs(at), db = fabs(delta), bb = fabs(W(S_B + 6, k, i));
        if (ag_isnormal_pos(aa) && aa > ma) ma = aa;
        if (ag_isnormal_pos(db) && db > mdb) mdb = db;
        if (ag_isnormal_pos(bb) && bb > mb) mb = bb;
    }
}

/* ------------------------------------------------------------------ step kernel
 *
 * One launch does the predictor-corrector work of a step for a block of 32
 * real particles (lane l of every warp: real particle 32 b + l) and their
 * variational particles, with the block-cooperative force evaluation of the
 * batched kernel: the four warps split each particle's force terms (their
 * partial sums added ((w3 + w2) + w1) + w0), and the eight node tables of the
 * step are built once, at its start, by the whole block (the node times do
 * not change while the corrector iterates).  A variational particle's
 * acceleration is its real particle's Jacobian (summed from the warps'
 * partial Jacobians) applied to its state.  The IAS15 state stays in global
 * memory; its predictor and corrector run as one task per particle component
 * over the block's threads.  Block b predicts and corrects the particles of
 * plist[pstart[b] .. pstart[b+1]): its real particles, their variational
 * particles and (last block) any particle no real particle lists, so that a
 * node needs no grid-wide barrier.  The maxima over the real particles
 * (max|delta b6|, max|a|, max|b6|; bit patterns of non-negative doubles
 * order like unsigned integers) go to red[0..2].
 *
 * Several blocks: in one cooperative launch when every block fits on the
 * device at once (each block builds the tables; after each iteration the
 * blocks' maxima meet in global memory across a bounded grid barrier and
 * every block takes the same convergence decision), else one iteration per
 * launch with the host deciding convergence, the first launch of a step
 * (`first`: node 0 and the tables) leaving the tables in gtab for the
 * launches after it.  One block (up to 32 real
 * particles): every iteration of the step in one launch, with the host's
 * convergence rule (relative corrector change below 1e-16, no longer
 * decreasing after two iterations, or 12 iterations) and the iteration count
 * in red[3].  A node time outside the ephemeris sets ASSIST's coverage status
 * and ends the launch. */
struct ShStepArgs {
    ShView W;
    AgForceIO io;            /* x, v, a: the predicted states and accelerations */
    const int* vowner;       /* real particle of each variational entry of io */
    const int* plist;
    const int* pstart;
    unsigned long long* red; /* [0..3] the step's maxima and iterations; [4..12] three rotating
                                reduction buffers of a cooperative launch */
    AgCoopTab* gtab;         /* the step's eight node tables (several blocks, one launch per iteration) */
    unsigned* bar;           /* grid barrier of a cooperative launch: arrivals, generation, gave up */
    int coop;                /* several blocks in one cooperative launch run the whole step */
    double tn[8];            /* node times: t + (tc + hstep h_n), from the host */
    double hstep;
    int first;
};

struct ShStepSmem {
    AgCoopTab tab[8];
    AgCoopScratch scr;
    AgCoopSeps seps;
    double pa[4][3][32];     /* partial accelerations of the four warps */
    double pj[4][18][32];    /* partial Jacobians; pj[0] holds their sum */
    double pja[9][32];       /* d acc / dA of the non-gravitational term (warp 0) */
    double pcx[8][9], pcv[8][8];   /* predictor coefficients of nodes 1..7 */
    int png[32];
    unsigned long long red[3];
    int more;
    int bar_ok;
};

/* Barrier of all blocks of a cooperative launch (the runtime makes every
 * block resident or refuses the launch).  Thread 0 of each block reads the
 * generation, then counts its arrival; the last arrival resets the count and
 * advances the generation, the others poll it.  A block that has polled
 * SH_BAR_POLLS times stops waiting, records that in bar[2] and returns
 * false; its block then leaves the kernel, and the other blocks stop at
 * their own limits, so the launch always ends. */
#define SH_BAR_POLLS (1 << 21)
__device__ __forceinline__ bool sh_grid_sync(unsigned* bar, int* ok_smem) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(&bar[0], 1u) == gridDim.x - 1) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicAdd(&bar[1], 1u);
        } else {
            int polls = 0;
            while (*vgen == gen) {
                if (++polls > SH_BAR_POLLS) { ok = 0; atomicExch(&bar[2], 1u); break; }
                __nanosleep(64);
            }
            __threadfence();
        }
        *ok_smem = ok;
    }
    __syncthreads();
    return *ok_smem != 0;
}

/* Accelerations of the block's particles at node n (table S.tab[n]) into
 * io.a; ends with a block barrier. */
__device__ __forceinline__ void sh_step_forces(ShStepSmem& S, const AgForceIO& io, const int* vowner, const DevEphem& E,
                                               const ForceCfg& c, int n, bool jac, int v0, int v1) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, r0 = 32 * blockIdx.x;
    const int ir = r0 + lane;
    const bool live = ir < io.n_real;
    const AgCoopTab& T = S.tab[n];
    double xp[3] = {0.0, 0.0, 0.0}, vp[3] = {0.0, 0.0, 0.0}, prm[3] = {0.0, 0.0, 0.0};
    const double* Ap = nullptr;
    if (live) {
        for (int k = 0; k < 3; k++) { xp[k] = io.x[k * io.stride + ir]; vp[k] = io.v[k * io.stride + ir]; }
        if (io.params) { prm[0] = io.params[3 * ir]; prm[1] = io.params[3 * ir + 1]; prm[2] = io.params[3 * ir + 2]; Ap = prm; }
    }
    double acc[3] = {0.0, 0.0, 0.0};
    if (jac) {
        if (live) {
            double J[3][6], JA[3][3];
            bool ng = false;
            if (wid == 0) ag_coop_force_part<true>(0, T, E, c, xp, vp, Ap, acc, J, JA, &ng);
            else ag_coop_force_part<true>(wid, T, E, c, xp, vp, Ap, acc, J);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 6; b++) S.pj[wid][6 * a + b][lane] = J[a][b];
            if (wid == 0) {
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) S.pja[3 * a + b][lane] = JA[a][b];
                S.png[lane] = ng;
            }
        }
    } else if (wid < 2) {
        ag_coop_force_split01(wid, live, S.seps, lane, T, E, c, xp, vp, Ap, acc);
    } else if (live) {
        ag_coop_force_part<false>(wid, T, E, c, xp, vp, Ap, acc, nullptr);
    }
    if (live) { S.pa[wid][0][lane] = acc[0]; S.pa[wid][1][lane] = acc[1]; S.pa[wid][2][lane] = acc[2]; }
    __syncthreads();
    if (tid < 96 && r0 + lane < io.n_real) {
        const int k = wid;                       /* component k on warp k */
        io.a[k * io.stride + ir] = ((S.pa[3][k][lane] + S.pa[2][k][lane]) + S.pa[1][k][lane]) + S.pa[0][k][lane];
        if (jac)
            for (int b = 0; b < 6; b++) {
                const int e = 6 * k + b;
                S.pj[0][e][lane] = ((S.pj[3][e][lane] + S.pj[2][e][lane]) + S.pj[1][e][lane]) + S.pj[0][e][lane];
            }
    }
    if (jac) {
        __syncthreads();
        for (int q = v0 + tid; q < v1; q += blockDim.x) {
            const int p = io.var_index[q], l = vowner[q] - r0;
            const int cfg = io.var_cfg ? io.var_cfg[q] : -1;
            double J[3][6], JA[3][3];
            for (int a = 0; a < 3; a++) {
                for (int b = 0; b < 6; b++) J[a][b] = S.pj[0][6 * a + b][l];
                for (int b = 0; b < 3; b++) JA[a][b] = S.pja[3 * a + b][l];
            }
            const double dx[3] = {io.x[p], io.x[io.stride + p], io.x[2 * io.stride + p]};
            const double dv[3] = {io.v[p], io.v[io.stride + p], io.v[2 * io.stride + p]};
            double dA[3] = {0.0, 0.0, 0.0};
            if (io.params && cfg >= 0) {
                const size_t r = 3 * (size_t)(io.n_real + cfg);
                dA[0] = io.params[r]; dA[1] = io.params[r + 1]; dA[2] = io.params[r + 2];
            }
            double out[3];
            ag_apply_jac(J, JA, S.png[l] != 0, dx, dv, dA, out);
            io.a[p] = out[0]; io.a[io.stride + p] = out[1]; io.a[2 * io.stride + p] = out[2];
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(128) sh_k_step(const DevEphem* __restrict__ Ep, ForceCfg c, ShStepArgs A) {
    extern __shared__ __align__(16) unsigned char sh_smem[];
    ShStepSmem& S = *reinterpret_cast<ShStepSmem*>(sh_smem);
    const DevEphem& E = *Ep;
    const ShView& W = A.W;
    const AgForceIO& io = A.io;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nt = blockDim.x;
    const int q0 = 3 * A.pstart[blockIdx.x], q1 = 3 * A.pstart[blockIdx.x + 1];   /* (particle, component) tasks */
    const int n_real = io.n_real, r0 = 32 * blockIdx.x, r1 = min(r0 + 32, n_real);
    const int v0 = (io.var_start && r0 < r1) ? io.var_start[r0] : 0;
    const int v1 = (io.var_start && r0 < r1) ? io.var_start[r1] : 0;
    const bool jac = v1 > v0;                    /* block-uniform */
    const bool single = gridDim.x == 1;
    const bool whole = single || A.coop;         /* the launch runs the step's whole corrector loop */
    /* the predictor's coefficients of the step's nodes, once per launch */
    if (tid >= 1 && tid < 8) sh_predict_coeffs(tid, A.hstep, S.pcx[tid], S.pcv[tid]);
    __syncthreads();
    if (A.first) {
        /* the step's eight node tables */
        int bad = 0;
        for (int n = 0; n < 8; n++) {
            AgStageCursor cur;
            int stage_fail = 0;
            bad |= ag_coop_table_pass1<false>(E, c, A.tn[n], S.scr, S.tab[n], tid, nullptr, cur, &stage_fail);
            __syncthreads();
            ag_coop_table_pass2(E, c, A.tn[n], S.tab[n], S.scr, tid);
            __syncthreads();
            if (c.geocentric == 1) { ag_coop_rel_geo(E, S.tab[n], tid); __syncthreads(); }
        }
        if (c.forces & AG_F_EIH)
            for (int n = wid; n < 8; n += 4) ag_coop_eih_sources(E, c, S.tab[n].T, lane);
        bad = __syncthreads_or(bad);
        if (bad) {
            /* every block builds the same tables: all of them leave here */
            if (tid == 0) {
                if (n_real > 0) atomicMax(io.status, (int)AG_ERR_COVERAGE);
                if (whole && blockIdx.x == 0) { A.red[0] = A.red[1] = A.red[2] = 0ull; A.red[3] = 1ull; }
            }
            return;
        }
        if (!whole && blockIdx.x == 0) {
            const double* src = reinterpret_cast<const double*>(S.tab);
            double* dst = reinterpret_cast<double*>(A.gtab);
            for (int q = tid; q < (int)(sizeof(S.tab) / sizeof(double)); q += nt) dst[q] = src[q];
        }
        /* node 0: the start of the step */
        for (int q = q0 + tid; q < q1; q += nt) sh_predict(W, A.plist[q / 3], q % 3, 0, nullptr, nullptr);
        __syncthreads();
        sh_step_forces(S, io, A.vowner, E, c, 0, jac, v0, v1);
        for (int q = q0 + tid; q < q1; q += nt) sh_start(W, A.plist[q / 3], q % 3);
    } else {
        const double* src = reinterpret_cast<const double*>(A.gtab);
        double* dst = reinterpret_cast<double*>(S.tab);
        for (int q = tid; q < (int)(sizeof(S.tab) / sizeof(double)); q += nt) dst[q] = src[q];
    }
    double pc_last = 1e300;
    int iters = 1;
    while (true) {
        if (tid < 3) S.red[tid] = 0ull;
        double mdb = 0.0, ma = 0.0, mb = 0.0;
        for (int node = 1; node < 8; node++) {
            for (int q = q0 + tid; q < q1; q += nt) sh_predict(W, A.plist[q / 3], q % 3, node, S.pcx[node], S.pcv[node]);
            __syncthreads();
            sh_step_forces(S, io, A.vowner, E, c, node, jac, v0, v1);
            for (int q = q0 + tid; q < q1; q += nt) sh_update(W, A.plist[q / 3], q % 3, n_real, node, mdb, ma, mb);
        }
        for (int o = 16; o > 0; o >>= 1) {
            mdb = fmax(mdb, __shfl_xor_sync(0xffffffffu, mdb, o));
            ma = fmax(ma, __shfl_xor_sync(0xffffffffu, ma, o));
            mb = fmax(mb, __shfl_xor_sync(0xffffffffu, mb, o));
        }
        if (lane == 0) {
            atomicMax(&S.red[0], (unsigned long long)__double_as_longlong(mdb));
            atomicMax(&S.red[1], (unsigned long long)__double_as_longlong(ma));
            atomicMax(&S.red[2], (unsigned long long)__double_as_longlong(mb));
        }
        __syncthreads();
        if (!whole) {
            if (tid < 3) atomicMax(&A.red[tid], S.red[tid]);
            return;
        }
        if (A.coop) {
            /* the maxima over all blocks: buffer iters % 3 collects this
             * iteration's, block 0 clears the next one (last read two
             * barriers ago), every block reads the result after the barrier */
            unsigned long long* rb = A.red + 4 + 3 * (iters % 3);
            if (tid < 3) atomicMax(&rb[tid], S.red[tid]);
            if (blockIdx.x == 0 && tid < 3) A.red[4 + 3 * ((iters + 1) % 3) + tid] = 0ull;
            if (!sh_grid_sync(A.bar, &S.bar_ok)) return;
            if (tid < 3) S.red[tid] = atomicOr(&rb[tid], 0ull);
            __syncthreads();
        }
        if (tid == 0) {
            const double pc_err = __longlong_as_double((long long)S.red[0]) / __longlong_as_double((long long)S.red[1]);
            const bool conv = (pc_err < 1e-16) || (iters > 2 && pc_last <= pc_err) || (iters >= 12);
            S.more = !conv;
            pc_last = pc_err;
            if (conv && blockIdx.x == 0) {
                A.red[0] = S.red[0]; A.red[1] = S.red[1]; A.red[2] = S.red[2];
                A.red[3] = (unsigned long long)iters;
            }
        }
        __syncthreads();
        if (!S.more) return;
        iters++;
    }
}

static int sh_step_attr(void) {
    static bool done[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && done[dev]) return 0;
    const cudaError_t e = cudaFuncSetAttribute(sh_k_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ShStepSmem));
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return (int)e;
}

/* b and e of component k of particle i for the next step from the last
 * accepted step's br, er (the shift of the acceleration polynomial by the
 * step-size ratio; b and e zeroed when the ratio passes 20). */
__device__ __forceinline__ void sh_predict_next(const ShView& W, int i, int k, double ratio) {
    if (ratio > 20.0) {
        for (int q = 0; q < 7; q++) { W(S_E + q, k, i) = 0.0; W(S_B + q, k, i) = 0.0; }
        return;
    }
    double qp[8];
    qp[1] = ratio;
    for (int q = 2; q < 8; q++) qp[q] = qp[q - 1] * ratio;
    constexpr double binom[8][8] = {
        {1, 0, 0, 0, 0, 0, 0, 0}, {1, 1, 0, 0, 0, 0, 0, 0}, {1, 2, 1, 0, 0, 0, 0, 0}, {1, 3, 3, 1, 0, 0, 0, 0},
        {1, 4, 6, 4, 1, 0, 0, 0}, {1, 5, 10, 10, 5, 1, 0, 0}, {1, 6, 15, 20, 15, 6, 1, 0}, {1, 7, 21, 35, 35, 21, 7, 1}};
    double br[7], er[7];
#pragma unroll
    for (int q = 0; q < 7; q++) { br[q] = W(S_BR + q, k, i); er[q] = W(S_ER + q, k, i); }
#pragma unroll
    for (int j = 0; j < 7; j++) {
        double s = 0.0;
#pragma unroll
        for (int q = 6; q >= j; q--) s = fma(br[q], binom[q + 1][j + 1], s);
        const double e = qp[j + 1] * s;
        W(S_E + j, k, i) = e;
        W(S_B + j, k, i) = e + (br[j] - er[j]);
    }
}

/* Accepted step of size hstep: one thread per particle component.  x and v
 * advance by the step's quadratures with compensated sums, the start-of-step
 * state is kept for dense output, then b and e are predicted for a next step
 * of hstep * ratio. */
__global__ void sh_k_accept(ShView W, int n, double hstep, double ratio) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, i = t / 3, k = t - 3 * i;
    if (i >= n) return;
    const double h2 = hstep * hstep;
    double b[7];
#pragma unroll
    for (int q = 0; q < 7; q++) b[q] = W(S_B + q, k, i);
    const double a0 = W(S_A0, k, i);
    W(S_PX, k, i) = W(S_X0, k, i) + W(S_XC, k, i);
    W(S_PV, k, i) = W(S_V0, k, i) + W(S_VC, k, i);
    W(S_PA, k, i) = a0;
    double ix = b[6] / 72. + b[5] / 56. + b[4] / 42. + b[3] / 30. + b[2] / 20. + b[1] / 12. + b[0] / 6. + a0 / 2.;
    ix = fma(ix, h2, W(S_V0, k, i) * hstep);
    double y = ix + W(S_XC, k, i);
    const double x0 = W(S_X0, k, i);
    double s = x0 + y;
    W(S_XC, k, i) = y - (s - x0);
    W(S_X0, k, i) = s;
    double iv = b[6] / 8. + b[5] / 7. + b[4] / 6. + b[3] / 5. + b[2] / 4. + b[1] / 3. + b[0] / 2. + a0;
    iv = iv * hstep;
    y = iv + W(S_VC, k, i);
    const double v0 = W(S_V0, k, i);
    s = v0 + y;
    W(S_VC, k, i) = y - (s - v0);
    W(S_V0, k, i) = s;
#pragma unroll
    for (int q = 0; q < 7; q++) { W(S_ER + q, k, i) = W(S_E + q, k, i); W(S_BR + q, k, i) = b[q]; }
    sh_predict_next(W, i, k, ratio);
}

/* Rejected step: b and e from the last accepted step for the retry's size
 * (zero: none accepted yet, both cleared); one thread per particle component. */
__global__ void sh_k_reject(ShView W, int n, double ratio, int zero) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, i = t / 3, k = t - 3 * i;
    if (i >= n) return;
    if (zero) {
        for (int q = 0; q < 7; q++) { W(S_B + q, k, i) = 0.0; W(S_E + q, k, i) = 0.0; }
        return;
    }
    sh_predict_next(W, i, k, ratio);
}

/* All particles at one time t with the block-cooperative evaluation: block b
 * takes particles [32 b, 32 b + 32) (state n x 6, params n x 3 or null),
 * builds the table of t and splits each particle's terms over its four
 * warps; the partial sums are added ((w3 + w2) + w1) + w0 as in the step
 * kernel. */
__global__ void __launch_bounds__(128) sh_k_forces_coop(const DevEphem* __restrict__ Ep, ForceCfg c, int n, double t,
                                                        const double* __restrict__ state,
                                                        const double* __restrict__ params, double* acc, int* status) {
    extern __shared__ __align__(16) unsigned char sh_smem[];
    ShStepSmem& S = *reinterpret_cast<ShStepSmem*>(sh_smem);
    const DevEphem& E = *Ep;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int i = 32 * blockIdx.x + lane;
    const bool live = i < n;
    AgStageCursor cur;
    int stage_fail = 0;
    int bad = ag_coop_table_pass1<false>(E, c, t, S.scr, S.tab[0], tid, nullptr, cur, &stage_fail);
    bad = __syncthreads_or(bad);
    if (bad) {
        if (status && tid < 32 && live) status[i] = AG_ERR_COVERAGE;
        return;
    }
    ag_coop_table_pass2(E, c, t, S.tab[0], S.scr, tid);
    __syncthreads();
    if (c.geocentric == 1) { ag_coop_rel_geo(E, S.tab[0], tid); __syncthreads(); }
    if (wid == 1 && (c.forces & AG_F_EIH)) ag_coop_eih_sources(E, c, S.tab[0].T, lane);
    __syncthreads();
    double x[3] = {0.0, 0.0, 0.0}, v[3] = {0.0, 0.0, 0.0}, prm[3] = {0.0, 0.0, 0.0};
    const double* Ap = nullptr;
    if (live) {
        for (int k = 0; k < 3; k++) { x[k] = state[6 * (size_t)i + k]; v[k] = state[6 * (size_t)i + 3 + k]; }
        if (params) { prm[0] = params[3 * (size_t)i]; prm[1] = params[3 * (size_t)i + 1]; prm[2] = params[3 * (size_t)i + 2]; Ap = prm; }
    }
    double a[3] = {0.0, 0.0, 0.0};
    if (wid < 2) ag_coop_force_split01(wid, live, S.seps, lane, S.tab[0], E, c, x, v, Ap, a);
    else if (live) ag_coop_force_part<false>(wid, S.tab[0], E, c, x, v, Ap, a, nullptr);
    if (live) { S.pa[wid][0][lane] = a[0]; S.pa[wid][1][lane] = a[1]; S.pa[wid][2][lane] = a[2]; }
    __syncthreads();
    if (tid < 96 && live) {
        const int k = wid;
        acc[3 * (size_t)i + k] = ((S.pa[3][k][lane] + S.pa[2][k][lane]) + S.pa[1][k][lane]) + S.pa[0][k][lane];
        if (k == 0 && status) status[i] = AG_OK;
    }
}

int ag_launch_forces_coop(const DevEphem& E, const ForceCfg& c, int n, double t, const double* state,
                          const double* params, double* acc, int* status, cudaStream_t s) {
    if (n <= 0) return 0;
    static bool done[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (!(dev >= 0 && dev < 64 && done[dev])) {
        const cudaError_t e = cudaFuncSetAttribute(sh_k_forces_coop, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)sizeof(ShStepSmem));
        if (e != cudaSuccess) return (int)e;
        if (dev >= 0 && dev < 64) done[dev] = true;
    }
    sh_k_forces_coop<<<(n + 31) / 32, 128, sizeof(ShStepSmem), s>>>(E.self_dev, c, n, t, state, params, acc, status);
    return (int)cudaGetLastError();
}

/* ------------------------------------------------------------------ host side */

struct AgSharedSim {
    int cap = 0;                  /* particle capacity (stride) */
    double* d_ws = nullptr;
    double* d_params = nullptr;
    size_t params_cap = 0;
    int* d_vstart = nullptr;
    int* d_vindex = nullptr;
    int* d_vcfg = nullptr;
    size_t vcap = 0;
    int* d_plist = nullptr;       /* particles per block of the step kernel */
    int* d_pstart = nullptr;
    int* d_vowner = nullptr;      /* real particle of each variational entry */
    size_t pcap = 0;
    int nblocks = 1;
    AgCoopTab* d_tab = nullptr;   /* the step's node tables (several blocks) */
    unsigned long long* d_red = nullptr;  /* 16 words: maxima, iterations, rotating buffers */
    unsigned* d_bar = nullptr;    /* grid barrier of the cooperative step launch */
    int coop_blocks = -1;         /* blocks a cooperative step launch can hold (-1: not yet asked) */
    int* d_status = nullptr;
    cudaStream_t stream = nullptr;
    double* h_pin = nullptr;      /* pinned staging, 6*cap doubles */
    int n = 0, n_real = 0;
    bool state_on_device = false; /* device x0/v0 match sim->particles */
    double t = 0, tc = 0, dt_last_success = 0, dir = 0;
};

AgSharedSim* ag_shared_create(void) { return new AgSharedSim(); }
void ag_shared_free(AgSharedSim* s) {
    if (!s) return;
    if (s->d_ws) cudaFree(s->d_ws);
    if (s->d_params) cudaFree(s->d_params);
    if (s->d_vstart) cudaFree(s->d_vstart);
    if (s->d_vindex) cudaFree(s->d_vindex);
    if (s->d_vcfg) cudaFree(s->d_vcfg);
    if (s->d_plist) cudaFree(s->d_plist);
    if (s->d_pstart) cudaFree(s->d_pstart);
    if (s->d_vowner) cudaFree(s->d_vowner);
    if (s->d_tab) cudaFree(s->d_tab);
    if (s->d_red) cudaFree(s->d_red);
    if (s->d_bar) cudaFree(s->d_bar);
    if (s->d_status) cudaFree(s->d_status);
    if (s->h_pin) cudaFreeHost(s->h_pin);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

static int sh_reserve(AgSharedSim* s, int n) {
    if (!s->stream && ag_cuda_check(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "stream")) return 1;
    if (!s->d_red) {
        if (ag_cuda_check(cudaMalloc(&s->d_red, 16 * sizeof(unsigned long long)), "cudaMalloc(red)")) return 1;
        if (ag_cuda_check(cudaMalloc(&s->d_bar, 4 * sizeof(unsigned)), "cudaMalloc(barrier)")) return 1;
        if (ag_cuda_check(cudaMalloc(&s->d_status, sizeof(int)), "cudaMalloc(status)")) return 1;
        if (ag_cuda_check(cudaMalloc(&s->d_tab, 8 * sizeof(AgCoopTab)), "cudaMalloc(node tables)")) return 1;
    }
    if (n <= s->cap) return 0;
    int cap = n < 64 ? 64 : n;
    double* ws = nullptr;
    if (ag_cuda_check(cudaMalloc(&ws, sizeof(double) * (size_t)S_NF * 3 * cap), "cudaMalloc(IAS15 state)")) return 1;
    cudaMemsetAsync(ws, 0, sizeof(double) * (size_t)S_NF * 3 * cap, s->stream);
    if (s->d_ws) cudaFree(s->d_ws);
    s->d_ws = ws;
    if (s->h_pin) cudaFreeHost(s->h_pin);
    /* staging: 5 fields x 3 components (X0, V0, A0, XC, VC) on copy-back */
    if (ag_cuda_check(cudaMallocHost(&s->h_pin, sizeof(double) * 15 * (size_t)cap), "cudaMallocHost")) return 1;
    s->cap = cap;
    s->state_on_device = false;
    return 0;
}

/* Upload variational bookkeeping (per real particle: its variational
 * particles in var_config order) and the Marsden parameters. */
static int sh_upload_vars(AgSharedSim* s, struct reb_simulation* r, const double* params, AgForceIO* io) {
    const int n = r->N, n_real = r->N - r->N_var;
    std::vector<int> cnt((size_t)n_real + 1, 0), start((size_t)n_real + 1, 0);
    const int nvc = r->N_var_config;
    for (int v = 0; v < nvc; v++) {
        const int tp = r->var_config[v].testparticle;
        if (tp >= 0 && tp < n_real && r->var_config[v].index >= 0 && r->var_config[v].index < n) cnt[(size_t)tp]++;
    }
    for (int j = 0; j < n_real; j++) start[(size_t)j + 1] = start[(size_t)j] + cnt[(size_t)j];
    std::vector<int> idx((size_t)start[(size_t)n_real] + 1), cfg((size_t)start[(size_t)n_real] + 1), fill(start.begin(), start.end());
    for (int v = 0; v < nvc; v++) {
        const int tp = r->var_config[v].testparticle;
        if (tp >= 0 && tp < n_real && r->var_config[v].index >= 0 && r->var_config[v].index < n) {
            idx[(size_t)fill[(size_t)tp]] = r->var_config[v].index;
            cfg[(size_t)fill[(size_t)tp]] = v;
            fill[(size_t)tp]++;
        }
    }
    const size_t nv = (size_t)start[(size_t)n_real];
    if (n_real + 1 + nv > s->vcap) {
        if (s->d_vstart) cudaFree(s->d_vstart);
        if (s->d_vindex) cudaFree(s->d_vindex);
        if (s->d_vcfg) cudaFree(s->d_vcfg);
        s->vcap = (size_t)n_real + 1 + nv + 64;
        if (ag_cuda_check(cudaMalloc(&s->d_vstart, sizeof(int) * s->vcap), "cudaMalloc(vars)") ||
            ag_cuda_check(cudaMalloc(&s->d_vindex, sizeof(int) * s->vcap), "cudaMalloc(vars)") ||
            ag_cuda_check(cudaMalloc(&s->d_vcfg, sizeof(int) * s->vcap), "cudaMalloc(vars)"))
            return 1;
    }
    cudaMemcpyAsync(s->d_vstart, start.data(), sizeof(int) * ((size_t)n_real + 1), cudaMemcpyHostToDevice, s->stream);
    if (nv) {
        cudaMemcpyAsync(s->d_vindex, idx.data(), sizeof(int) * nv, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->d_vcfg, cfg.data(), sizeof(int) * nv, cudaMemcpyHostToDevice, s->stream);
    }
    /* block lists of the step kernel: block b owns real particles
     * [32 b, 32 b + 32) and their variational particles; particles no real
     * particle lists go to the last block */
    const int nb = n_real > 0 ? (n_real + 31) / 32 : 1;
    std::vector<int> owner((size_t)n, -1), pstart((size_t)nb + 1, 0), plist((size_t)n), vowner(nv + 1, 0);
    for (int j = 0; j < n_real; j++) owner[(size_t)j] = j / 32;
    for (int j = 0; j < n_real; j++)
        for (int q = start[(size_t)j]; q < start[(size_t)j + 1]; q++) {
            vowner[(size_t)q] = j;
            if (idx[(size_t)q] >= n_real && owner[(size_t)idx[(size_t)q]] < 0) owner[(size_t)idx[(size_t)q]] = j / 32;
        }
    for (int p = 0; p < n; p++) {
        if (owner[(size_t)p] < 0) owner[(size_t)p] = nb - 1;
        pstart[(size_t)owner[(size_t)p] + 1]++;
    }
    for (int b = 0; b < nb; b++) pstart[(size_t)b + 1] += pstart[(size_t)b];
    {
        std::vector<int> at(pstart.begin(), pstart.end() - 1);
        for (int p = 0; p < n; p++) plist[(size_t)at[(size_t)owner[(size_t)p]]++] = p;
    }
    if ((size_t)n + nb + nv + 1 > s->pcap) {
        if (s->d_plist) cudaFree(s->d_plist);
        if (s->d_pstart) cudaFree(s->d_pstart);
        if (s->d_vowner) cudaFree(s->d_vowner);
        s->d_plist = s->d_pstart = s->d_vowner = nullptr;
        s->pcap = (size_t)n + nb + nv + 1 + 64;
        if (ag_cuda_check(cudaMalloc(&s->d_plist, sizeof(int) * s->pcap), "cudaMalloc(block lists)") ||
            ag_cuda_check(cudaMalloc(&s->d_pstart, sizeof(int) * s->pcap), "cudaMalloc(block lists)") ||
            ag_cuda_check(cudaMalloc(&s->d_vowner, sizeof(int) * s->pcap), "cudaMalloc(block lists)"))
            return 1;
    }
    cudaMemcpyAsync(s->d_plist, plist.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(s->d_pstart, pstart.data(), sizeof(int) * ((size_t)nb + 1), cudaMemcpyHostToDevice, s->stream);
    if (nv) cudaMemcpyAsync(s->d_vowner, vowner.data(), sizeof(int) * nv, cudaMemcpyHostToDevice, s->stream);
    s->nblocks = nb;
    io->var_start = nv ? s->d_vstart : nullptr;
    io->var_index = s->d_vindex;
    io->var_cfg = s->d_vcfg;
    io->params = nullptr;
    if (params) {
        const size_t np = 3 * (size_t)(n_real + nvc);
        if (np > s->params_cap) {
            if (s->d_params) cudaFree(s->d_params);
            s->params_cap = np + 64;
            if (ag_cuda_check(cudaMalloc(&s->d_params, sizeof(double) * s->params_cap), "cudaMalloc(params)")) return 1;
        }
        cudaMemcpyAsync(s->d_params, params, sizeof(double) * np, cudaMemcpyHostToDevice, s->stream);
        io->params = s->d_params;
    }
    /* the host vectors above must outlive the async copies */
    return ag_cuda_check(cudaStreamSynchronize(s->stream), "upload variational map");
}

int ag_shared_forces(AgSharedSim* s, const DevEphem& E, const ForceCfg& c, struct reb_simulation* r,
                     const double* params, int* status_out) {
    const int n = r->N, n_real = r->N - r->N_var;
    if (n <= 0) return 0;
    if (sh_reserve(s, n)) return 1;
    AgForceIO io;
    std::memset(&io, 0, sizeof(io));
    if (sh_upload_vars(s, r, params, &io)) return 1;
    ShView W{s->d_ws, s->cap};
    double* h = s->h_pin;
    for (int i = 0; i < n; i++) {
        const reb_particle& p = r->particles[i];
        h[0 * (size_t)s->cap + i] = p.x; h[1 * (size_t)s->cap + i] = p.y; h[2 * (size_t)s->cap + i] = p.z;
        h[3 * (size_t)s->cap + i] = p.vx; h[4 * (size_t)s->cap + i] = p.vy; h[5 * (size_t)s->cap + i] = p.vz;
    }
    double* xp = &W.w[(size_t)S_XP * 3 * s->cap];
    double* vp = &W.w[(size_t)S_VP * 3 * s->cap];
    double* at = &W.w[(size_t)S_AT * 3 * s->cap];
    cudaMemcpyAsync(xp, h, sizeof(double) * 3 * (size_t)s->cap, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(vp, h + 3 * (size_t)s->cap, sizeof(double) * 3 * (size_t)s->cap, cudaMemcpyHostToDevice, s->stream);
    cudaMemsetAsync(at, 0, sizeof(double) * 3 * (size_t)s->cap, s->stream);
    cudaMemsetAsync(s->d_status, 0, sizeof(int), s->stream);
    io.n_real = n_real; io.stride = s->cap; io.x = xp; io.v = vp; io.a = at; io.status = s->d_status;
    int e = ag_launch_forces_table(E, c, r->t, io, s->stream);
    if (e) return ag_cuda_check((cudaError_t)e, "force kernel");
    cudaMemcpyAsync(h + 6 * (size_t)s->cap, at, sizeof(double) * 3 * (size_t)s->cap, cudaMemcpyDeviceToHost, s->stream);
    int st = 0;
    cudaMemcpyAsync(&st, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, s->stream);
    if (ag_cuda_check(cudaStreamSynchronize(s->stream), "force kernel")) return 1;
    const double* a = h + 6 * (size_t)s->cap;
    for (int i = 0; i < n; i++) {
        r->particles[i].ax += a[0 * (size_t)s->cap + i];
        r->particles[i].ay += a[1 * (size_t)s->cap + i];
        r->particles[i].az += a[2 * (size_t)s->cap + i];
    }
    s->state_on_device = false;
    *status_out = st;
    return 0;
}

/* Integrate r to tmax with IAS15 on the device.  Returns 0 or 1 (CUDA error);
 * *status_out receives an ASSIST status of the force model. */
int ag_shared_integrate(AgSharedSim* s, const DevEphem& E, const ForceCfg& c, struct reb_simulation* r,
                        const double* params, double tmax, ShIntegrateOut* out) {
    const int n = r->N, n_real = r->N - r->N_var;
    out->status = 0;
    if (n <= 0 || r->t == tmax) return 0;
    if (sh_tables_init()) return ag_cuda_check(cudaErrorInvalidValue, "IAS15 tables");
    if (ag_cuda_check((cudaError_t)sh_step_attr(), "IAS15 step kernel shared memory")) return 1;
    if (sh_reserve(s, n)) return 1;
    AgForceIO io;
    std::memset(&io, 0, sizeof(io));
    if (sh_upload_vars(s, r, params, &io)) return 1;
    ShView W{s->d_ws, s->cap};
    const size_t F = 3 * (size_t)s->cap;
    const int tpb = 128, blocks3 = (3 * n + tpb - 1) / tpb, nb = s->nblocks;
    cudaStream_t st = s->stream;
    double dir = tmax >= r->t ? 1.0 : -1.0;
    /* the host particles are authoritative: upload them every call; keep the
     * predictor state only when this call continues the previous one */
    const bool cont = s->state_on_device && s->t == r->t && s->n == n && s->dir == dir;
    {
        double* h = s->h_pin;
        for (int i = 0; i < n; i++) {
            const reb_particle& p = r->particles[i];
            h[0 * (size_t)s->cap + i] = p.x; h[1 * (size_t)s->cap + i] = p.y; h[2 * (size_t)s->cap + i] = p.z;
            h[3 * (size_t)s->cap + i] = p.vx; h[4 * (size_t)s->cap + i] = p.vy; h[5 * (size_t)s->cap + i] = p.vz;
        }
        cudaMemcpyAsync(W.w + (size_t)S_X0 * F, h, sizeof(double) * F, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(W.w + (size_t)S_V0 * F, h + F, sizeof(double) * F, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(W.w + (size_t)S_XC * F, 0, sizeof(double) * 2 * F, st);
        if (!cont) {
            cudaMemsetAsync(W.w + (size_t)S_B * F, 0, sizeof(double) * 35 * F, st);
            s->dt_last_success = 0.0;
        }
        s->t = r->t;
        s->tc = 0.0;
        s->n = n;
        s->dir = dir;
    }
    s->n_real = n_real;
    io.n_real = n_real; io.stride = s->cap;
    io.x = W.w + (size_t)S_XP * F; io.v = W.w + (size_t)S_VP * F; io.a = W.w + (size_t)S_AT * F;
    io.status = s->d_status;
    const double h_nodes[8] = IAS15_H_INIT;
    double dt = r->dt;
    if (dt * dir <= 0) dt = dir * std::fabs(dt != 0 ? dt : 0.001);
    const double eps = r->ri_ias15.epsilon, min_dt = r->ri_ias15.min_dt;
    unsigned long long red[4];
    int hstat = 0;
    unsigned bar_gave_up = 0;
    /* several blocks run a step in one cooperative launch when all of them
     * fit on the device at once; otherwise one launch per iteration
     * (ASSIST_GB300_SHARED_COOP=0 forces that path) */
    if (s->coop_blocks < 0) {
        int dev = 0, sms = 0, bps = 0, can = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&can, cudaDevAttrCooperativeLaunch, dev);
        if (const char* ev = getenv("ASSIST_GB300_SHARED_COOP"))
            if (atoi(ev) == 0) can = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, sh_k_step, tpb, sizeof(ShStepSmem)) != cudaSuccess) bps = 0;
        s->coop_blocks = can ? bps * sms : 0;
    }
    bool use_coop = nb > 1 && nb <= s->coop_blocks;
    long long steps = 0;
    while (s->t != tmax) {
        const double rem = (tmax - s->t) - s->tc;
        bool last = false;
        double hstep = dt;
        if (std::fabs(dt) >= std::fabs(rem)) { hstep = rem; last = true; }
        ShStepArgs A;
        A.W = W; A.io = io; A.vowner = s->d_vowner; A.plist = s->d_plist; A.pstart = s->d_pstart; A.red = s->d_red;
        A.gtab = s->d_tab;
        A.bar = s->d_bar;
        A.coop = 0;
        A.hstep = hstep;
        A.tn[0] = s->t;
        for (int node = 1; node < 8; node++) A.tn[node] = s->t + (s->tc + hstep * h_nodes[node]);
        A.first = 1;
        cudaMemsetAsync(s->d_status, 0, sizeof(int), st);
        int iters = 1;
        if (nb == 1 || use_coop) {
            /* one block, or every block resident in a cooperative launch: the
             * whole predictor-corrector loop in one launch */
            if (nb == 1) {
                sh_k_step<<<1, tpb, sizeof(ShStepSmem), st>>>(E.self_dev, c, A);
                if (ag_cuda_check(cudaGetLastError(), "IAS15 step kernel")) return 1;
            } else {
                A.coop = 1;
                cudaMemsetAsync(s->d_red, 0, 16 * sizeof(unsigned long long), st);
                cudaMemsetAsync(s->d_bar, 0, 4 * sizeof(unsigned), st);
                const DevEphem* ep = E.self_dev;
                ForceCfg cc = c;
                void* args[] = {(void*)&ep, (void*)&cc, (void*)&A};
                const cudaError_t le =
                    cudaLaunchCooperativeKernel((const void*)sh_k_step, nb, tpb, args, sizeof(ShStepSmem), st);
                if (le == cudaErrorCooperativeLaunchTooLarge) {
                    /* the blocks no longer fit at once: this step and the
                     * rest in one launch per iteration */
                    cudaGetLastError();
                    s->coop_blocks = 0;
                    use_coop = false;
                    continue;
                }
                if (ag_cuda_check(le, "IAS15 step kernel (cooperative)")) return 1;
                cudaMemcpyAsync(&bar_gave_up, s->d_bar + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
            }
            cudaMemcpyAsync(red, s->d_red, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(&hstat, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (ag_cuda_check(cudaStreamSynchronize(st), "IAS15 step")) return 1;
            if (bar_gave_up) {
                ag_set_error("IAS15 step kernel: a block stopped waiting at the grid barrier");
                return 1;
            }
            iters = (int)red[3];
            out->evals += 1 + 7 * (long long)iters;
            if (hstat != 0) out->status = hstat;
        } else {
            out->evals++;
            double pc_last = 1e300, pc_err = 0.0;
            while (true) {
                cudaMemsetAsync(s->d_red, 0, 3 * sizeof(unsigned long long), st);
                sh_k_step<<<nb, tpb, sizeof(ShStepSmem), st>>>(E.self_dev, c, A);
                if (ag_cuda_check(cudaGetLastError(), "IAS15 step kernel")) return 1;
                A.first = 0;
                out->evals += 7;
                cudaMemcpyAsync(red, s->d_red, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(&hstat, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, st);
                if (ag_cuda_check(cudaStreamSynchronize(st), "IAS15 iteration")) return 1;
                if (hstat != 0) { out->status = hstat; break; }
                double mdb, ma;
                std::memcpy(&mdb, &red[0], 8);
                std::memcpy(&ma, &red[1], 8);
                pc_err = mdb / ma;
                const bool conv = (pc_err < 1e-16) || (iters > 2 && pc_last <= pc_err) || (iters >= 12);
                if (conv) break;
                pc_last = pc_err;
                iters++;
            }
        }
        if (out->status) break;
        out->iterations += iters;
        double mb, ma;
        std::memcpy(&ma, &red[1], 8);
        std::memcpy(&mb, &red[2], 8);
        double dt_new = hstep;
        bool reject = false;
        if (eps > 0.0) {
            const double err = mb / ma;
            const double safety = 0.25;
            if (std::isnormal(err)) dt_new = std::pow(eps / err, 1.0 / 7.0) * hstep;
            else dt_new = hstep / safety;
            if (std::fabs(dt_new) < min_dt) dt_new = std::copysign(min_dt, dt_new);
            const double ratio = dt_new / hstep;
            if (std::fabs(ratio) < safety) reject = true;
            else if (std::fabs(ratio) > 1.0 / safety) dt_new = hstep / safety;
        }
        if (reject) {
            out->rejected++;
            if (s->dt_last_success != 0.0) sh_k_reject<<<blocks3, tpb, 0, st>>>(W, n, dt_new / s->dt_last_success, 0);
            else sh_k_reject<<<blocks3, tpb, 0, st>>>(W, n, 0.0, 1);
            dt = dt_new;
            continue;
        }
        sh_k_accept<<<blocks3, tpb, 0, st>>>(W, n, hstep, dt_new / hstep);
        out->accepted++;
        {
            const double y = hstep + s->tc;
            const double sum = s->t + y;
            s->tc = y - (sum - s->t);
            s->t = sum;
        }
        s->dt_last_success = hstep;
        out->dt_last_done = hstep;
        dt = dt_new;
        steps++;
        if (last) { s->t = tmax; s->tc = 0.0; }
        if (out->max_steps > 0 && steps >= out->max_steps && s->t != tmax) { out->status = -1; break; }
    }
    /* copy back: current state and the last step's start state / b for dense output */
    double* h = s->h_pin;
    cudaMemcpyAsync(h, W.w + (size_t)S_X0 * F, sizeof(double) * 5 * F, cudaMemcpyDeviceToHost, st);
    if (ag_cuda_check(cudaStreamSynchronize(st), "copy back")) return 1;
    const double* X0 = h; const double* V0 = h + F; const double* XC = h + 3 * F; const double* VC = h + 4 * F;
    for (int i = 0; i < n; i++) {
        reb_particle& p = r->particles[i];
        p.x = X0[i] + XC[i]; p.y = X0[s->cap + i] + XC[s->cap + i]; p.z = X0[2 * (size_t)s->cap + i] + XC[2 * (size_t)s->cap + i];
        p.vx = V0[i] + VC[i]; p.vy = V0[s->cap + i] + VC[s->cap + i]; p.vz = V0[2 * (size_t)s->cap + i] + VC[2 * (size_t)s->cap + i];
    }
    if (out->dense) {
        /* start-of-last-step positions, velocities, accelerations and b */
        std::vector<double> tmp(3 * F);
        cudaMemcpy(tmp.data(), W.w + (size_t)S_PX * F, sizeof(double) * 3 * F, cudaMemcpyDeviceToHost);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                out->dense_x0[3 * i + k] = tmp[(size_t)k * s->cap + i];
                out->dense_v0[3 * i + k] = tmp[F + (size_t)k * s->cap + i];
                out->dense_a0[3 * i + k] = tmp[2 * F + (size_t)k * s->cap + i];
            }
        std::vector<double> br(7 * F);
        cudaMemcpy(br.data(), W.w + (size_t)S_BR * F, sizeof(double) * 7 * F, cudaMemcpyDeviceToHost);
        for (int q = 0; q < 7; q++)
            for (int i = 0; i < n; i++)
                for (int k = 0; k < 3; k++) out->dense_b[q][3 * i + k] = br[(size_t)q * F + (size_t)k * s->cap + i];
    }
    r->t = s->t;
    r->dt = dt;
    s->state_on_device = true;
    return 0;
}

/* State at fraction h of the last accepted step of size dt, from that step's
 * start (x, v, a) and converged b, as ASSIST interpolates it
 * (src/assist.c:556-597: the same s- and sv-coefficient recurrences and the
 * same sums, without contraction), into XP, VP. */
__global__ void sh_k_interp(ShView W, int n, double dt, double h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s[9], sv[8];
    s[0] = __dmul_rn(dt, h);
    s[1] = __ddiv_rn(__dmul_rn(s[0], s[0]), 2.);
    s[2] = __ddiv_rn(__dmul_rn(s[1], h), 3.);
    s[3] = __ddiv_rn(__dmul_rn(s[2], h), 2.);
    s[4] = __ddiv_rn(__dmul_rn(__dmul_rn(3., s[3]), h), 5.);
    s[5] = __ddiv_rn(__dmul_rn(__dmul_rn(2., s[4]), h), 3.);
    s[6] = __ddiv_rn(__dmul_rn(__dmul_rn(5., s[5]), h), 7.);
    s[7] = __ddiv_rn(__dmul_rn(__dmul_rn(3., s[6]), h), 4.);
    s[8] = __ddiv_rn(__dmul_rn(__dmul_rn(7., s[7]), h), 9.);
    sv[0] = __dmul_rn(dt, h);
    for (int k = 1; k < 8; k++) sv[k] = __ddiv_rn(__dmul_rn(__dmul_rn((double)k, sv[k - 1]), h), (double)(k + 1));
    for (int k = 0; k < 3; k++) {
        double x = __dmul_rn(s[8], W(S_BR + 6, k, i));
        for (int q = 5; q >= 0; q--) x = __dadd_rn(x, __dmul_rn(s[q + 2], W(S_BR + q, k, i)));
        x = __dadd_rn(x, __dmul_rn(s[1], W(S_PA, k, i)));
        x = __dadd_rn(x, __dmul_rn(s[0], W(S_PV, k, i)));
        double v = __dmul_rn(sv[7], W(S_BR + 6, k, i));
        for (int q = 5; q >= 0; q--) v = __dadd_rn(v, __dmul_rn(sv[q + 1], W(S_BR + q, k, i)));
        v = __dadd_rn(v, __dmul_rn(sv[0], W(S_PA, k, i)));
        W(S_XP, k, i) = __dadd_rn(W(S_PX, k, i), x);
        W(S_VP, k, i) = __dadd_rn(W(S_PV, k, i), v);
    }
}

/* Dense output of the drop-in on the device: the n particles at fraction h
 * of the last step (of size dt) written into out[].x..vz.  Returns 0, or 1
 * when the device holds no step of these n particles. */
int ag_shared_interpolate(AgSharedSim* s, int n, double dt, double h, struct reb_particle* out) {
    if (!s || !s->state_on_device || s->n != n || !s->d_ws) return 1;
    ShView W{s->d_ws, s->cap};
    const size_t F = 3 * (size_t)s->cap;
    sh_k_interp<<<(n + 127) / 128, 128, 0, s->stream>>>(W, n, dt, h);
    double* hb = s->h_pin;
    if (ag_cuda_check(cudaGetLastError(), "interpolation kernel") ||
        ag_cuda_check(cudaMemcpyAsync(hb, W.w + (size_t)S_XP * F, sizeof(double) * 2 * F, cudaMemcpyDeviceToHost,
                                      s->stream), "interpolation copy") ||
        ag_cuda_check(cudaStreamSynchronize(s->stream), "interpolation"))
        return 1;
    for (int i = 0; i < n; i++) {
        out[i].x = hb[i]; out[i].y = hb[(size_t)s->cap + i]; out[i].z = hb[2 * (size_t)s->cap + i];
        out[i].vx = hb[F + i]; out[i].vy = hb[F + (size_t)s->cap + i]; out[i].vz = hb[F + 2 * (size_t)s->cap + i];
    }
    return 0;
}

/* Copy of the shared-step IAS15 tables (diagnostics). out: h[8], rrinv[64], c[49], d[49], fx[72], fv[64]. */
extern "C" int ag_debug_shared_tables(double* out) {
    int e = sh_tables_init();
    if (e) return e;
    cudaMemcpyFromSymbol(out, sh_h, sizeof(double) * 8);
    cudaMemcpyFromSymbol(out + 8, sh_rrinv, sizeof(double) * 64);
    cudaMemcpyFromSymbol(out + 72, sh_c, sizeof(double) * 49);
    cudaMemcpyFromSymbol(out + 121, sh_d, sizeof(double) * 49);
    cudaMemcpyFromSymbol(out + 170, sh_fx, sizeof(double) * 72);
    return (int)cudaMemcpyFromSymbol(out + 242, sh_fv, sizeof(double) * 64);
}
