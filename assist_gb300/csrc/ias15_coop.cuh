/*
 * ias15_coop.cuh -- block-cooperative grouped batched IAS15 (included by
 * kernels_coop.cu).
 *
 * A group of up to 32 particles that share their step times (the same
 * grouping as the warp-grouped kernel) is integrated by one 128-thread block:
 * lane l of every warp works on particle l, and the four warps split the
 * work of each force evaluation so that it runs on all four SM sub-partitions
 * (each has its own FP64 pipe):
 *
 *   warp 0  planets' direct gravity (ASSIST's order, Sun last), Marsden
 *           non-gravitational term, Earth J2-J4, geocentric indirect term
 *   warp 1  EIH/PPN relativity (its per-source sums too), GR potential/simple
 *   warp 2  first half of the asteroids
 *   warp 3  second half of the asteroids, Sun J2
 * (with variational particles, whose Jacobians fill warp 0's registers,
 * Earth J2-J4 stays on warp 2).  Batches are grouped so that particles with
 * non-gravitational parameters share groups: a group whose members have none
 * skips warp 0's costliest term.
 * Warps 0 and 1 both need the eleven particle-planet separations: each forms
 * half and they exchange them through shared memory at a named barrier
 * (without Jacobians; with them each warp forms all eleven).
 *
 * The partial accelerations (and partial Jacobians) meet in shared memory and
 * are summed in a fixed order ((w3 + w2) + w1) + w0, so the planets' terms,
 * the largest, come last as in ASSIST's sum.  The body table of each
 * substep time is built by the whole block: column components of the .440
 * record and asteroid components of the SPK records on different threads, in
 * the reference's exact arithmetic.  Each IAS15 state component has an owner
 * warp that predicts it, forms its acceleration from the partials and
 * updates its g, b and e: x, y, z belong to warps 0, 2, 3 (warps 1, 2, 3
 * with variational particles); the three
 * components of a variational particle share one warp (its J.dx product reads
 * only its own predicted values).
 * Per-particle control values (t, dt, convergence, retirement) are computed
 * identically by all four warps from shared data, so every branch around a
 * block barrier is uniform.
 *
 * Per evaluation this cuts the FP64 instructions on one sub-partition to
 * roughly a third of the warp-grouped kernel's, which is what bounds the
 * longest groups (the tail of a batch).
 *
 * Memory: without variational particles the block keeps the eight node
 * tables of a step (the node times do not change while the predictor-
 * corrector iterates, so each table is built once per step), each with the
 * origin-minus-body half of every separation formed once, and the group's
 * IAS15 state (40 fields x 3 components x 32 lanes) in dynamic shared
 * memory.  The plain kernel is built for two resident blocks per SM (236
 * registers) and for three (168); the host picks three only for batches
 * with many groups per block.
 */

#include "coop_forces.cuh"

/* b, e of one component from the last accepted step's br, er (the shift of
 * the acceleration polynomial to the new step). */
template <int C>
__device__ __forceinline__ void ag_predict_next_comp(const Ws<C>& W, int comp, double ratio) {
    if (ratio > 20.0) {
        for (int k = 0; k < 7; k++) { W(W_E + k, comp) = 0.0; W(W_B + k, comp) = 0.0; }
        return;
    }
    double q[8];
    q[1] = ratio;
    for (int k = 2; k < 8; k++) q[k] = q[k - 1] * ratio;
    constexpr double binom[8][8] = {
        {1, 0, 0, 0, 0, 0, 0, 0}, {1, 1, 0, 0, 0, 0, 0, 0}, {1, 2, 1, 0, 0, 0, 0, 0}, {1, 3, 3, 1, 0, 0, 0, 0},
        {1, 4, 6, 4, 1, 0, 0, 0}, {1, 5, 10, 10, 5, 1, 0, 0}, {1, 6, 15, 20, 15, 6, 1, 0}, {1, 7, 21, 35, 35, 21, 7, 1}};
    double br[7], er[7];
#pragma unroll
    for (int k = 0; k < 7; k++) { br[k] = W(W_BR + k, comp); er[k] = W(W_ER + k, comp); }
#pragma unroll
    for (int j = 0; j < 7; j++) {
        double s = 0.0;
#pragma unroll
        for (int k = 6; k >= j; k--) s = fma(br[k], binom[k + 1][j + 1], s);
        const double e = q[j + 1] * s;
        W(W_E + j, comp) = e;
        W(W_B + j, comp) = e + (br[j] - er[j]);
    }
}

/* Owner warp of IAS15 component comp: x, y, z -> warps 0, 2, 3 (warps
 * 1..3 with variational particles, which go to warps 0, 0, 1, 2, 3, 1). */
template <int NV>
__device__ __forceinline__ int ag_coop_owner(int comp) {
    if (comp < 3) return NV == 0 ? (comp == 0 ? 0 : comp + 1) : comp + 1;
    const int q = (comp - 3) / 3;
    return q < 2 ? 0 : ((q == 2 || q == 5) ? 1 : (q == 3 ? 2 : 3));
}

/* Position component owned by warp w (-1: none). */
template <int NV>
__device__ __forceinline__ int ag_coop_pcomp(int w) {
    return NV == 0 ? (w == 0 ? 0 : (w == 1 ? -1 : w - 1)) : w - 1;
}

template <int NV>
struct AgCoopShared {
    static constexpr int C = 3 * (1 + NV);
    AgCoopTab tab[NV == 0 ? 8 : 1]; /* body tables; without Jacobians one per node, kept through the
                                       predictor-corrector iterations of a step (the node times do
                                       not change while it iterates) */
    AgCoopScratch scr;
    double xs[C][32], vs[C][32];                    /* state at the current node */
    double pa[4][3][32];                            /* partial accelerations */
    typename std::conditional<NV == 0, AgCoopSeps, char>::type seps;   /* warp 0 <-> warp 1 separations */
    double pj[NV > 0 ? 4 : 1][NV > 0 ? 18 : 1][32]; /* partial Jacobians */
    double ra[3][32], rdb[3][32];                   /* |a|, |delta b6| of x, y, z at node 7 */
    double rb6[3][32];                              /* |b6| of x, y, z after convergence */
    double pcx[8][9], pcv[8][8];                    /* predictor coefficients of nodes 1..7 of the step */
    double ptn[8];                                  /* and the node times */
    AgF2 xsf[NV == 0 ? 3 : 1][32];                  /* the state's position as float pairs (asteroid terms) */
    double sdn[32], sdc[32];                        /* each lane's next-step proposal, capped and uncapped */
    int srej[32];                                   /* and whether it rejects the step */
    int fin[3][32];
    int g, stop;
    int stage_fail;                                 /* a staged record copy did not complete */
    int wg_off;                                     /* learned warm start switched off for this group */
    int rot;                                        /* role rotation of this block */
};

/* Shared buffers of the learned warm start (dynamic shared memory, present
 * only when a network is loaded or steps are logged). */
struct AgWarmSmem {
    AgMlpSmem M;
    double corr[7][3][32];          /* (br - er)_kc of each lane */
    float bpa[7][3][32];            /* |b_pred_kc| */
    float tgt[7][3][32];            /* logged targets */
    float xf[32][AG_MLP_IN + 1];    /* features of this step (logged with the target) */
    double kappa[7][32];
    int valid[32];
};

/* Distance from (x, y, z) to the nearest of the eleven planets in the table. */
__device__ __forceinline__ double ag_nearest_planet(const AgTable& T, double x, double y, double z) {
    double m = 1e300;
#pragma unroll
    for (int k = 0; k < AG_NPL; k++) {
        const double dx = x - T.P.x[k], dy = y - T.P.y[k], dz = z - T.P.z[k];
        m = fmin(m, fma(dx, dx, fma(dy, dy, dz * dz)));
    }
    return sqrt(m);
}

/* Node-0 part of the learned warm start for one group (all threads of the
 * block call it): owners publish (br - er) and |b_pred| of the particle's
 * x, y, z (variational particles keep the plain prediction), warp 0 forms
 * the features, the block runs the network, owners add kappa_k y_kc to b.
 * Every 8th step of a group is a plain probe (no inference).  Returns whether
 * the network ran (block-uniform).  Kept out of line so the plain kernel's
 * register allocation is not shaped by it. */
template <int NV>
__device__ __noinline__ bool ag_coop_warm_start(const AgBatchArgs& A, double* ws, int nslots, int slot, AgWarmSmem& WS,
                                               const AgTable& Tab, int lane, int wid, bool live, bool warm, bool wl_on,
                                               double hstep, double dtls, long long steps, bool& w_applied,
                                               bool& w_probe, unsigned long long& n_wused,
                                               unsigned long long& n_wfall) {
    const Ws<3 * (1 + NV)> W{ws, nslots, slot};
    const int pc = ag_coop_pcomp<NV>(wid);
    if (live && pc >= 0)
        for (int k = 0; k < 7; k++) {
            WS.corr[k][pc][lane] = W(W_BR + k, pc) - W(W_ER + k, pc);
            WS.bpa[k][pc][lane] = (float)fabs(W(W_B + k, pc));
        }
    __syncthreads();
    if (wid == 0) {
        bool ok = false;
        if (live) {
            double corr[7][3], kap[7];
            float bpa[7][3], x[AG_MLP_IN];
            for (int k = 0; k < 7; k++)
                for (int c = 0; c < 3; c++) { corr[k][c] = WS.corr[k][c][lane]; bpa[k][c] = WS.bpa[k][c][lane]; }
            const double x0 = W(W_X0, 0), y0 = W(W_X0, 1), z0 = W(W_X0, 2);
            const double rx = sqrt(fma(x0, x0, fma(y0, y0, z0 * z0)));
            ok = ag_warm_features(corr, bpa, hstep, dtls, rx, ag_nearest_planet(Tab, x0, y0, z0), x, kap);
            for (int k = 0; k < 7; k++) WS.kappa[k][lane] = kap[k];
            for (int i = 0; i < AG_MLP_IN; i++) { WS.xf[lane][i] = x[i]; WS.M.X[lane][i] = __float2bfloat16_rn(x[i]); }
        } else {
            for (int i = 0; i < AG_MLP_IN; i++) WS.M.X[lane][i] = __float2bfloat16_rn(0.0f);
        }
        WS.valid[lane] = ok ? 1 : 0;
    }
    __syncthreads();
    const bool valid = live && WS.valid[lane];
    w_probe = warm && valid && wl_on && (steps & 7) == 7;
    const bool want = warm && valid && wl_on && !w_probe;
    const bool ran = __syncthreads_or(want);
    if (ran) {
        ag_mlp_infer_block(*A.mlp, WS.M, wid, lane);
        if (want) {
            bool ok_y = true;
            for (int o = 0; o < AG_MLP_OUT; o++) {
                const float y = WS.M.Y[lane][o];
                ok_y = ok_y && isfinite(y) && fabsf(y) <= AG_MLP_YCLIP;
            }
            if (ok_y) {
                w_applied = true;
                if (pc >= 0)
                    for (int k = 0; k < 7; k++)
                        W(W_B + k, pc) = fma(WS.kappa[k][lane], (double)WS.M.Y[lane][3 * k + pc], W(W_B + k, pc));
                if (wid == 0) n_wused++;
            } else if (wid == 0) {
                n_wfall++;
            }
        }
    }
    return ran;
}

/* Dynamic shared memory of a block: the warm-start buffers (when present)
 * or, in the plain kernel without variational particles, the group's IAS15
 * state (40 fields x 3 components x 32 lanes, 30 KB).  Otherwise the state
 * stays in the global workspace, indexed by slot (both would not leave room
 * for two blocks per SM). */
template <int NV, bool WARM, bool STAGE = false>
struct AgCoopDyn {
    static constexpr bool ws_shared = NV == 0 && !WARM;
    static constexpr size_t warm = WARM ? (sizeof(AgWarmSmem) + 15) / 16 * 16 : 0;
    static constexpr size_t ws = ws_shared ? sizeof(double) * W_NF * 3 * 32 : 0;
    static constexpr size_t stage_off = warm + ws;        /* the staged .440 record (STAGE) */
    static constexpr size_t stage = STAGE ? (sizeof(AgRecStage) + 15) / 16 * 16 : 0;
    static constexpr size_t bytes = warm + ws + stage;
};

/* OCC: resident blocks per SM the kernel is compiled for.  The plain kernel
 * comes in three builds: 2 (242 registers), 3 (168 registers, a few
 * spills: faster on batches with many groups per block, slower on small
 * batches whose longest groups set the time), and 2 with the active .440
 * record staged in shared memory by bulk copies (STAGE; its 8 KB buffer does
 * not fit beside three blocks); the variational and warm-start
 * instantiations have only 2 (their Jacobians or network buffers would
 * spill or not fit). */
template <int NV, bool WARM, int OCC = 2, bool STAGE = false>
__global__ void __launch_bounds__(128, OCC) ag_k_coop(const DevEphem* __restrict__ Ep, ForceCfg cf, AgBatchArgs A) {
    constexpr int C = 3 * (1 + NV);
    const DevEphem& E = *Ep;
    __shared__ AgCoopShared<NV> S;
    /* Role rotation: warp w of a block runs on sub-partition w % 4 of its SM,
     * and the four roles (planets / relativity / asteroids / asteroids and
     * Sun J2) do unequal FP64 work.  Blocks sharing an SM take successive
     * rotations (a per-SM counter) so that each sub-partition's FP64 pipe
     * serves a mix of roles; within a block everything below uses the
     * logical warp index wid and thread index tid. */
    if (threadIdx.x == 0) {
        int r = 0;
        if (A.sm_slots) {
            unsigned smid;
            asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
            r = atomicAdd(&A.sm_slots[smid & (AG_SM_SLOTS - 1)], 1) & 3;
        }
        S.rot = r;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = ((threadIdx.x >> 5) + S.rot) & 3, tid = (wid << 5) | lane;
    AgCoopTab& Tab = S.tab[0];
    const int slot = blockIdx.x * 32 + lane;
    extern __shared__ __align__(16) unsigned char ag_dyn_smem[];
    AgRecStage* const R =
        STAGE ? reinterpret_cast<AgRecStage*>(ag_dyn_smem + AgCoopDyn<NV, WARM, STAGE>::stage_off) : nullptr;
    AgStageCursor cur;
    constexpr bool wss = AgCoopDyn<NV, WARM>::ws_shared;
    const Ws<C> W{wss ? reinterpret_cast<double*>(ag_dyn_smem + AgCoopDyn<NV, WARM>::warm) : A.ws,
                  wss ? 32 : A.nslots, wss ? lane : slot};
    const long long clk0 = clock64();
    unsigned long long n_acc = 0, n_rej = 0, n_ev = 0, n_it = 0, n_wused = 0, n_wfall = 0, n_tab = 0;
    if (tid == 0) {
        for (int k = 0; k < (NV == 0 ? 8 : 1); k++) S.tab[k].T.status = AG_OK;
        S.stop = 0;
        S.stage_fail = 0;
        if (STAGE) ag_mbar_init(&R->bar);
    }
    /* learned warm start and step logging */
    AgWarmSmem& WS = *reinterpret_cast<AgWarmSmem*>(ag_dyn_smem);
    const bool warm = WARM && A.mlp != nullptr;
    const bool logp = WARM && A.log_x != nullptr;

    while (true) {
        __syncthreads();
        if (tid == 0) S.g = atomicAdd(A.queue, 1);
        __syncthreads();
        const int g = S.g;
        if (g >= A.n_groups) break;
        const int gs = A.grp_size[g], g0 = A.grp_start[g];
        if (S.stop || S.stage_fail) {
            /* run-time budget spent (or a record copy lost): groups still
             * queued are not integrated (state untouched) and say so */
            if (wid == 0 && lane < gs) {
                const int p = A.order[g0 + lane];
                if (A.status) A.status[p] = AG_ST_TIMEOUT;
                if (NV == 0 && A.out_start != nullptr)
                    for (int q = A.out_start[p]; q < A.out_start[p + 1]; q++)
                        for (int k = 0; k < 6; k++) A.out_state[6 * (size_t)q + k] = __longlong_as_double(0x7ff8000000000000LL);
            }
            continue;
        }
        const int pid = lane < gs ? A.order[g0 + lane] : -1;
        double t = A.t0[A.order[g0]], tc = 0.0, dtls = 0.0;
        const double tend = pid >= 0 ? A.t_end[pid] : t;
        double dir;
        {
            const double d = pid >= 0 ? (tend - t) : 0.0;
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
            for (int comp = 0; comp < C; comp++) {
                    if (ag_coop_owner<NV>(comp) != wid) continue;
                double x0, v0;
                if (comp < 3) { x0 = s0[comp]; v0 = s0[3 + comp]; }
                else {
                    const double* vs = A.var_state + ((size_t)pid * NV + (comp - 3) / 3) * 6;
                    x0 = vs[(comp - 3) % 3]; v0 = vs[3 + (comp - 3) % 3];
                }
                W(W_X0, comp) = x0; W(W_V0, comp) = v0; W(W_XC, comp) = 0.0; W(W_VC, comp) = 0.0;
                for (int k = 0; k < 7; k++) {
                    W(W_B + k, comp) = 0.0; W(W_E + k, comp) = 0.0; W(W_BR + k, comp) = 0.0; W(W_ER + k, comp) = 0.0;
                }
            }
            if (A.params) {
                prm[0] = A.params[3 * (size_t)pid]; prm[1] = A.params[3 * (size_t)pid + 1]; prm[2] = A.params[3 * (size_t)pid + 2];
                has_prm = true;
            }
        }
        bool finish_now = live && (tend == t);
        long long steps = 0;
        /* dense output cursor (times sorted along the integration) */
        const bool dense = NV == 0 && A.out_start != nullptr;
        int on = 0, on_end = 0;
        if (dense && live) { on = A.out_start[pid]; on_end = A.out_start[pid + 1]; }
        /* warm start per group: on until its learned steps take longer than
         * its plain probes (every 8th step), timed by thread 0 with clock64
         * from the step's first body table to its converged corrector: the
         * inference's cost against the iterations it saves, where the group
         * iterates until its slowest member has converged */
        long long wg_t_l = 0, wg_t_p = 0, clk_step = 0;
        int wg_n_l = 0, wg_n_p = 0;
        if (tid == 0) S.wg_off = 0;
        /* and per member: on until its learned starts converge in more
         * iterations than its plain probes */
        bool wl_on = warm;
        int wl_sum_l = 0, wl_n_l = 0, wl_sum_p = 0, wl_n_p = 0;
        while (true) {
            /* ---- retire lanes whose particle is complete */
            if (__any_sync(AG_FULL, finish_now)) {
                if (finish_now) {
                    for (int comp = 0; comp < C; comp++) {
                    if (ag_coop_owner<NV>(comp) != wid) continue;
                        const double x1 = W(W_X0, comp) + W(W_XC, comp), v1 = W(W_V0, comp) + W(W_VC, comp);
                        if (dense && comp < 3) {
                            /* times left at a completed particle are its t_end: the end
                             * state; a particle stopped early leaves NaN at the times it
                             * did not reach */
                            const bool done_ok = pstat == AG_ST_OK;
                            const double nan = __longlong_as_double(0x7ff8000000000000LL);
                            for (int q = on; q < on_end; q++) {
                                A.out_state[6 * (size_t)q + comp] = done_ok ? x1 : nan;
                                A.out_state[6 * (size_t)q + 3 + comp] = done_ok ? v1 : nan;
                            }
                        }
                        if (comp < 3) {
                            double* s0 = A.state + 6 * (size_t)pid;
                            s0[comp] = x1; s0[3 + comp] = v1;
                            S.fin[comp][lane] = isfinite(x1) && isfinite(v1);
                        } else {
                            double* vs = A.var_state + ((size_t)pid * NV + (comp - 3) / 3) * 6;
                            vs[(comp - 3) % 3] = x1; vs[3 + (comp - 3) % 3] = v1;
                        }
                    }
                }
                __syncthreads();
                if (finish_now) {
                    const bool finite = S.fin[0][lane] && S.fin[1][lane] && S.fin[2][lane];
                    if (pstat == AG_ST_OK && !finite) pstat = AG_ST_NONFINITE;
                    if (wid == 0 && A.status) A.status[pid] = pstat;
                    live = false;
                    finish_now = false;
                }
            }
            if (!__any_sync(AG_FULL, live)) break;
            /* ---- watchdog (thread 0 decides for the block) */
            if (tid == 0 && (S.stage_fail || (A.watchdog_cycles > 0 && clock64() - clk0 > A.watchdog_cycles))) S.stop = 1;
            __syncthreads();
            if (S.stop) {
                pstat = AG_ST_TIMEOUT;
                finish_now = live;
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
            /* the predictor's coefficients of nodes 1..7, (h_n hstep)^(k+1) over
             * the factorial-like products of IAS15's quadrature, once per step
             * (the group's step is the block's) rather than by every warp at
             * every node of every iteration; read after the next barrier */
            if (tid >= 1 && tid < 8) {
                /* the product rounded on its own, as the oracle forms a node time */
                S.ptn[tid] = t + (tc + __dmul_rn(hstep, ag_ias.h[tid]));
                const double s0 = hstep * ag_ias.h[tid];
                double x = s0 * s0 * 0.5, v = s0;
                S.pcx[tid][0] = s0; S.pcx[tid][1] = x; S.pcv[tid][0] = v;
#pragma unroll
                for (int k = 2; k < 9; k++) { x = x * ag_ias.fx[tid][k]; S.pcx[tid][k] = x; }
#pragma unroll
                for (int k = 1; k < 8; k++) { v = v * ag_ias.fv[tid][k]; S.pcv[tid][k] = v; }
            }

            /* ---- node 0: accelerations at the step start, g from the predicted b */
            if (WARM && tid == 0) clk_step = clock64();
            int bad = ag_coop_table_pass1<STAGE>(E, cf, t, S.scr, Tab, tid, R, cur, &S.stage_fail);
            n_tab++;
            if (live)
                for (int comp = 0; comp < C; comp++)
                    if (ag_coop_owner<NV>(comp) == wid) {
                        S.xs[comp][lane] = W(W_X0, comp); S.vs[comp][lane] = W(W_V0, comp);
                        if constexpr (NV == 0 && !WARM) S.xsf[comp][lane] = ag_f2_of(W(W_X0, comp));
                    }
            bad = __syncthreads_or(bad);
            if (bad) { pstat = S.stage_fail ? AG_ST_TIMEOUT : AG_ST_COVERAGE; finish_now = live; continue; }
            ag_coop_table_pass2(E, cf, t, Tab, S.scr, tid);
            __syncthreads();
            if (cf.geocentric == 1) { ag_coop_rel_geo(E, Tab, tid); __syncthreads(); }
            if (wid == 1 && (cf.forces & AG_F_EIH)) ag_coop_eih_sources(E, cf, Tab.T, lane);
            int fst = AG_OK;
            {
                const double xp[3] = {S.xs[0][lane], S.xs[1][lane], S.xs[2][lane]};
                const double vp[3] = {S.vs[0][lane], S.vs[1][lane], S.vs[2][lane]};
                double acc[3] = {0.0, 0.0, 0.0};
                if (NV > 0) {
                    if (live) {
                        double J[3][6];
                        fst = ag_coop_force_part<true>(wid, Tab, E, cf, xp, vp, has_prm ? prm : nullptr, acc, J);
                        for (int a = 0; a < 3; a++)
                            for (int b = 0; b < 6; b++) S.pj[wid][6 * a + b][lane] = J[a][b];
                    }
                } else if (wid < 2) {
                    if constexpr (NV == 0)
                        ag_coop_force_split01(wid, live, S.seps, lane, Tab, E, cf, xp, vp, has_prm ? prm : nullptr, acc);
                } else if (live) {
                    AgF2 xf3[3];
                    const AgF2* xfp = nullptr;          /* the float-pair position, where it was split */
                    if constexpr (NV == 0 && !WARM) {
                        xf3[0] = S.xsf[0][lane]; xf3[1] = S.xsf[1][lane]; xf3[2] = S.xsf[2][lane];
                        xfp = xf3;
                    }
                    fst = ag_coop_force_part<false, !WARM>(wid, Tab, E, cf, xp, vp, has_prm ? prm : nullptr, acc, nullptr,
                                                           nullptr, nullptr, xfp);
                }
                if (live) {
                    S.pa[wid][0][lane] = acc[0]; S.pa[wid][1][lane] = acc[1]; S.pa[wid][2][lane] = acc[2];
                    if (wid == 0) n_ev++;
                }
            }
            bad = __syncthreads_or(fst != AG_OK);
            if (bad) { pstat = AG_ST_COVERAGE; finish_now = live; continue; }
            if (live) {
                for (int comp = 0; comp < C; comp++) {
                    if (ag_coop_owner<NV>(comp) != wid) continue;
                    double at;
                    if (comp < 3) {
                        at = ((S.pa[3][comp][lane] + S.pa[2][comp][lane]) + S.pa[1][comp][lane]) + S.pa[0][comp][lane];
                    } else {
                        const int q = (comp - 3) / 3, a = (comp - 3) % 3;
                        double Jr[6];
                        for (int b = 0; b < 6; b++)
                            Jr[b] = ((S.pj[3][6 * a + b][lane] + S.pj[2][6 * a + b][lane]) + S.pj[1][6 * a + b][lane]) +
                                    S.pj[0][6 * a + b][lane];
                        const double* dxq = &S.xs[3 + 3 * q][0];
                        const double* dvq = &S.vs[3 + 3 * q][0];
                        double s = Jr[0] * dxq[lane];
                        s = fma(Jr[1], dxq[32 + lane], s); s = fma(Jr[2], dxq[64 + lane], s);
                        s = fma(Jr[3], dvq[lane], s); s = fma(Jr[4], dvq[32 + lane], s); s = fma(Jr[5], dvq[64 + lane], s);
                        at = s;
                    }
                    W(W_A0, comp) = at;
                }
            }
            /* ---- learned warm start: features, BF16 inference, b += kappa y */
            bool w_applied = false, w_probe = false, w_ran = false;
            if constexpr (WARM) {
                if (warm || logp)
                    w_ran = ag_coop_warm_start<NV>(A, W.w, W.ns, W.slot, WS, Tab.T, lane, wid, live, warm,
                                                   wl_on && S.wg_off == 0, hstep, dtls, steps, w_applied, w_probe,
                                                   n_wused, n_wfall);
            }
            if (live) {
                for (int comp = 0; comp < C; comp++) {
                    if (ag_coop_owner<NV>(comp) != wid) continue;
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
            int iters = 1, it_lane = 0;
            double pc_last = 1e300, ma7 = 0.0;
            bool conv = !live;
            bool cov = false;
            while (true) {
                for (int n = 1; n < 8; n++) {
                    const double tn = S.ptn[n];
                    AgCoopTab& TabN = S.tab[NV == 0 ? n : 0];
                    const bool build = NV != 0 || iters == 1;     /* block-uniform */
                    bad = build ? ag_coop_table_pass1<STAGE>(E, cf, tn, S.scr, TabN, tid, R, cur, &S.stage_fail) : 0;
                    n_tab += build ? 1 : 0;
                    if (!conv) {
                        const double* sx = S.pcx[n];
                        const double* sv = S.pcv[n];
                        for (int comp = 0; comp < C; comp++) {
                    if (ag_coop_owner<NV>(comp) != wid) continue;
                            double px = sx[8] * W(W_B + 6, comp);
#pragma unroll
                            for (int j = 5; j >= 0; j--) px = fma(sx[j + 2], W(W_B + j, comp), px);
                            px = fma(sx[1], W(W_A0, comp), px);
                            px = fma(sx[0], W(W_V0, comp), px);
                            const double xn = W(W_X0, comp) + (px + W(W_XC, comp));
                            S.xs[comp][lane] = xn;
                            if constexpr (NV == 0 && !WARM) S.xsf[comp][lane] = ag_f2_of(xn);
                            double pv = sv[7] * W(W_B + 6, comp);
#pragma unroll
                            for (int j = 5; j >= 0; j--) pv = fma(sv[j + 1], W(W_B + j, comp), pv);
                            pv = fma(sv[0], W(W_A0, comp), pv);
                            S.vs[comp][lane] = W(W_V0, comp) + (pv + W(W_VC, comp));
                        }
                    }
                    bad = __syncthreads_or(bad);
                    if (bad) { cov = true; break; }
                    if (build) {
                        ag_coop_table_pass2(E, cf, tn, TabN, S.scr, tid);
                        __syncthreads();
                        if (cf.geocentric == 1) { ag_coop_rel_geo(E, TabN, tid); __syncthreads(); }
                        if (wid == 1 && (cf.forces & AG_F_EIH)) ag_coop_eih_sources(E, cf, TabN.T, lane);
                    }
                    {
                        const double xp[3] = {S.xs[0][lane], S.xs[1][lane], S.xs[2][lane]};
                        const double vp[3] = {S.vs[0][lane], S.vs[1][lane], S.vs[2][lane]};
                        double acc[3] = {0.0, 0.0, 0.0};
                        if (NV > 0) {
                            if (!conv) {
                                double J[3][6];
                                ag_coop_force_part<true>(wid, TabN, E, cf, xp, vp, has_prm ? prm : nullptr, acc, J);
                                for (int a = 0; a < 3; a++)
                                    for (int b = 0; b < 6; b++) S.pj[wid][6 * a + b][lane] = J[a][b];
                            }
                        } else if (wid < 2) {
                            if constexpr (NV == 0)
                                ag_coop_force_split01(wid, !conv, S.seps, lane, TabN, E, cf, xp, vp, has_prm ? prm : nullptr, acc);
                        } else if (!conv) {
                            AgF2 xf3[3];
                            const AgF2* xfp = nullptr;
                            if constexpr (NV == 0 && !WARM) {
                                xf3[0] = S.xsf[0][lane]; xf3[1] = S.xsf[1][lane]; xf3[2] = S.xsf[2][lane];
                                xfp = xf3;
                            }
                            ag_coop_force_part<false, !WARM>(wid, TabN, E, cf, xp, vp, has_prm ? prm : nullptr, acc, nullptr,
                                                             nullptr, nullptr, xfp);
                        }
                        if (!conv) {
                            S.pa[wid][0][lane] = acc[0]; S.pa[wid][1][lane] = acc[1]; S.pa[wid][2][lane] = acc[2];
                            if (wid == 0) n_ev++;
                        }
                    }
                    __syncthreads();
                    if (!conv) {
                        for (int comp = 0; comp < C; comp++) {
                    if (ag_coop_owner<NV>(comp) != wid) continue;
                            double at;
                            if (comp < 3) {
                                at = ((S.pa[3][comp][lane] + S.pa[2][comp][lane]) + S.pa[1][comp][lane]) + S.pa[0][comp][lane];
                            } else {
                                const int q = (comp - 3) / 3, a = (comp - 3) % 3;
                                double Jr[6];
                                for (int b = 0; b < 6; b++)
                                    Jr[b] = ((S.pj[3][6 * a + b][lane] + S.pj[2][6 * a + b][lane]) + S.pj[1][6 * a + b][lane]) +
                                            S.pj[0][6 * a + b][lane];
                                const double* dxq = &S.xs[3 + 3 * q][0];
                                const double* dvq = &S.vs[3 + 3 * q][0];
                                double s = Jr[0] * dxq[lane];
                                s = fma(Jr[1], dxq[32 + lane], s); s = fma(Jr[2], dxq[64 + lane], s);
                                s = fma(Jr[3], dvq[lane], s); s = fma(Jr[4], dvq[32 + lane], s); s = fma(Jr[5], dvq[64 + lane], s);
                                at = s;
                            }
                            double gn = (at - W(W_A0, comp)) * ag_ias.rrinv[n][0];
                            for (int j = 1; j < n; j++) gn = (gn - W(W_G + j - 1, comp)) * ag_ias.rrinv[n][j];
                            const double delta = gn - W(W_G + n - 1, comp);
                            W(W_G + n - 1, comp) = gn;
                            for (int k = 0; k < n - 1; k++) W(W_B + k, comp) = fma(delta, ag_ias.c[n - 1][k], W(W_B + k, comp));
                            W(W_B + n - 1, comp) += delta;
                            if (n == 7 && comp < 3) {
                                const double aa = fabs(at), db = fabs(delta);
                                S.ra[comp][lane] = ag_isnormal_pos(aa) ? aa : 0.0;
                                S.rdb[comp][lane] = ag_isnormal_pos(db) ? db : 0.0;
                            }
                        }
                    }
                }
                if (cov) break;
                __syncthreads();
                if (!conv) {
                    double maxa = 0.0, maxdb = 0.0;
                    for (int k = 0; k < 3; k++) {
                        maxa = ag_max_nonneg(maxa, S.ra[k][lane]);
                        maxdb = ag_max_nonneg(maxdb, S.rdb[k][lane]);
                    }
                    ma7 = maxa;
                    const double pc_err = maxdb / maxa;
                    conv = (pc_err < 1e-16) || (iters > 2 && pc_last <= pc_err) || (iters >= 12);
                    if (conv) { it_lane = iters; if (wid == 0) n_it += (unsigned long long)iters; }
                    else pc_last = pc_err;
                }
                if (__all_sync(AG_FULL, conv)) break;
                iters++;
            }
            if (cov) { pstat = S.stage_fail ? AG_ST_TIMEOUT : AG_ST_COVERAGE; finish_now = live; continue; }
            if (warm && live) {
                if (w_applied) { wl_sum_l += it_lane; wl_n_l++; }
                else if (w_probe) {
                    wl_sum_p += it_lane; wl_n_p++;
                    /* the plain predictor converges faster for this member: fall back */
                    if (wl_n_p >= 4 && wl_n_l >= 8 && (long long)wl_sum_l * wl_n_p > (long long)wl_sum_p * wl_n_l) {
                        wl_on = false;
                        if (wid == 0) n_wfall++;
                    }
                }
            }
            if (warm && !A.warm_no_time_fallback && tid == 0 && S.wg_off == 0) {
                /* the step so far: body tables, forces, the start, the corrector */
                const long long dt_clk = clock64() - clk_step;
                const bool probe = (steps & 7) == 7;
                if (w_ran) { wg_t_l += dt_clk; wg_n_l++; }
                else if (probe) { wg_t_p += dt_clk; wg_n_p++; }
                /* the group's learned steps take longer than its plain probes: the
                 * plain predictor for the rest of the group */
                if (wg_n_p >= 3 && wg_n_l >= 12 && (double)wg_t_l / wg_n_l > (double)wg_t_p / wg_n_p) {
                    S.wg_off = 1;
                    n_wfall++;
                }
            }
            /* ---- step-size control: each lane's choice, the group takes the smallest */
            if (live && ag_coop_pcomp<NV>(wid) >= 0) {
                const double bb = fabs(W(W_B + 6, ag_coop_pcomp<NV>(wid)));
                S.rb6[ag_coop_pcomp<NV>(wid)][lane] = ag_isnormal_pos(bb) ? bb : 0.0;
            }
            __syncthreads();
            double dt_new_l = 1e300, dt_nocap_l = 1e300;
            bool rej_l = false;
            /* warp 0 forms each lane's proposal (the power and the divisions
             * are FP64 work that every warp would repeat); the others read it */
            if (wid == 0) {
                if (A.epsilon > 0.0 && live) {
                    double mb = 0.0;
                    for (int k = 0; k < 3; k++) mb = ag_max_nonneg(mb, S.rb6[k][lane]);
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
                S.sdn[lane] = dt_new_l; S.sdc[lane] = dt_nocap_l; S.srej[lane] = rej_l ? 1 : 0;
            }
            __syncthreads();
            if (wid != 0) { dt_new_l = S.sdn[lane]; dt_nocap_l = S.sdc[lane]; rej_l = S.srej[lane] != 0; }
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
                if (live) {
                    if (wid == 0) n_rej++;
                    for (int comp = 0; comp < C; comp++) {
                    if (ag_coop_owner<NV>(comp) != wid) continue;
                        if (dtls != 0.0) ag_predict_next_comp<C>(W, comp, dt_new / dtls);
                        else
                            for (int k = 0; k < 7; k++) { W(W_B + k, comp) = 0.0; W(W_E + k, comp) = 0.0; }
                    }
                }
                dt = dt_new;
                continue;
            }
            /* ---- log (features, target) pairs of accepted steps: target =
             * (b_conv - b_pred) / kappa with b_pred = e + (br - er), the plain prediction */
            if (logp) {
                const bool lg = live && WS.valid[lane] && (steps % A.log_every) == 0;
                if (lg && ag_coop_pcomp<NV>(wid) >= 0)
                    for (int k = 0; k < 7; k++) {
                        const int c = ag_coop_pcomp<NV>(wid);
                        const double bp = W(W_E + k, c) + (W(W_BR + k, c) - W(W_ER + k, c));
                        WS.tgt[k][c][lane] = (float)((W(W_B + k, c) - bp) / WS.kappa[k][lane]);
                    }
                __syncthreads();
                if (lg && wid == 0) {
                    bool fin = true;
                    for (int k = 0; k < 7; k++)
                        for (int c = 0; c < 3; c++) fin = fin && isfinite(WS.tgt[k][c][lane]) && fabsf(WS.tgt[k][c][lane]) < 1e6f;
                    if (fin) {
                        const int row = atomicAdd(A.log_count, 1);
                        if (row < A.log_cap) {
                            for (int i = 0; i < AG_MLP_IN; i++) A.log_x[(size_t)row * AG_MLP_IN + i] = WS.xf[lane][i];
                            for (int k = 0; k < 7; k++)
                                for (int c = 0; c < 3; c++) A.log_t[(size_t)row * AG_MLP_OUT + 3 * k + c] = WS.tgt[k][c][lane];
                        }
                    }
                }
            }
            /* ---- dense output: states at the output times this step covers,
             * from the step's polynomial (the interpolation of ASSIST's
             * assist_interpolate, src/assist.c:556-597: s- and sv-coefficients
             * built by the same recurrences, x from the step-start x, v, a, b) */
            if (dense && live) {
                const double tstep_end = (t + tc) + hstep;
                while (on < on_end && dir * (A.out_t[on] - tstep_end) <= 0.0 && !(last && A.out_t[on] == tend)) {
                    const double h = ((A.out_t[on] - t) - tc) / hstep;
                    double s[9], sv[8];
                    s[0] = hstep * h;
                    s[1] = s[0] * s[0] / 2.;
                    s[2] = s[1] * h / 3.;
                    s[3] = s[2] * h / 2.;
                    s[4] = 3. * s[3] * h / 5.;
                    s[5] = 2. * s[4] * h / 3.;
                    s[6] = 5. * s[5] * h / 7.;
                    s[7] = 3. * s[6] * h / 4.;
                    s[8] = 7. * s[7] * h / 9.;
                    sv[0] = hstep * h;
                    sv[1] = sv[0] * h / 2.;
                    sv[2] = 2. * sv[1] * h / 3.;
                    sv[3] = 3. * sv[2] * h / 4.;
                    sv[4] = 4. * sv[3] * h / 5.;
                    sv[5] = 5. * sv[4] * h / 6.;
                    sv[6] = 6. * sv[5] * h / 7.;
                    sv[7] = 7. * sv[6] * h / 8.;
                    if (ag_coop_pcomp<NV>(wid) >= 0) {
                        const int c = ag_coop_pcomp<NV>(wid);
                        const double b0 = W(W_B + 0, c), b1 = W(W_B + 1, c), b2 = W(W_B + 2, c), b3 = W(W_B + 3, c),
                                     b4 = W(W_B + 4, c), b5 = W(W_B + 5, c), b6 = W(W_B + 6, c);
                        const double a0 = W(W_A0, c), v0 = W(W_V0, c);
                        A.out_state[6 * (size_t)on + c] =
                            W(W_X0, c) + (s[8] * b6 + s[7] * b5 + s[6] * b4 + s[5] * b3 + s[4] * b2 + s[3] * b1 +
                                          s[2] * b0 + s[1] * a0 + s[0] * v0);
                        A.out_state[6 * (size_t)on + 3 + c] = v0 + sv[7] * b6 + sv[6] * b5 + sv[5] * b4 + sv[4] * b3 +
                                                              sv[3] * b2 + sv[2] * b1 + sv[1] * b0 + sv[0] * a0;
                    }
                    on++;
                }
            }
            /* ---- accept */
            if (live) {
                if (wid == 0) n_acc++;
                const double h2 = hstep * hstep;
                for (int comp = 0; comp < C; comp++) {
                    if (ag_coop_owner<NV>(comp) != wid) continue;
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
                    ag_predict_next_comp<C>(W, comp, dt_new / hstep);
                }
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
    if (wid == 0) {
        atomicAdd(&A.counters[0], n_acc);
        atomicAdd(&A.counters[1], n_rej);
        atomicAdd(&A.counters[2], n_ev);
        atomicAdd(&A.counters[3], n_it);
        atomicAdd(&A.counters[4], n_wused);
        atomicAdd(&A.counters[5], n_wfall);
        if (tid == 0) atomicAdd(&A.counters[6], n_tab);   /* body tables, one per block and node time */
    }
    /* a copy that did not complete in time: wait for it once more (bounded)
     * before the block's shared memory is released */
    if (STAGE && tid == 0 && S.stage_fail) ag_mbar_wait(&R->bar, cur.phase ^ 1u);
}

/* Opt the kernel in to its dynamic shared memory (above the 48 KB default). */
template <int NV, bool WARM, int OCC, bool STAGE = false>
static int ag_coop_dyn_attr() {
    if (AgCoopDyn<NV, WARM, STAGE>::bytes == 0) return 0;
    return (int)cudaFuncSetAttribute(ag_k_coop<NV, WARM, OCC, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)AgCoopDyn<NV, WARM, STAGE>::bytes);
}

template <int NV, bool WARM, int OCC, bool STAGE = false>
static int ag_coop_blocks_per_sm() {
    int bps = 0;
    if (ag_coop_dyn_attr<NV, WARM, OCC, STAGE>() == 0)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ag_k_coop<NV, WARM, OCC, STAGE>, 128,
                                                      AgCoopDyn<NV, WARM, STAGE>::bytes);
    return bps;
}

/* Slots (32 per resident block) of the plain (nv = 0: occ 2 or 3, stage
 * only with occ 2) or variational (nv = 6) kernel, or of their learned
 * warm-start builds (warm), on the current device. */
int ag_coop_max_slots(int nv, int occ, int stage, int warm) {
    int dev = 0, sms = 0, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (nv == 6) bps = warm ? ag_coop_blocks_per_sm<6, true, 2>() : ag_coop_blocks_per_sm<6, false, 2>();
    else if (warm) bps = ag_coop_blocks_per_sm<0, true, 2>();
    else if (occ == 3) bps = ag_coop_blocks_per_sm<0, false, 3>();
    else if (stage) bps = ag_coop_blocks_per_sm<0, false, 2, true>();
    else bps = ag_coop_blocks_per_sm<0, false, 2>();
    if (bps < 1) bps = 1;
    return sms * bps * 32;
}

int ag_launch_coop(const DevEphem& E, const ForceCfg& c, const AgBatchArgs& a, int nv, int occ, int stage,
                   cudaStream_t s) {
    int e = ag_ias_tables_init();
    if (e) return e;
    const int blocks = (a.nslots + 31) / 32;
    if (nv == 6 && (a.mlp || a.log_x)) {
        if ((e = ag_coop_dyn_attr<6, true, 2>())) return e;
        ag_k_coop<6, true, 2><<<blocks, 128, AgCoopDyn<6, true>::bytes, s>>>(E.self_dev, c, a);
    } else if (nv == 6) {
        ag_k_coop<6, false, 2><<<blocks, 128, AgCoopDyn<6, false>::bytes, s>>>(E.self_dev, c, a);
    } else if (a.mlp || a.log_x) {
        if ((e = ag_coop_dyn_attr<0, true, 2>())) return e;
        ag_k_coop<0, true, 2><<<blocks, 128, AgCoopDyn<0, true>::bytes, s>>>(E.self_dev, c, a);
    } else if (occ == 3) {
        if ((e = ag_coop_dyn_attr<0, false, 3>())) return e;
        ag_k_coop<0, false, 3><<<blocks, 128, AgCoopDyn<0, false>::bytes, s>>>(E.self_dev, c, a);
    } else if (stage) {
        if ((e = ag_coop_dyn_attr<0, false, 2, true>())) return e;
        ag_k_coop<0, false, 2, true><<<blocks, 128, AgCoopDyn<0, false, true>::bytes, s>>>(E.self_dev, c, a);
    } else {
        if ((e = ag_coop_dyn_attr<0, false, 2>())) return e;
        ag_k_coop<0, false, 2><<<blocks, 128, AgCoopDyn<0, false>::bytes, s>>>(E.self_dev, c, a);
    }
    return (int)cudaGetLastError();
}

/* What a launch of this kernel sets up on its first use on a device (the
 * IAS15 tables, the shared-memory opt-ins of every build), done ahead of a
 * stream capture. */
int ag_coop_ready(void) {
    int e = ag_ias_tables_init();
    if (!e) e = ag_coop_dyn_attr<0, false, 2>();
    if (!e) e = ag_coop_dyn_attr<0, false, 3>();
    if (!e) e = ag_coop_dyn_attr<0, false, 2, true>();
    if (!e) e = ag_coop_dyn_attr<0, true, 2>();
    if (!e) e = ag_coop_dyn_attr<6, true, 2>();
    return e;
}
