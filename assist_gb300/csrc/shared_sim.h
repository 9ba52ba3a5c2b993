/*
 * shared_sim.h -- host interface of the shared-step device IAS15 (kernels_shared.cu).
 */
#ifndef ASSIST_GB300_SHARED_SIM_H
#define ASSIST_GB300_SHARED_SIM_H

#include "../../include/rebound.h"
#include "internal.h"

struct ShIntegrateOut {
    long long accepted = 0, rejected = 0, evals = 0, iterations = 0;
    int status = 0;               /* ASSIST status of the force model, -1 step budget */
    long long max_steps = 0;
    double dt_last_done = 0.0;
    bool dense = false;           /* copy the last step's start state and b */
    double* dense_x0 = nullptr;
    double* dense_v0 = nullptr;
    double* dense_a0 = nullptr;
    double* dense_b[7] = {nullptr};
};

int ag_shared_forces(AgSharedSim* s, const DevEphem& E, const ForceCfg& c, struct reb_simulation* r,
                     const double* params, int* status_out);
int ag_shared_integrate(AgSharedSim* s, const DevEphem& E, const ForceCfg& c, struct reb_simulation* r,
                        const double* params, double tmax, ShIntegrateOut* out);
/* the n particles at fraction h of the last step (size dt) on the device, into out[] (0, or 1: no such step) */
int ag_shared_interpolate(AgSharedSim* s, int n, double dt, double h, struct reb_particle* out);

#endif
