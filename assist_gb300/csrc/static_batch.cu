/*
 * static_batch.cu -- the batched IAS15 entry point that allocates nothing.
 *
 * assist_gb300_integrate_batch_device_static runs the independent-step
 * batched IAS15 kernel (ag_k_batch<0>, the kernel behind
 * assist_gb300_integrate_batch_device with group_steps = 0) with all of its
 * scratch in one file-scope __device__ array of fixed size instead of device
 * memory from cudaMalloc:
 *
 *   bytes [0, 256)           queue position (int at 0) and the eight step
 *                            counters (unsigned long long at 64); both must
 *                            start at zero and are cleared by a kernel at the
 *                            start of every call
 *   bytes [256, 256 + 4n)    the queue order (particle i at position i),
 *                            written by the same kernel
 *   the rest (256-aligned)   the per-slot IAS15 workspace, 40 x 3 doubles a
 *                            slot; the kernel initialises a slot's fields
 *                            each time it takes a particle, so it needs no
 *                            clearing
 *
 * Nothing here calls cudaMalloc, cudaFree, an event or stream constructor or
 * any other allocating routine, on the device or on the host.  The scratch
 * address comes from cudaGetSymbolAddress, once per device, with that device
 * current.
 */
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "assist.h"
#include "device_forces.cuh"
#include "internal.h"

#define AG_STATIC_HEADER_BYTES 256
#define AG_STATIC_WS_DOUBLES_PER_SLOT (40 * 3)

static_assert(ASSIST_GB300_STATIC_SCRATCH_BYTES % 256 == 0, "scratch size must be a multiple of 256 bytes");
static_assert(AG_STATIC_HEADER_BYTES + 4ull * ASSIST_GB300_STATIC_MAX_PARTICLES + 256ull * AG_STATIC_WS_DOUBLES_PER_SLOT * 8 <=
                  ASSIST_GB300_STATIC_SCRATCH_BYTES,
              "scratch must hold the order of the largest batch and at least 256 workspace slots");

static __device__ __align__(256) unsigned char ag_static_scratch[ASSIST_GB300_STATIC_SCRATCH_BYTES];

/* Clear the queue position and the counters; write the identity queue order. */
__global__ void ag_k_static_reset(unsigned char* scratch, int n) {
    int* queue = reinterpret_cast<int*>(scratch);
    unsigned long long* counters = reinterpret_cast<unsigned long long*>(scratch + 64);
    int* order = reinterpret_cast<int*>(scratch + AG_STATIC_HEADER_BYTES);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *queue = 0;
    if (i < 8) counters[i] = 0ull;
    for (int k = i; k < n; k += gridDim.x * blockDim.x) order[k] = k;
}

/* Per-device scratch address (looked up once per device). */
static void* g_static_ptr[64];

static int ag_static_scratch_address(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return ag_cuda_check(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) {
        ag_set_error("device ordinal out of range for the static scratch table");
        return 1;
    }
    if (!g_static_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, ag_static_scratch);
        if (e != cudaSuccess) return ag_cuda_check(e, "cudaGetSymbolAddress(static scratch)");
        g_static_ptr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_static_ptr[dev]);
    return 0;
}

extern "C" int assist_gb300_integrate_batch_device_static(const struct assist_ephem* e,
                                                         const struct assist_gb300_options* o, int n,
                                                         const double* d_t0, const double* d_t_end, double* d_state,
                                                         const double* d_params, int* d_status, void* stream,
                                                         struct assist_gb300_batch_stats* stats) {
    if (!o) { ag_set_error("options are required"); return ASSIST_ERROR_N; }
    if (n < 0) {
        ag_set_error("static-scratch batch: the particle count must not be negative");
        return ASSIST_ERROR_N;
    }
    if (n > ASSIST_GB300_STATIC_MAX_PARTICLES) {
        char msg[160];
        std::snprintf(msg, sizeof(msg), "static-scratch batch: %d particles requested, at most %d fit in its %d MiB scratch",
                      n, ASSIST_GB300_STATIC_MAX_PARTICLES, ASSIST_GB300_STATIC_SCRATCH_BYTES >> 20);
        ag_set_error(msg);
        return ASSIST_ERROR_N;
    }
    if (o->warm_start) {
        ag_set_error("static-scratch batch: the learned warm start needs the allocating entry points");
        return ASSIST_ERROR_N;
    }
    if (n == 0) { if (stats) std::memset(stats, 0, sizeof(*stats)); return ASSIST_SUCCESS; }
    if (!(o->dt0 > 0) || !(o->epsilon >= 0)) { ag_set_error("dt0 must be > 0 and epsilon >= 0"); return ASSIST_ERROR_N; }
    /* the ephemeris's device view as it stands: this path neither allocates
     * nor uploads one (an ephemeris edited since its last ordinary device
     * call is refused) */
    DevEphem D;
    int st = ag_ephem_device_current(e, &D);
    if (st) return st;
    unsigned char* scratch = nullptr;
    if (ag_static_scratch_address(&scratch)) return ASSIST_ERROR_EPHEM_FILE;
    const size_t ws_off = ((AG_STATIC_HEADER_BYTES + 4 * (size_t)n + 255) / 256) * 256;
    const size_t slot_bytes = sizeof(double) * AG_STATIC_WS_DOUBLES_PER_SLOT;
    long long nslots = (long long)((ASSIST_GB300_STATIC_SCRATCH_BYTES - ws_off) / slot_bytes);
    const int tpb = 128;
    const long long dev_slots = ag_batch_max_slots(0, tpb);
    if (nslots > dev_slots) nslots = dev_slots;
    if (nslots > n) nslots = n;
    cudaStream_t s = (cudaStream_t)stream;
    ag_k_static_reset<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, s>>>(scratch, n);
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return ag_cuda_check(le, "static scratch reset") ? ASSIST_ERROR_EPHEM_FILE : 0;
    AgBatchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = n;
    a.nslots = (int)nslots;
    a.order = reinterpret_cast<const int*>(scratch + AG_STATIC_HEADER_BYTES);
    a.queue = reinterpret_cast<int*>(scratch);
    a.counters = reinterpret_cast<unsigned long long*>(scratch + 64);
    a.ws = reinterpret_cast<double*>(scratch + ws_off);
    a.t0 = d_t0; a.t_end = d_t_end; a.state = d_state; a.params = d_params; a.var_state = nullptr;
    a.status = d_status;
    a.epsilon = o->epsilon; a.min_dt = o->min_dt; a.dt0 = o->dt0; a.max_steps = o->max_steps;
    a.dt_floor = o->dt_floor;
    double wd = 300.0;
    if (const char* w = getenv("ASSIST_GB300_WATCHDOG_S")) wd = atof(w);
    a.watchdog_cycles = wd > 0 ? (long long)(wd * 2.1e9) : 0;
    const ForceCfg c = ag_make_cfg(o);
    const int rc = ag_launch_batch(D, c, a, 0, tpb, s);
    if (rc) { ag_cuda_check((cudaError_t)rc, "static-scratch batch kernel launch"); return ASSIST_ERROR_EPHEM_FILE; }
    if (stats) {
        unsigned long long cnt[8];
        if (ag_cuda_check(cudaMemcpyAsync(cnt, a.counters, sizeof(cnt), cudaMemcpyDeviceToHost, s), "read counters") ||
            ag_cuda_check(cudaStreamSynchronize(s), "static-scratch batch kernel"))
            return ASSIST_ERROR_EPHEM_FILE;
        stats->steps_accepted = (long long)cnt[0];
        stats->steps_rejected = (long long)cnt[1];
        stats->force_evals = (long long)cnt[2];
        stats->pc_iterations = (long long)cnt[3];
        stats->warm_start_used = (long long)cnt[4];
        stats->warm_start_fallback = (long long)cnt[5];
        stats->tables_built = (long long)cnt[6];
        stats->kernel_ms = -1.0;   /* not timed: timing would need events */
    }
    return ASSIST_SUCCESS;
}
