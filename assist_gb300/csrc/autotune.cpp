/*
 * autotune.cpp -- build selection for the block-cooperative batched IAS15.
 *
 * The default batched kernel comes in three builds that run each group's
 * arithmetic identically and differ only in how a block uses the SM: two
 * resident blocks per SM (242 registers), three (168 registers, a few
 * spills), and two with the active .440 record staged in shared memory by
 * bulk copies.  Which is fastest depends on the batch: three blocks win when
 * there are many groups per block, two when a few long groups set the time.
 * assist_gb300_autotune_device times every build on the caller's own batch
 * (the whole batch: a sample would not keep its groups per resident block)
 * and records the fastest under a signature of the batch -- device, group
 * count, mean and longest integration length, share of non-gravitational
 * particles, force model, planets format -- in memory and in a text file
 * (ASSIST_GB300_TUNE_CACHE, default ~/.cache/assist_gb300/tune.txt; an empty
 * value keeps it in memory only).  Later calls in automatic mode
 * (blocks_per_sm = 0, ephem_staging = 0) whose batch has a recorded
 * signature use the recorded build; others use the group-count rule.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <sys/stat.h>

#include "../../include/assist.h"
#include "internal.h"

static std::mutex g_tune_mu;
static std::map<std::string, int> g_tune;      /* signature -> build (2, 3, 4; 5 the learned start) */
static bool g_tune_loaded = false;
static std::string g_tune_last_key;            /* signature of the last plain block-cooperative batch */

static std::string ag_tune_path() {
    const char* p = getenv("ASSIST_GB300_TUNE_CACHE");
    if (p) return std::string(p);
    const char* h = getenv("HOME");
    if (!h || !*h) return std::string();
    return std::string(h) + "/.cache/assist_gb300/tune.txt";
}

static void ag_tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const std::string path = ag_tune_path();
    if (path.empty()) return;
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return;
    char line[1024];
    while (std::fgets(line, sizeof(line), f)) {
        char key[900];
        int choice = 0;
        if (std::sscanf(line, "%899s %d", key, &choice) == 2 && (choice >= 2 && choice <= 5))
            g_tune[key] = choice;
    }
    std::fclose(f);
}

static void ag_tune_store_locked(const std::string& key, int choice, const double* ms, int nc) {
    g_tune[key] = choice;
    const std::string path = ag_tune_path();
    if (path.empty()) return;
    std::string dir = path.substr(0, path.find_last_of('/'));
    for (size_t k = 1; k < dir.size(); k++)
        if (dir[k] == '/') { dir[k] = '\0'; mkdir(dir.c_str(), 0755); dir[k] = '/'; }
    if (!dir.empty()) mkdir(dir.c_str(), 0755);
    FILE* f = std::fopen(path.c_str(), "a");
    if (!f) return;
    std::fprintf(f, "%s %d", key.c_str(), choice);
    for (int k = 0; k < nc; k++) std::fprintf(f, " %.3f", ms[k]);
    std::fprintf(f, "\n");
    std::fclose(f);
}

std::string ag_tune_key(int n_groups, int n, const double* t0, const double* te, const unsigned char* has_ng,
                        int forces, int gr_eih_sources, int geocentric, int planets_spk) {
    int dev = 0;
    cudaGetDevice(&dev);
    static std::string dev_tag[64];            /* device name and SM count, looked up once per device */
    if (dev < 0 || dev >= 64) dev = 63;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (dev_tag[dev].empty()) {
            cudaDeviceProp prop;
            std::memset(&prop, 0, sizeof(prop));
            cudaGetDeviceProperties(&prop, dev);
            dev_tag[dev] = std::string(prop.name) + "/sm" + std::to_string(prop.multiProcessorCount);
        }
    }
    double sum = 0.0, mx = 0.0;
    long long ng = 0;
    for (int i = 0; i < n; i++) {
        const double L = std::fabs(te[(size_t)i] - t0[(size_t)i]);
        sum += L;
        if (L > mx) mx = L;
        if (has_ng && has_ng[(size_t)i]) ng++;
    }
    const double mean = n > 0 ? sum / n : 0.0;
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s|g%d|L%d|R%d|ng%d|f%x|eih%d|geo%d|%s", dev_tag[dev].c_str(),
                  (int)std::lround(4.0 * std::log2(std::max(n_groups, 1))),
                  (int)std::lround(2.0 * std::log2(std::max(mean, 1e-3))),
                  (int)std::lround(2.0 * std::log2(std::max(mx / std::max(mean, 1e-9), 1.0))),
                  (int)std::lround(10.0 * (n > 0 ? (double)ng / n : 0.0)), forces, gr_eih_sources, geocentric,
                  planets_spk ? "spk" : "440");
    std::string key(buf);
    for (auto& ch : key)
        if (ch == ' ') ch = '_';
    return key;
}

int ag_tune_lookup(const std::string& key) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    ag_tune_load_locked();
    auto it = g_tune.find(key);
    return it == g_tune.end() ? 0 : it->second;
}

void ag_tune_note(const std::string& key) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_last_key = key;
}

extern "C" int assist_gb300_autotune_device(const struct assist_ephem* e, const struct assist_gb300_options* o, int n,
                                            const double* d_t0, const double* d_t_end, const double* d_state,
                                            const double* d_params, int n_var, const double* d_var_state,
                                            void* stream, struct assist_gb300_tune_result* res) {
    if (!o || !res || n < 0 || (n > 0 && (!d_t0 || !d_t_end || !d_state)) || (n_var != 0 && n_var != 6) ||
        (n_var && n > 0 && !d_var_state)) {
        ag_set_error("autotune: options, result, n_var 0 or 6 and the batch's device arrays are required");
        return ASSIST_ERROR_N;
    }
    std::memset(res, 0, sizeof(*res));
    if (n == 0) return ASSIST_SUCCESS;
    if (o->group_steps != 2 || (n_var && !o->warm_start)) {
        ag_set_error("autotune: it chooses between the builds of the block-cooperative kernel (group_steps = 2); "
                     "with variational particles only between the plain and the learned warm start");
        return ASSIST_ERROR_N;
    }
    /* candidates: the plain builds (two blocks per SM; without variational
     * particles also three, and two with the staged record for .440 planets),
     * then the learned warm start when asked for */
    const bool spk = e && e->spk_planets;
    int cand[4], nc = 0;
    cand[nc++] = 2;
    if (!n_var) {
        cand[nc++] = 3;
        if (!spk) cand[nc++] = 4;
    }
    if (o->warm_start) cand[nc++] = 5;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nvd = (size_t)n * (size_t)n_var * 6;
    double* d_st = nullptr;
    double* d_var = nullptr;
    int* d_status = nullptr;
    if (ag_cuda_check(cudaMalloc(&d_st, sizeof(double) * 6 * (size_t)n), "cudaMalloc(autotune state)") ||
        (nvd && ag_cuda_check(cudaMalloc(&d_var, sizeof(double) * nvd), "cudaMalloc(autotune variational state)")) ||
        ag_cuda_check(cudaMalloc(&d_status, sizeof(int) * (size_t)n), "cudaMalloc(autotune status)")) {
        if (d_st) cudaFree(d_st);
        if (d_var) cudaFree(d_var);
        return ASSIST_ERROR_EPHEM_FILE;
    }
    double best = 1e300;
    int rc = ASSIST_SUCCESS;
    std::string key;
    for (int k = 0; k < nc && rc == ASSIST_SUCCESS; k++) {
        struct assist_gb300_options oc = *o;
        oc.blocks_per_sm = cand[k] == 3 ? 3 : 2;
        oc.ephem_staging = cand[k] == 4 ? 1 : 2;
        oc.warm_start = cand[k] == 5 ? 2 : 0;
        double ms = 1e300;
        for (int rep = 0; rep < 2; rep++) {
            if (ag_cuda_check(cudaMemcpyAsync(d_st, d_state, sizeof(double) * 6 * (size_t)n, cudaMemcpyDeviceToDevice, s),
                              "autotune state copy") ||
                (nvd && ag_cuda_check(cudaMemcpyAsync(d_var, d_var_state, sizeof(double) * nvd, cudaMemcpyDeviceToDevice, s),
                                      "autotune state copy"))) {
                rc = ASSIST_ERROR_EPHEM_FILE;
                break;
            }
            struct assist_gb300_batch_stats st;
            rc = assist_gb300_integrate_batch_device(e, &oc, n, d_t0, d_t_end, d_st, d_params, n_var, d_var, d_status,
                                                     s, &st);
            if (rc != ASSIST_SUCCESS) break;
            ms = std::min(ms, st.kernel_ms);
        }
        res->candidate[k] = cand[k];
        res->kernel_ms[k] = ms;
        if (ms < best) { best = ms; res->chosen = cand[k]; }
        /* the signature is recorded as the call being tuned forms it: plain
         * without warm_start; with it, as the learned run formed it */
        if (rc == ASSIST_SUCCESS && (k == 0 || cand[k] == 5)) {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            key = g_tune_last_key;
        }
    }
    res->n_candidates = nc;
    cudaFree(d_st);
    if (d_var) cudaFree(d_var);
    cudaFree(d_status);
    if (rc != ASSIST_SUCCESS) return rc;
    if (key.empty()) {
        ag_set_error("autotune: no batch signature was formed");
        return ASSIST_ERROR_N;
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    ag_tune_load_locked();
    ag_tune_store_locked(key, res->chosen, res->kernel_ms, nc);
    std::snprintf(res->signature, sizeof(res->signature), "%s", key.c_str());
    return ASSIST_SUCCESS;
}
