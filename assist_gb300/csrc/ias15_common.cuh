/*
 * ias15_common.cuh -- device pieces shared by the batched IAS15 kernels
 * (kernels_ias15.cu: independent and warp-grouped; kernels_coop.cu:
 * block-cooperative): per-particle status codes, the Gauss-Radau tables in
 * constant memory, the slot-major workspace accessor and the polynomial
 * shift that predicts the next step's b.  Each translation unit that
 * includes it holds its own copy of the constant tables and uploads it on
 * its first launch on a device.
 */
#ifndef ASSIST_GB300_IAS15_COMMON_CUH
#define ASSIST_GB300_IAS15_COMMON_CUH

#include <cuda_runtime.h>

#include "ias15_constants.h"

#define AG_ST_OK 0
#define AG_ST_COVERAGE 1
#define AG_ST_NONFINITE 2
#define AG_ST_BUDGET 3
#define AG_ST_UNDERFLOW 4
#define AG_ST_TIMEOUT 5

struct IasTables {
    double h[8];
    double rrinv[8][8];      /* 1/(h_n - h_j) */
    double c[7][7];          /* b_k += c[j][k] * dg_j, k < j */
    double d[7][7];          /* g_j = b_j + sum_{k>j} d[j][k] b_k */
    double fx[8][9];         /* position predictor ratios: s_k = s_(k-1) * fx[n][k] */
    double fv[8][8];         /* velocity predictor ratios */
};
static __constant__ IasTables ag_ias;     /* one copy per translation unit, uploaded by its own init */

static bool g_tables_ready[64];

/* Build the IAS15 tables on the host (same expressions as the oracle's
 * predictor: h*(k-1)/(k+1) and h*k/(k+1)). */
static int ag_ias_tables_init(void) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && g_tables_ready[dev]) return 0;
    IasTables T;
    const double h[8] = IAS15_H_INIT;
    const double rr[28] = IAS15_RR_INIT;
    const double cc[21] = IAS15_C_INIT;
    const double dd[21] = IAS15_D_INIT;
    for (int n = 0; n < 8; n++) T.h[n] = h[n];
    for (int n = 0; n < 8; n++) for (int j = 0; j < 8; j++) T.rrinv[n][j] = 0.0;
    int q = 0;
    for (int n = 1; n < 8; n++) for (int j = 0; j < n; j++) T.rrinv[n][j] = 1.0 / rr[q++];
    for (int j = 0; j < 7; j++) for (int k = 0; k < 7; k++) { T.c[j][k] = 0.0; T.d[j][k] = 0.0; }
    q = 0;
    for (int j = 1; j < 7; j++) for (int k = 0; k < j; k++) T.c[j][k] = cc[q++];
    for (int j = 0; j < 7; j++) T.c[j][j] = 1.0;
    q = 0;
    for (int j = 0; j < 6; j++) for (int k = j + 1; k < 7; k++) T.d[j][k] = dd[q++];
    for (int j = 0; j < 7; j++) T.d[j][j] = 1.0;
    for (int n = 0; n < 8; n++) {
        T.fx[n][0] = T.fx[n][1] = 0.0;
        for (int k = 2; k < 9; k++) T.fx[n][k] = h[n] * (double)(k - 1) / (double)(k + 1);
        T.fv[n][0] = 0.0;
        for (int k = 1; k < 8; k++) T.fv[n][k] = h[n] * (double)k / (double)(k + 1);
    }
    cudaError_t e = cudaMemcpyToSymbol(ag_ias, &T, sizeof(T));
    if (e != cudaSuccess) return (int)e;
    if (dev >= 0 && dev < 64) g_tables_ready[dev] = true;
    return 0;
}

/* workspace fields */
enum { W_X0 = 0, W_V0, W_A0, W_XC, W_VC, W_B, W_G = W_B + 7, W_E = W_G + 7, W_BR = W_E + 7, W_ER = W_BR + 7, W_NF = W_ER + 7 };


template <int C>
struct Ws {
    double* w;
    int ns, slot;
    __device__ __forceinline__ double& operator()(int f, int comp) const { return w[((size_t)f * C + comp) * ns + slot]; }
};

/* b, e from the last accepted step's br, er with step ratio q (the shift of
 * the acceleration polynomial to the new step). */
template <int C>
__device__ __forceinline__ void ag_predict_next(const Ws<C>& W, double ratio) {
    if (ratio > 20.0) {
        for (int comp = 0; comp < C; comp++)
            for (int k = 0; k < 7; k++) { W(W_E + k, comp) = 0.0; W(W_B + k, comp) = 0.0; }
        return;
    }
    double q[8];
    q[1] = ratio;
    for (int k = 2; k < 8; k++) q[k] = q[k - 1] * ratio;
    constexpr double binom[8][8] = {
        {1, 0, 0, 0, 0, 0, 0, 0}, {1, 1, 0, 0, 0, 0, 0, 0}, {1, 2, 1, 0, 0, 0, 0, 0}, {1, 3, 3, 1, 0, 0, 0, 0},
        {1, 4, 6, 4, 1, 0, 0, 0}, {1, 5, 10, 10, 5, 1, 0, 0}, {1, 6, 15, 20, 15, 6, 1, 0}, {1, 7, 21, 35, 35, 21, 7, 1}};
#pragma unroll 1
    for (int comp = 0; comp < C; comp++) {
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
}


#ifndef AG_FULL
#define AG_FULL 0xffffffffu
#endif

__device__ __forceinline__ double warp_min(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(AG_FULL, v, o));
    return v;
}

#endif
