/*
 * mlp.cuh -- the learned IAS15 warm start on the device: the features of a
 * particle's step, BF16 tensor-core inference for a group of 32 particles,
 * and the parameter layout shared with the training kernels.
 *
 * Network (no counterpart in the reference; ASSIST uses IAS15's own
 * predictor): 32 features -> 256 -> 256 -> 21, tanh-form GELU, weights kept
 * [out][in].  Training runs in FP32 (kernels_mlp.cu); inference reads BF16
 * copies of the weights and accumulates in FP32 on the tensor cores with
 * mma.sync m16n8k16 (one group is only 32 rows, below tcgen05's smallest
 * tile, and runs inside the FP64-bound IAS15 kernel).
 *
 * What it predicts.  IAS15's predictor sets b = e + (br - er): the shifted
 * polynomial of the last step plus the last step's correction.  The network
 * predicts the change of that correction, y_kc = (b_conv - b_pred)_kc /
 * kappa_k with kappa_k = max_c |br - er|_kc, from
 *   x[3k+c]  (br - er)_kc / kappa_k                      (21)
 *   x[21+k]  log2(kappa_k / max_c |b_pred_kc|) / 16       (7)
 *   x[28]    log2 |dt| / 8,   x[29] dt / dt_last - 1,
 *   x[30]    log2 |x| / 4,    x[31] log2(nearest planet distance) / 8.
 * The corrector then iterates from b_pred + kappa * y; its own convergence
 * test and error estimate decide as before.
 */
#ifndef ASSIST_GB300_MLP_CUH
#define ASSIST_GB300_MLP_CUH

#include <cuda_bf16.h>

#define AG_MLP_IN 32
#define AG_MLP_HID 256
#define AG_MLP_OUT 21
#define AG_MLP_OUTP 24                     /* output rows padded to 3 MMA n-tiles */
#define AG_MLP_LDX (AG_MLP_IN + 8)         /* shared-memory row strides (bf16), padded */
#define AG_MLP_LDH (AG_MLP_HID + 8)
#define AG_MLP_YCLIP 4.0f                  /* outputs beyond this are rejected */

/* Device copies of the network for inference. */
struct AgMlpDev {
    const __nv_bfloat16* W1;   /* [HID][IN] */
    const __nv_bfloat16* W2;   /* [HID][HID] */
    const __nv_bfloat16* W3;   /* [OUTP][HID], rows >= OUT zero */
    const float* b1;           /* [HID] */
    const float* b2;           /* [HID] */
    const float* b3;           /* [OUTP] */
};

/* Per-block buffers of one inference (dynamic shared memory). */
struct AgMlpSmem {
    __nv_bfloat16 X[32][AG_MLP_LDX];
    __nv_bfloat16 H1[32][AG_MLP_LDH];
    __nv_bfloat16 H2[32][AG_MLP_LDH];
    float Y[32][AG_MLP_OUTP];
};

__device__ __forceinline__ float ag_gelu(float z) {
    return 0.5f * z * (1.0f + tanhf(0.7978845608028654f * (z + 0.044715f * z * z * z)));
}

__device__ __forceinline__ void ag_mma_bf16_16816(float* d, const unsigned* a, const unsigned* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ unsigned ag_ld_bf16x2(const __nv_bfloat16* p) {
    return *reinterpret_cast<const unsigned*>(p);
}

/* out[32][n0 .. n0 + 8 NT) = act(in[32][K] W[n][K]^T + bias) by one warp
 * (two 16-row m-tiles).  GELU writes bf16 to outh (row stride LDH), otherwise
 * FP32 to outf (row stride OUTP). */
template <int K, int LDI, int NT, bool GELU>
__device__ __forceinline__ void ag_mlp_layer(const __nv_bfloat16* in, const __nv_bfloat16* __restrict__ W,
                                             const float* __restrict__ bias, int n0, __nv_bfloat16* outh,
                                             float* outf, int lane) {
    const int g = lane >> 2, tg = lane & 3;
    float acc[2][NT][4];
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int nt = 0; nt < NT; nt++)
#pragma unroll
            for (int i = 0; i < 4; i++) acc[m][nt][i] = 0.0f;
#pragma unroll 2
    for (int k0 = 0; k0 < K; k0 += 16) {
        unsigned a[2][4];
#pragma unroll
        for (int m = 0; m < 2; m++) {
            const __nv_bfloat16* r0 = in + (m * 16 + g) * LDI + k0 + tg * 2;
            const __nv_bfloat16* r1 = r0 + 8 * LDI;
            a[m][0] = ag_ld_bf16x2(r0); a[m][1] = ag_ld_bf16x2(r1);
            a[m][2] = ag_ld_bf16x2(r0 + 8); a[m][3] = ag_ld_bf16x2(r1 + 8);
        }
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
            const __nv_bfloat16* wr = W + (size_t)(n0 + nt * 8 + g) * K + k0 + tg * 2;
            const unsigned b[2] = {__ldg(reinterpret_cast<const unsigned*>(wr)),
                                   __ldg(reinterpret_cast<const unsigned*>(wr + 8))};
#pragma unroll
            for (int m = 0; m < 2; m++) ag_mma_bf16_16816(acc[m][nt], a[m], b);
        }
    }
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int nt = 0; nt < NT; nt++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = m * 16 + g + (i >= 2 ? 8 : 0);
                const int c = n0 + nt * 8 + tg * 2 + (i & 1);
                const float v = acc[m][nt][i] + bias[c];
                if (GELU) outh[r * AG_MLP_LDH + c] = __float2bfloat16_rn(ag_gelu(v));
                else outf[r * AG_MLP_OUTP + c] = v;
            }
}

/* Inference for the 32 rows in M.X by a 128-thread block (all threads call
 * it; it synchronises the block).  Result in M.Y. */
__device__ __forceinline__ void ag_mlp_infer_block(const AgMlpDev& N, AgMlpSmem& M, int wid, int lane) {
    for (int half = 0; half < 2; half++)
        ag_mlp_layer<AG_MLP_IN, AG_MLP_LDX, 4, true>(&M.X[0][0], N.W1, N.b1, 64 * wid + 32 * half, &M.H1[0][0],
                                                     nullptr, lane);
    __syncthreads();
    for (int half = 0; half < 2; half++)
        ag_mlp_layer<AG_MLP_HID, AG_MLP_LDH, 4, true>(&M.H1[0][0], N.W2, N.b2, 64 * wid + 32 * half, &M.H2[0][0],
                                                      nullptr, lane);
    __syncthreads();
    if (wid < 3)
        ag_mlp_layer<AG_MLP_HID, AG_MLP_LDH, 1, false>(&M.H2[0][0], N.W3, N.b3, 8 * wid, nullptr, &M.Y[0][0], lane);
    __syncthreads();
}

/* Features of one particle's step (see the header comment) and the
 * per-order scales kappa_k.  corr[k][c] = (br - er)_kc, bpa[k][c] =
 * |b_pred_kc|.  Returns false when the learned start does not apply (no
 * previous correction, no previous step, non-finite inputs). */
__device__ __forceinline__ bool ag_warm_features(const double (*corr)[3], const float (*bpa)[3], double hstep,
                                                 double dtls, double rx, double dnear, float* x, double* kappa) {
    bool ok = dtls != 0.0 && hstep != 0.0 && rx > 0.0 && dnear > 0.0;
#pragma unroll
    for (int k = 0; k < 7; k++) {
        const double kap = fmax(fabs(corr[k][0]), fmax(fabs(corr[k][1]), fabs(corr[k][2])));
        const float sig = fmaxf(bpa[k][0], fmaxf(bpa[k][1], bpa[k][2]));
        ok = ok && ag_isnormal_pos(kap) && sig > 0.0f;
        kappa[k] = kap;
        const double ik = ok ? 1.0 / kap : 0.0;
        for (int c = 0; c < 3; c++) x[3 * k + c] = (float)(corr[k][c] * ik);
        x[21 + k] = ok ? log2f((float)kap / sig) * (1.0f / 16.0f) : 0.0f;
    }
    x[28] = ok ? log2f((float)fabs(hstep)) * 0.125f : 0.0f;
    x[29] = ok ? fminf(fmaxf((float)(hstep / dtls) - 1.0f, -1.0f), 3.0f) : 0.0f;
    x[30] = ok ? log2f((float)rx) * 0.25f : 0.0f;
    x[31] = ok ? log2f((float)dnear) * 0.125f : 0.0f;
    return ok;
}

#endif
