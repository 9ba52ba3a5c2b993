/*
 * kernels_mlp.cu -- training and inference entry points of the warm-start
 * network (no counterpart in the reference).
 *
 * Training is hand-written FP32: a tiled SGEMM with general strides (so the
 * transposed products of the backward pass need no copies), the bias + GELU
 * epilogue, GELU backward, bias-gradient column sums and Adam.  The network,
 * its loss and Adam are the ones restated by the oracle's mlp_oracle.py:
 *   L = 1/(2B) sum_b sum_o (Y - T)^2,  Adam(0.9, 0.999, 1e-8), bias-corrected.
 * After every parameter change the BF16 inference copies are refreshed.
 *
 * State is per process and device-current at the time of the calls (one
 * network, as the IAS15 kernels read one).
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <random>
#include <vector>

#include "assist.h"
#include "device_ephem.cuh"
#include "internal.h"
#include "mlp.cuh"

namespace {

constexpr int NIN = AG_MLP_IN, NH = AG_MLP_HID, NO = AG_MLP_OUT, NOP = AG_MLP_OUTP;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NO * NH, NPARAM = OFF_B3 + NO;

struct Net {
    bool ready = false;            /* device buffers allocated */
    bool loaded = false;           /* parameters set (init, set_params) */
    float* p = nullptr;            /* FP32 master parameters, oracle layout */
    float* g = nullptr;            /* gradient */
    float* m = nullptr;            /* Adam moments */
    float* v = nullptr;
    long long step = 0;            /* Adam step count */
    __nv_bfloat16* w16 = nullptr;  /* W1 | W2 | W3 (padded to NOP rows) */
    float* b3p = nullptr;          /* b3 padded to NOP */
    AgMlpDev* d_dev = nullptr;     /* device copy of the inference view */
    AgMlpDev h_dev;
    /* training work buffers, grown on demand */
    float* work = nullptr;
    size_t work_cap = 0;
    double* d_loss = nullptr;
    /* pair logging of the next batched integrations */
    float* log_x = nullptr;
    float* log_t = nullptr;
    int log_cap = 0, log_every = 0;
    int* d_log_count = nullptr;
};

Net g_net;
std::mutex g_net_mu;

/* C[i][j] = alpha * sum_k A(i,k) B(k,j) + beta * C[i][j];
 * A(i,k) = A[i*sai + k*sak], B(k,j) = B[k*sbk + j*sbj].  64x64 tile, 256
 * threads, 4x4 outputs a thread, K in steps of 16 through shared memory. */
__global__ void __launch_bounds__(256) k_sgemm(int M, int N, int K, float alpha, const float* __restrict__ A,
                                               long long sai, long long sak, const float* __restrict__ B,
                                               long long sbk, long long sbj, float beta, float* __restrict__ C,
                                               int ldc) {
    __shared__ float As[16][64 + 1];
    __shared__ float Bs[16][64 + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            const int kk = e / 64, ii = e % 64;
            const int i = i0 + ii, k = k0 + kk;
            As[kk][ii] = (i < M && k < K) ? A[(long long)i * sai + (long long)k * sak] : 0.0f;
            const int j = j0 + ii;
            Bs[kk][ii] = (j < N && k < K) ? B[(long long)k * sbk + (long long)j * sbj] : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; r++) a[r] = As[kk][ty * 4 + r];
#pragma unroll
            for (int c = 0; c < 4; c++) b[c] = Bs[kk][tx * 4 + c];
#pragma unroll
            for (int r = 0; r < 4; r++)
#pragma unroll
                for (int c = 0; c < 4; c++) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            const int i = i0 + ty * 4 + r, j = j0 + tx * 4 + c;
            if (i < M && j < N) {
                float* o = C + (long long)i * ldc + j;
                *o = alpha * acc[r][c] + (beta != 0.0f ? beta * *o : 0.0f);
            }
        }
}

/* Z += bias (per column); A = gelu(Z) when act, else A = Z. */
__global__ void k_bias_act(float* Z, float* Aout, const float* bias, int rows, int cols, int act) {
    const long long n = (long long)rows * cols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float z = Z[e] + bias[e % cols];
        Z[e] = z;
        Aout[e] = act ? ag_gelu(z) : z;
    }
}

/* dY = (Y - T) / B and the loss sum 0.5 sum (Y - T)^2 / B. */
__global__ void k_loss_grad(const float* Y, const float* T, float* dY, long long n, float invB, double* loss) {
    double s = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float r = Y[e] - T[e];
        dY[e] = r * invB;
        s += 0.5 * (double)r * (double)r * (double)invB;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

/* dZ = dA * gelu'(Z) (in place on dA). */
__global__ void k_gelu_back(float* dA, const float* Z, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float z = Z[e];
        const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
        const float th = tanhf(u);
        const float d = 0.5f * (1.0f + th) + 0.5f * z * (1.0f - th * th) * 0.7978845608028654f * (1.0f + 3.0f * 0.044715f * z * z);
        dA[e] *= d;
    }
}

/* db[j] = sum_i dZ[i][j]; one block per column. */
__global__ void k_colsum(const float* dZ, float* db, int rows, int cols) {
    const int j = blockIdx.x;
    float s = 0.0f;
    for (int i = threadIdx.x; i < rows; i += blockDim.x) s += dZ[(long long)i * cols + j];
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[j] = red[0];
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, int n, float lr, float c1, float c2) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float gg = g[e];
    const float mm = 0.9f * m[e] + 0.1f * gg;
    const float vv = 0.999f * v[e] + 0.001f * gg * gg;
    m[e] = mm; v[e] = vv;
    p[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + 1e-8f);
}

/* BF16 inference copies: W1 | W2 | W3 padded to NOP rows; b3 padded. */
__global__ void k_to_bf16(const float* p, __nv_bfloat16* w16, float* b3p) {
    const int n1 = NH * NIN, n2 = NH * NH, n3 = NOP * NH;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n1 + n2 + n3; e += gridDim.x * blockDim.x) {
        float x;
        if (e < n1) x = p[OFF_W1 + e];
        else if (e < n1 + n2) x = p[OFF_W2 + (e - n1)];
        else {
            const int q = e - n1 - n2;
            x = q < NO * NH ? p[OFF_W3 + q] : 0.0f;
        }
        w16[e] = __float2bfloat16_rn(x);
    }
    if (blockIdx.x == 0 && threadIdx.x < NOP) b3p[threadIdx.x] = threadIdx.x < NO ? p[OFF_B3 + threadIdx.x] : 0.0f;
}

/* Standalone BF16 inference of n rows (the IAS15 kernel's device function). */
__global__ void __launch_bounds__(128) k_infer(const AgMlpDev* __restrict__ Np, const float* X, float* Y, int n) {
    extern __shared__ __align__(16) unsigned char dyn[];
    AgMlpSmem& M = *reinterpret_cast<AgMlpSmem*>(dyn);
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = blockIdx.x * 32;
    for (int e = threadIdx.x; e < 32 * NIN; e += 128) {
        const int r = e / NIN, c = e % NIN;
        M.X[r][c] = __float2bfloat16_rn(r0 + r < n ? X[(long long)(r0 + r) * NIN + c] : 0.0f);
    }
    __syncthreads();
    ag_mlp_infer_block(*Np, M, wid, lane);
    for (int e = threadIdx.x; e < 32 * NO; e += 128) {
        const int r = e / NO, c = e % NO;
        if (r0 + r < n) Y[(long long)(r0 + r) * NO + c] = M.Y[r][c];
    }
}

int grid_for(long long n, int tpb) {
    long long b = (n + tpb - 1) / tpb;
    return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

void sgemm(int M, int N, int K, const float* A, long long sai, long long sak, const float* B, long long sbk,
           long long sbj, float beta, float* C, int ldc, cudaStream_t s) {
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    k_sgemm<<<grid, 256, 0, s>>>(M, N, K, 1.0f, A, sai, sak, B, sbk, sbj, beta, C, ldc);
}

int ensure_net() {
    if (g_net.ready) return 0;
    Net& n = g_net;
    const size_t w16n = (size_t)NH * NIN + (size_t)NH * NH + (size_t)NOP * NH;
    if (ag_cuda_check(cudaMalloc(&n.p, sizeof(float) * NPARAM), "cudaMalloc(mlp)") ||
        ag_cuda_check(cudaMalloc(&n.g, sizeof(float) * NPARAM), "cudaMalloc(mlp)") ||
        ag_cuda_check(cudaMalloc(&n.m, sizeof(float) * NPARAM), "cudaMalloc(mlp)") ||
        ag_cuda_check(cudaMalloc(&n.v, sizeof(float) * NPARAM), "cudaMalloc(mlp)") ||
        ag_cuda_check(cudaMalloc(&n.w16, sizeof(__nv_bfloat16) * w16n), "cudaMalloc(mlp)") ||
        ag_cuda_check(cudaMalloc(&n.b3p, sizeof(float) * NOP), "cudaMalloc(mlp)") ||
        ag_cuda_check(cudaMalloc(&n.d_dev, sizeof(AgMlpDev)), "cudaMalloc(mlp)") ||
        ag_cuda_check(cudaMalloc(&n.d_loss, sizeof(double)), "cudaMalloc(mlp)") ||
        ag_cuda_check(cudaMalloc(&n.d_log_count, sizeof(int)), "cudaMalloc(mlp)"))
        return 1;
    cudaMemset(n.m, 0, sizeof(float) * NPARAM);
    cudaMemset(n.v, 0, sizeof(float) * NPARAM);
    cudaMemset(n.d_log_count, 0, sizeof(int));
    n.h_dev.W1 = n.w16;
    n.h_dev.W2 = n.w16 + (size_t)NH * NIN;
    n.h_dev.W3 = n.w16 + (size_t)NH * NIN + (size_t)NH * NH;
    n.h_dev.b1 = n.p + OFF_B1;
    n.h_dev.b2 = n.p + OFF_B2;
    n.h_dev.b3 = n.b3p;
    if (ag_cuda_check(cudaMemcpy(n.d_dev, &n.h_dev, sizeof(AgMlpDev), cudaMemcpyHostToDevice), "upload mlp view")) return 1;
    n.ready = true;
    return 0;
}

int refresh_bf16() {
    k_to_bf16<<<256, 256>>>(g_net.p, g_net.w16, g_net.b3p);
    return ag_cuda_check(cudaGetLastError(), "mlp bf16 copy");
}

float* work(size_t nfloat) {
    if (nfloat > g_net.work_cap) {
        if (g_net.work) cudaFree(g_net.work);
        g_net.work = nullptr;
        g_net.work_cap = 0;
        if (ag_cuda_check(cudaMalloc(&g_net.work, sizeof(float) * nfloat), "cudaMalloc(mlp work)")) return nullptr;
        g_net.work_cap = nfloat;
    }
    return g_net.work;
}

/* Forward (FP32) and backward of B rows into g_net.g; loss to *loss. */
int forward_backward(const float* X, const float* T, int B, double* loss) {
    float* w = work((size_t)B * (4 * NH + 2 * NO + 2 * NH));
    if (!w) return 1;
    float *Z1 = w, *A1 = Z1 + (size_t)B * NH, *Z2 = A1 + (size_t)B * NH, *A2 = Z2 + (size_t)B * NH;
    float *Y = A2 + (size_t)B * NH, *dY = Y + (size_t)B * NO, *dA2 = dY + (size_t)B * NO, *dA1 = dA2 + (size_t)B * NH;
    const float* P = g_net.p;
    float* G = g_net.g;
    cudaStream_t s = 0;
    /* forward */
    sgemm(B, NH, NIN, X, NIN, 1, P + OFF_W1, 1, NIN, 0.0f, Z1, NH, s);
    k_bias_act<<<grid_for((long long)B * NH, 256), 256, 0, s>>>(Z1, A1, P + OFF_B1, B, NH, 1);
    sgemm(B, NH, NH, A1, NH, 1, P + OFF_W2, 1, NH, 0.0f, Z2, NH, s);
    k_bias_act<<<grid_for((long long)B * NH, 256), 256, 0, s>>>(Z2, A2, P + OFF_B2, B, NH, 1);
    sgemm(B, NO, NH, A2, NH, 1, P + OFF_W3, 1, NH, 0.0f, Y, NO, s);
    k_bias_act<<<grid_for((long long)B * NO, 256), 256, 0, s>>>(Y, Y, P + OFF_B3, B, NO, 0);
    /* loss and dY */
    cudaMemsetAsync(g_net.d_loss, 0, sizeof(double), s);
    k_loss_grad<<<grid_for((long long)B * NO, 256), 256, 0, s>>>(Y, T, dY, (long long)B * NO, 1.0f / (float)B, g_net.d_loss);
    /* layer 3: dW3 = dY^T A2, db3 = colsum dY, dA2 = dY W3 */
    sgemm(NO, NH, B, dY, 1, NO, A2, NH, 1, 0.0f, G + OFF_W3, NH, s);
    k_colsum<<<NO, 256, 0, s>>>(dY, G + OFF_B3, B, NO);
    sgemm(B, NH, NO, dY, NO, 1, P + OFF_W3, NH, 1, 0.0f, dA2, NH, s);
    k_gelu_back<<<grid_for((long long)B * NH, 256), 256, 0, s>>>(dA2, Z2, (long long)B * NH);
    /* layer 2 */
    sgemm(NH, NH, B, dA2, 1, NH, A1, NH, 1, 0.0f, G + OFF_W2, NH, s);
    k_colsum<<<NH, 256, 0, s>>>(dA2, G + OFF_B2, B, NH);
    sgemm(B, NH, NH, dA2, NH, 1, P + OFF_W2, NH, 1, 0.0f, dA1, NH, s);
    k_gelu_back<<<grid_for((long long)B * NH, 256), 256, 0, s>>>(dA1, Z1, (long long)B * NH);
    /* layer 1 */
    sgemm(NH, NIN, B, dA1, 1, NH, X, NIN, 1, 0.0f, G + OFF_W1, NIN, s);
    k_colsum<<<NH, 256, 0, s>>>(dA1, G + OFF_B1, B, NH);
    if (ag_cuda_check(cudaGetLastError(), "mlp forward/backward")) return 1;
    if (loss && ag_cuda_check(cudaMemcpy(loss, g_net.d_loss, sizeof(double), cudaMemcpyDeviceToHost), "mlp loss"))
        return 1;
    return 0;
}

}  // namespace

/* Inference view for the IAS15 kernels (null when no network is loaded). */
const AgMlpDev* ag_mlp_device_view(void) { return g_net.loaded ? g_net.d_dev : nullptr; }

int ag_mlp_log_config(float** x, float** t, int* cap, int* every, int** count) {
    *x = g_net.log_x; *t = g_net.log_t; *cap = g_net.log_cap; *every = g_net.log_every; *count = g_net.d_log_count;
    return g_net.log_x && g_net.ready ? 1 : 0;
}

extern "C" int assist_gb300_warm_n_params(void) { return NPARAM; }

extern "C" int assist_gb300_warm_init(unsigned long long seed) {
    std::lock_guard<std::mutex> lk(g_net_mu);
    if (ensure_net()) return ASSIST_ERROR_EPHEM_FILE;
    std::vector<float> h(NPARAM, 0.0f);
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    for (int i = 0; i < NH * NIN; i++) h[OFF_W1 + i] = (float)(nd(rng) * std::sqrt(2.0 / NIN));
    for (int i = 0; i < NH * NH; i++) h[OFF_W2 + i] = (float)(nd(rng) * std::sqrt(2.0 / NH));
    for (int i = 0; i < NO * NH; i++) h[OFF_W3 + i] = (float)(nd(rng) * 0.1 * std::sqrt(1.0 / NH));
    if (ag_cuda_check(cudaMemcpy(g_net.p, h.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice), "mlp init"))
        return ASSIST_ERROR_EPHEM_FILE;
    cudaMemset(g_net.m, 0, sizeof(float) * NPARAM);
    cudaMemset(g_net.v, 0, sizeof(float) * NPARAM);
    g_net.step = 0;
    g_net.loaded = true;
    return refresh_bf16() ? ASSIST_ERROR_EPHEM_FILE : ASSIST_SUCCESS;
}

extern "C" int assist_gb300_warm_set_params(const float* params, int n) {
    std::lock_guard<std::mutex> lk(g_net_mu);
    if (n != NPARAM) { ag_set_error("warm-start parameter count mismatch"); return ASSIST_ERROR_N; }
    if (ensure_net()) return ASSIST_ERROR_EPHEM_FILE;
    if (ag_cuda_check(cudaMemcpy(g_net.p, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice), "mlp params"))
        return ASSIST_ERROR_EPHEM_FILE;
    cudaMemset(g_net.m, 0, sizeof(float) * NPARAM);
    cudaMemset(g_net.v, 0, sizeof(float) * NPARAM);
    g_net.step = 0;
    g_net.loaded = true;
    return refresh_bf16() ? ASSIST_ERROR_EPHEM_FILE : ASSIST_SUCCESS;
}

extern "C" int assist_gb300_warm_get_params(float* params, int n) {
    std::lock_guard<std::mutex> lk(g_net_mu);
    if (n != NPARAM || !g_net.loaded) { ag_set_error("no warm-start network or count mismatch"); return ASSIST_ERROR_N; }
    return ag_cuda_check(cudaMemcpy(params, g_net.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost), "mlp params")
               ? ASSIST_ERROR_EPHEM_FILE : ASSIST_SUCCESS;
}

extern "C" int assist_gb300_warm_grad(const float* d_x, const float* d_t, int n, float* grad, double* loss) {
    std::lock_guard<std::mutex> lk(g_net_mu);
    if (!g_net.loaded || n <= 0) { ag_set_error("no warm-start network or empty batch"); return ASSIST_ERROR_N; }
    if (forward_backward(d_x, d_t, n, loss)) return ASSIST_ERROR_EPHEM_FILE;
    if (grad && ag_cuda_check(cudaMemcpy(grad, g_net.g, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost), "mlp grad"))
        return ASSIST_ERROR_EPHEM_FILE;
    return ASSIST_SUCCESS;
}

extern "C" int assist_gb300_warm_train(const float* d_x, const float* d_t, int n, int steps, int batch, float lr,
                                       unsigned long long seed, double* loss_out) {
    std::lock_guard<std::mutex> lk(g_net_mu);
    if (!g_net.loaded || n <= 0 || batch <= 0 || steps < 0) { ag_set_error("warm_train: bad arguments or no network"); return ASSIST_ERROR_N; }
    if (batch > n) batch = n;
    std::mt19937_64 rng(seed);
    const int nb = n / batch;
    double last = 0.0;
    for (int s = 0; s < steps; s++) {
        const int b = (int)(rng() % (unsigned long long)nb);
        const float* X = d_x + (size_t)b * batch * NIN;
        const float* T = d_t + (size_t)b * batch * NO;
        const bool want_loss = (s == steps - 1) && loss_out;
        if (forward_backward(X, T, batch, want_loss ? &last : nullptr)) return ASSIST_ERROR_EPHEM_FILE;
        g_net.step++;
        const float c1 = 1.0f - std::pow(0.9f, (float)g_net.step), c2 = 1.0f - std::pow(0.999f, (float)g_net.step);
        k_adam<<<(NPARAM + 255) / 256, 256>>>(g_net.p, g_net.g, g_net.m, g_net.v, NPARAM, lr, c1, c2);
    }
    if (loss_out) *loss_out = last;
    return refresh_bf16() || ag_cuda_check(cudaDeviceSynchronize(), "mlp train") ? ASSIST_ERROR_EPHEM_FILE : ASSIST_SUCCESS;
}

extern "C" int assist_gb300_warm_adam_step(const float* grad, float lr) {
    std::lock_guard<std::mutex> lk(g_net_mu);
    if (!g_net.loaded) { ag_set_error("no warm-start network"); return ASSIST_ERROR_N; }
    if (ag_cuda_check(cudaMemcpy(g_net.g, grad, sizeof(float) * NPARAM, cudaMemcpyHostToDevice), "mlp grad upload"))
        return ASSIST_ERROR_EPHEM_FILE;
    g_net.step++;
    const float c1 = 1.0f - std::pow(0.9f, (float)g_net.step), c2 = 1.0f - std::pow(0.999f, (float)g_net.step);
    k_adam<<<(NPARAM + 255) / 256, 256>>>(g_net.p, g_net.g, g_net.m, g_net.v, NPARAM, lr, c1, c2);
    return refresh_bf16() || ag_cuda_check(cudaDeviceSynchronize(), "mlp adam") ? ASSIST_ERROR_EPHEM_FILE : ASSIST_SUCCESS;
}

extern "C" int assist_gb300_warm_infer(const float* d_x, int n, float* d_y) {
    std::lock_guard<std::mutex> lk(g_net_mu);
    if (!g_net.loaded || n <= 0) { ag_set_error("no warm-start network or empty batch"); return ASSIST_ERROR_N; }
    const int smem = (int)sizeof(AgMlpSmem);
    cudaFuncSetAttribute(k_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_infer<<<(n + 31) / 32, 128, smem>>>(g_net.d_dev, d_x, d_y, n);
    return ag_cuda_check(cudaDeviceSynchronize(), "mlp inference") ? ASSIST_ERROR_EPHEM_FILE : ASSIST_SUCCESS;
}

extern "C" int assist_gb300_warm_set_log(float* d_x, float* d_t, int capacity, int every) {
    std::lock_guard<std::mutex> lk(g_net_mu);
    if (ensure_net()) return ASSIST_ERROR_EPHEM_FILE;
    g_net.log_x = (d_x && d_t && capacity > 0) ? d_x : nullptr;
    g_net.log_t = g_net.log_x ? d_t : nullptr;
    g_net.log_cap = g_net.log_x ? capacity : 0;
    g_net.log_every = every > 0 ? every : 1;
    return ag_cuda_check(cudaMemset(g_net.d_log_count, 0, sizeof(int)), "mlp log reset") ? ASSIST_ERROR_EPHEM_FILE
                                                                                        : ASSIST_SUCCESS;
}

extern "C" int assist_gb300_warm_log_count(void) {
    std::lock_guard<std::mutex> lk(g_net_mu);
    if (!g_net.ready) return 0;
    int c = 0;
    cudaMemcpy(&c, g_net.d_log_count, sizeof(int), cudaMemcpyDeviceToHost);
    return c < g_net.log_cap ? c : g_net.log_cap;
}
