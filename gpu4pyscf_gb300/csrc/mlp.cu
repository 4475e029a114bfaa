// FP32 kernels of the learned initial-guess network (atom-pair MLP):
// forward and backward of dense layers, masked mean-squared error and Adam.
//
// The dense layers are small (width 256, one row per atom pair), so one
// tiled SIMT GEMM serves every product of the forward and backward passes:
// C[M,N] = op(A)[M,K] op(B)[K,N] (+ beta C) (+ bias) with an optional SiLU
// epilogue that also stores the pre-activation for the backward pass.
// Operands are addressed through element strides, so transposed operands
// (X^T dZ for the weight gradient, dZ W^T for the input gradient) need no
// copies.  64x64 output tile per 256-thread block, 4x4 outputs per thread,
// K staged through shared memory 16 at a time.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace {

thread_local std::string g_mlp_err;

constexpr int BM = 64, BN = 64, BK = 16;

__device__ __forceinline__ float sigmoidf_(float x) { return 1.f / (1.f + expf(-x)); }

__global__ void __launch_bounds__(256)
gemm_kernel(int M, int N, int K, const float *__restrict__ A, long long sam, long long sak,
            const float *__restrict__ B, long long sbk, long long sbn, const float *__restrict__ bias,
            int act, float beta, float *__restrict__ Z, float *__restrict__ C) {
    __shared__ float As[BK][BM + 4];
    __shared__ float Bs[BK][BN + 4];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += BK) {
        // 64x16 tile of A and 16x64 tile of B, 4 elements each per thread
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            int e = tid + t * 256;
            int mm = e / BK, kk = e % BK;
            int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < K) ? A[m * sam + k * sak] : 0.f;
            int kb = e / BN, nb = e % BN;
            int kg = k0 + kb, ng = n0 + nb;
            Bs[kb][nb] = (kg < K && ng < N) ? B[kg * sbk + ng * sbn] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int m = m0 + ty * 4 + i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int n = n0 + tx * 4 + j;
            if (n >= N) continue;
            float v = acc[i][j];
            if (beta != 0.f) v += beta * C[(long long)m * N + n];
            if (bias) v += bias[n];
            if (Z) Z[(long long)m * N + n] = v;
            if (act == 1) v = v * sigmoidf_(v);
            C[(long long)m * N + n] = v;
        }
    }
}

__global__ void silu_backward_kernel(long long n, const float *dY, const float *Z, float *dZ) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float z = Z[i], s = sigmoidf_(z);
        dZ[i] = dY[i] * (s + z * s * (1.f - s));
    }
}

// out[n] = sum_m X[m, n]; one thread per column, rows strided by block
__global__ void colsum_kernel(int M, int N, const float *X, float *out) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; ++m) s += X[(long long)m * N + n];
    out[n] = s;
}

// grad = 2 mask (y - t) / count, loss += sum mask (y - t)^2 / count
__global__ void mse_kernel(long long n, const float *y, const float *t, const float *mask, float inv_count,
                           float *grad, float *loss) {
    float local = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float w = mask ? mask[i] : 1.f;
        float d = (y[i] - t[i]) * w;
        grad[i] = 2.f * d * inv_count;
        local += d * d * inv_count;
    }
    for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, local);
}

__global__ void adam_kernel(long long n, float *p, const float *g, float *m, float *v, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float gi = g[i];
        float mi = b1 * m[i] + (1.f - b1) * gi;
        float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

int ck(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return 0;
    g_mlp_err = std::string(what) + ": " + cudaGetErrorString(e);
    return -2;
}

int grid_for(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}

}  // namespace

extern "C" {

const char *mlp_last_error(void) { return g_mlp_err.c_str(); }

int mlp_gemm(int M, int N, int K, const float *A, int64_t sam, int64_t sak, const float *B, int64_t sbk,
             int64_t sbn, const float *bias, int act, float beta, float *Z, float *C, void *stream) {
    if (M < 0 || N < 0 || K < 0 || !A || !B || !C || (act != 0 && act != 1)) {
        g_mlp_err = "mlp_gemm: invalid arguments";
        return -1;
    }
    if (M == 0 || N == 0) return 0;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
    gemm_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(M, N, K, A, sam, sak, B, sbk, sbn, bias, act, beta, Z, C);
    return ck(cudaGetLastError(), "mlp_gemm");
}

int mlp_silu_backward(int64_t n, const float *dY, const float *Z, float *dZ, void *stream) {
    if (n < 0 || !dY || !Z || !dZ) { g_mlp_err = "mlp_silu_backward: invalid arguments"; return -1; }
    if (n == 0) return 0;
    silu_backward_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, dY, Z, dZ);
    return ck(cudaGetLastError(), "mlp_silu_backward");
}

int mlp_colsum(int M, int N, const float *X, float *out, void *stream) {
    if (M < 0 || N <= 0 || !X || !out) { g_mlp_err = "mlp_colsum: invalid arguments"; return -1; }
    colsum_kernel<<<(N + 127) / 128, 128, 0, (cudaStream_t)stream>>>(M, N, X, out);
    return ck(cudaGetLastError(), "mlp_colsum");
}

int mlp_mse(int64_t n, const float *y, const float *t, const float *mask, float inv_count, float *grad,
            float *loss, void *stream) {
    if (n < 0 || !y || !t || !grad) { g_mlp_err = "mlp_mse: invalid arguments"; return -1; }
    if (n == 0) return 0;
    mse_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, y, t, mask, inv_count, grad, loss);
    return ck(cudaGetLastError(), "mlp_mse");
}

int mlp_adam(int64_t n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2, float eps,
             int step, void *stream) {
    if (n < 0 || !p || !g || !m || !v || step <= 0) { g_mlp_err = "mlp_adam: invalid arguments"; return -1; }
    if (n == 0) return 0;
    float c1 = 1.f / (1.f - powf(b1, (float)step));
    float c2 = 1.f / (1.f - powf(b2, (float)step));
    adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, p, g, m, v, lr, b1, b2, eps, c1, c2);
    return ck(cudaGetLastError(), "mlp_adam");
}

}  // extern "C"
