// gnn.cu -- training and inference kernels of the message-passing network that supplies
// GMRES initial guesses (a learned component the reference does not have).
//
// Graph: one node per RWG edge, neighbours = the other edges of its (one or two) triangles
// (at most 4; nbr [N, 4] int32, -1 where absent).  Layer l: h' = relu([h, mean_nbr(h)] W + b).
// Storage: activations and the forward copy of the weights in BF16, every product and sum
// accumulated in FP32, master weights and Adam moments in FP32, gradients in FP32.
//
// Kernels:
//   gnn_gemm      Y[N, M] = act(X[N, K] W[K, M] + b) (or X W^T with W [M, K]); 64 x 64 output
//                 tile per block, K in chunks of 32 staged in shared memory as FP32, 4 x 4
//                 outputs per thread; BF16 or FP32 inputs, BF16 or FP32 outputs.
//   gnn_gemm_tn   dW[K, M] += X[N, K]^T dY[N, M] over a chunk of rows per block (FP32 atomics).
//   gnn_colsum    db[M] += sum_n dY[n, M].
//   gnn_aggregate out[n] = [h[n], mean_j h[nbr(n, j)]] (concatenation, BF16).
//   gnn_aggregate_bwd  dh[n] += dcat[n, :F]; dh[j] += dcat[n, F:] / deg(n) for j in nbr(n).
//   gnn_relu_bwd  dZ = dY where Y > 0, else 0.
//   gnn_adam      Adam step on FP32 master weights, refreshes the BF16 copy.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace mb {

template <typename T>
__device__ __forceinline__ float to_f(T v);
template <>
__device__ __forceinline__ float to_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <typename T>
__device__ __forceinline__ T from_f(float v);
template <>
__device__ __forceinline__ float from_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

constexpr int kGT = 64, kGK = 32;

// TRANS_W: W is [M, K] (use W^T); else W is [K, M].
template <typename TX, typename TW, typename TY, bool TRANS_W>
__global__ void __launch_bounds__(256) gnn_gemm_kernel(const TX* __restrict__ X, const TW* __restrict__ W,
                                                       const float* __restrict__ bias, int64_t N, int K, int M,
                                                       int relu, TY* __restrict__ Y) {
    __shared__ float sx[kGK][kGT + 1];  // [k][row]
    __shared__ float sw[kGK][kGT + 1];  // [k][col]
    const int tid = threadIdx.x, tr = tid / 16, tc = tid % 16;
    const int64_t row0 = (int64_t)blockIdx.x * kGT;
    const int col0 = blockIdx.y * kGT;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kGK) {
        for (int e = tid; e < kGK * kGT; e += 256) {
            const int r = e / kGK, k = e % kGK;  // X tile: consecutive threads along k
            const int64_t gr = row0 + r;
            sx[k][r] = (gr < N && k0 + k < K) ? to_f<TX>(X[gr * K + k0 + k]) : 0.f;
        }
        for (int e = tid; e < kGK * kGT; e += 256) {
            float v;
            if (TRANS_W) {
                const int c = e / kGK, k = e % kGK;
                v = (col0 + c < M && k0 + k < K) ? to_f<TW>(W[(int64_t)(col0 + c) * K + k0 + k]) : 0.f;
                sw[k][c] = v;
            } else {
                const int k = e / kGT, c = e % kGT;
                v = (col0 + c < M && k0 + k < K) ? to_f<TW>(W[(int64_t)(k0 + k) * M + col0 + c]) : 0.f;
                sw[k][c] = v;
            }
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < kGK; ++k) {
            float a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a[q] = sx[k][tr * 4 + q];
                b[q] = sw[k][tc * 4 + q];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t r = row0 + tr * 4 + i;
        if (r >= N) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = col0 + tc * 4 + j;
            if (c >= M) continue;
            float v = acc[i][j] + (bias ? bias[c] : 0.f);
            if (relu) v = fmaxf(v, 0.f);
            Y[r * M + c] = from_f<TY>(v);
        }
    }
}

// dW[K, M] += X[rows, K]^T dY[rows, M] for the block's chunk of rows.
template <typename TX>
__global__ void __launch_bounds__(256) gnn_gemm_tn_kernel(const TX* __restrict__ X, const float* __restrict__ dY,
                                                          int64_t N, int K, int M, int64_t rows_per_block,
                                                          float* __restrict__ dW) {
    __shared__ float sx[kGK][kGT + 1];  // [n][k]
    __shared__ float sy[kGK][kGT + 1];  // [n][m]
    const int tid = threadIdx.x, tr = tid / 16, tc = tid % 16;
    const int k0 = blockIdx.x * kGT, m0 = blockIdx.y * kGT;
    const int64_t n_begin = (int64_t)blockIdx.z * rows_per_block;
    const int64_t n_end = n_begin + rows_per_block < N ? n_begin + rows_per_block : N;
    float acc[4][4] = {};
    for (int64_t n0 = n_begin; n0 < n_end; n0 += kGK) {
        for (int e = tid; e < kGK * kGT; e += 256) {
            const int n = e / kGT, c = e % kGT;
            const int64_t gn = n0 + n;
            sx[n][c] = (gn < n_end && k0 + c < K) ? to_f<TX>(X[gn * K + k0 + c]) : 0.f;
            sy[n][c] = (gn < n_end && m0 + c < M) ? dY[gn * M + m0 + c] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int n = 0; n < kGK; ++n) {
            float a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a[q] = sx[n][tr * 4 + q];
                b[q] = sy[n][tc * 4 + q];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int k = k0 + tr * 4 + i;
        if (k >= K) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + tc * 4 + j;
            if (m < M) atomicAdd(dW + (int64_t)k * M + m, acc[i][j]);
        }
    }
}

__global__ void gnn_colsum_kernel(const float* __restrict__ dY, int64_t N, int M, float* __restrict__ db) {
    const int m = blockIdx.x * 32 + threadIdx.x;
    if (m >= M) return;
    float s = 0.f;
    for (int64_t n = (int64_t)blockIdx.y * blockDim.y + threadIdx.y; n < N; n += (int64_t)gridDim.y * blockDim.y)
        s += dY[n * M + m];
    atomicAdd(db + m, s);
}

__global__ void gnn_aggregate_kernel(const __nv_bfloat16* __restrict__ h, const int32_t* __restrict__ nbr, int64_t N,
                                     int F, __nv_bfloat16* __restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N * F) return;
    const int64_t n = idx / F;
    const int f = (int)(idx % F);
    float s = 0.f;
    int deg = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int32_t q = nbr[4 * n + j];
        if (q >= 0) {
            s += __bfloat162float(h[(int64_t)q * F + f]);
            ++deg;
        }
    }
    out[n * 2 * F + f] = h[idx];
    out[n * 2 * F + F + f] = __float2bfloat16_rn(deg ? s / deg : 0.f);
}

__global__ void gnn_aggregate_bwd_kernel(const float* __restrict__ dcat, const int32_t* __restrict__ nbr, int64_t N,
                                         int F, float* __restrict__ dh) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N * F) return;
    const int64_t n = idx / F;
    const int f = (int)(idx % F);
    atomicAdd(dh + idx, dcat[n * 2 * F + f]);
    int deg = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) deg += nbr[4 * n + j] >= 0;
    if (!deg) return;
    const float g = dcat[n * 2 * F + F + f] / deg;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int32_t q = nbr[4 * n + j];
        if (q >= 0) atomicAdd(dh + (int64_t)q * F + f, g);
    }
}

__global__ void gnn_relu_bwd_kernel(const __nv_bfloat16* __restrict__ y, const float* __restrict__ dy, int64_t count,
                                    float* __restrict__ dz) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    dz[i] = __bfloat162float(y[i]) > 0.f ? dy[i] : 0.f;
}

__global__ void gnn_adam_kernel(float* __restrict__ w, float* __restrict__ m1, float* __restrict__ m2,
                                const float* __restrict__ g, int64_t count, float lr, float b1, float b2, float eps,
                                float c1, float c2, __nv_bfloat16* __restrict__ w16) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float wi = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16_rn(wi);
}

// ---- launchers ----------------------------------------------------------------------------
// dtype codes: 0 fp32, 1 bf16
int gnn_gemm(const void* X, int x_bf16, const void* W, int w_bf16, int trans_w, const float* bias, int64_t N, int K,
             int M, int relu, void* Y, int y_bf16, cudaStream_t s) {
    if (N <= 0 || K <= 0 || M <= 0) return MB_OK;
    const dim3 grid((unsigned)((N + kGT - 1) / kGT), (unsigned)((M + kGT - 1) / kGT));
    if (grid.x > 0x7fffffffu || grid.y > 65535) return set_error(MB_ERR_SIZE, "gnn_gemm: too large");
    using bf = __nv_bfloat16;
#define MB_G(TX, TW, TY, TR)                                                                                    \
    gnn_gemm_kernel<TX, TW, TY, TR><<<grid, 256, 0, s>>>(static_cast<const TX*>(X), static_cast<const TW*>(W), \
                                                          bias, N, K, M, relu, static_cast<TY*>(Y))
    // the combinations the network uses
    if (x_bf16 && w_bf16 && y_bf16 && !trans_w) MB_G(bf, bf, bf, false);
    else if (x_bf16 && w_bf16 && !y_bf16 && !trans_w) MB_G(bf, bf, float, false);
    else if (!x_bf16 && w_bf16 && !y_bf16 && trans_w) MB_G(float, bf, float, true);
    else if (!x_bf16 && !w_bf16 && !y_bf16 && trans_w) MB_G(float, float, float, true);
    else if (!x_bf16 && !w_bf16 && !y_bf16 && !trans_w) MB_G(float, float, float, false);
    else return set_error(MB_ERR_UNSUPPORTED, "gnn_gemm: unsupported dtype combination");
#undef MB_G
    return check_launch("gnn_gemm");
}

int gnn_gemm_tn(const void* X, int x_bf16, const float* dY, int64_t N, int K, int M, float* dW, cudaStream_t s) {
    if (N <= 0 || K <= 0 || M <= 0) return MB_OK;
    const int64_t chunks = (N + 2047) / 2048;
    const dim3 grid((unsigned)((K + kGT - 1) / kGT), (unsigned)((M + kGT - 1) / kGT), (unsigned)chunks);
    if (chunks > 65535) return set_error(MB_ERR_SIZE, "gnn_gemm_tn: too many rows");
    if (x_bf16)
        gnn_gemm_tn_kernel<__nv_bfloat16><<<grid, 256, 0, s>>>(static_cast<const __nv_bfloat16*>(X), dY, N, K, M,
                                                                2048, dW);
    else
        gnn_gemm_tn_kernel<float><<<grid, 256, 0, s>>>(static_cast<const float*>(X), dY, N, K, M, 2048, dW);
    return check_launch("gnn_gemm_tn");
}

int gnn_colsum(const float* dY, int64_t N, int M, float* db, cudaStream_t s) {
    if (N <= 0 || M <= 0) return MB_OK;
    const int64_t gy = (N + 255) / 256 < 1024 ? (N + 255) / 256 : 1024;
    gnn_colsum_kernel<<<dim3((unsigned)((M + 31) / 32), (unsigned)gy), dim3(32, 8), 0, s>>>(dY, N, M, db);
    return check_launch("gnn_colsum");
}

int gnn_aggregate(const void* h, const int32_t* nbr, int64_t N, int F, void* out, cudaStream_t s) {
    if (N <= 0) return MB_OK;
    const int64_t total = N * F;
    gnn_aggregate_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(static_cast<const __nv_bfloat16*>(h), nbr, N, F,
                                                                        static_cast<__nv_bfloat16*>(out));
    return check_launch("gnn_aggregate");
}

int gnn_aggregate_bwd(const float* dcat, const int32_t* nbr, int64_t N, int F, float* dh, cudaStream_t s) {
    if (N <= 0) return MB_OK;
    const int64_t total = N * F;
    gnn_aggregate_bwd_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(dcat, nbr, N, F, dh);
    return check_launch("gnn_aggregate_bwd");
}

int gnn_relu_bwd(const void* y, const float* dy, int64_t count, float* dz, cudaStream_t s) {
    if (count <= 0) return MB_OK;
    gnn_relu_bwd_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(static_cast<const __nv_bfloat16*>(y), dy,
                                                                       count, dz);
    return check_launch("gnn_relu_bwd");
}

int gnn_adam(float* w, float* m1, float* m2, const float* g, int64_t count, float lr, float b1, float b2, float eps,
             int step, void* w16, cudaStream_t s) {
    if (count <= 0) return MB_OK;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    gnn_adam_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(w, m1, m2, g, count, lr, b1, b2, eps, c1, c2,
                                                                    static_cast<__nv_bfloat16*>(w16));
    return check_launch("gnn_adam");
}

}  // namespace mb
