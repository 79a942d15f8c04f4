// gmres.cu -- dense complex GMRES(m) with FP64 refinement for the RWG system Z x = b.
//
// The reference solves with torch.linalg.solve (dense LU, mesh_BEM_solver_3d.py:174), which
// is O(E^3).  This solver keeps Z in complex64 (7.55 GB at E = 30720) and is HBM-bound:
//   * matvec_c64: y = Z v with Z complex64, v complex64, products in FP32, per-lane partial
//     sums in FP32 over a 1/32 slice of the row, warp reduction in FP64; one warp per row,
//     16-byte streaming loads of Z (the matrix is read once per iteration, 8 E^2 bytes);
//   * residual_c128: r = b - Z x with x, b complex128 and FP64 products (the refinement
//     residual of every restart cycle);
//   * Arnoldi by classical Gram-Schmidt with one re-orthogonalisation pass (CGS2) on a
//     complex128 basis, dot products accumulated in FP64 (block partials + FP64 atomics);
//   * Givens rotations and the small least-squares solve on the host (m <= 128 numbers).
// Each restart cycle starts from the FP64 residual, so the inner FP32 matvec limits only
// the per-cycle reduction, not the final accuracy (GMRES with iterative refinement).
// Every loop is bounded by max_iters; nothing waits on the device except cudaStreamSynchronize.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <complex>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "packed.cuh"
#include "spai_apply.cuh"

namespace mb {

constexpr int kGmresMaxRestart = 128;

struct c128 {
    double re, im;
};

// ---------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// y[row] = sum_j Z[row, j] v[j]; Z, v interleaved complex64; y complex128.
// One warp per row; lane l reads float4 (two complex) at 16-byte granularity when both the
// Z row and v start on a 16-byte boundary, else one complex at a time (v may be an
// 8-byte-aligned view such as X[1:n+1] of a complex64 array).
// `active` (may be null): a device flag of the preconditioned solver; 0 makes the launch a
// no-op (a step of a captured restart cycle after the cycle has ended).
__global__ void __launch_bounds__(256) matvec_c64_kernel(const float* __restrict__ z,
                                                         const float* __restrict__ v, int64_t n,
                                                         double* __restrict__ y,
                                                         const int* __restrict__ active = nullptr) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n || (active && !*active)) return;
    const float* zr = z + 2 * row * n;
    float ar = 0.f, ai = 0.f;
    const int64_t npair = n >> 1;  // float4 = two complex numbers
    const float4* z4 = reinterpret_cast<const float4*>(zr);
    const float4* v4 = reinterpret_cast<const float4*>(v);
    const bool aligned = (((reinterpret_cast<uintptr_t>(zr) | reinterpret_cast<uintptr_t>(v)) & 15) == 0);
    if (aligned) {
        int64_t p = lane;
        for (; p + 96 < npair; p += 128) {
            const float4 a0 = __ldcs(z4 + p), a1 = __ldcs(z4 + p + 32), a2 = __ldcs(z4 + p + 64),
                         a3 = __ldcs(z4 + p + 96);
            const float4 b0 = __ldg(v4 + p), b1 = __ldg(v4 + p + 32), b2 = __ldg(v4 + p + 64),
                         b3 = __ldg(v4 + p + 96);
#define MB_CMAC(A, B)                                     \
    ar = fmaf(A.x, B.x, fmaf(-A.y, B.y, ar));             \
    ai = fmaf(A.x, B.y, fmaf(A.y, B.x, ai));              \
    ar = fmaf(A.z, B.z, fmaf(-A.w, B.w, ar));             \
    ai = fmaf(A.z, B.w, fmaf(A.w, B.z, ai));
            MB_CMAC(a0, b0) MB_CMAC(a1, b1) MB_CMAC(a2, b2) MB_CMAC(a3, b3)
        }
        for (; p < npair; p += 32) {
            const float4 a0 = __ldcs(z4 + p);
            const float4 b0 = __ldg(v4 + p);
            MB_CMAC(a0, b0)
        }
#undef MB_CMAC
        if ((n & 1) && lane == 0) {
            const float zr0 = zr[2 * (n - 1)], zi0 = zr[2 * (n - 1) + 1];
            const float vr = v[2 * (n - 1)], vi = v[2 * (n - 1) + 1];
            ar = fmaf(zr0, vr, fmaf(-zi0, vi, ar));
            ai = fmaf(zr0, vi, fmaf(zi0, vr, ai));
        }
    } else {
        for (int64_t j = lane; j < n; j += 32) {
            const float zr0 = zr[2 * j], zi0 = zr[2 * j + 1], vr = v[2 * j], vi = v[2 * j + 1];
            ar = fmaf(zr0, vr, fmaf(-zi0, vi, ar));
            ai = fmaf(zr0, vi, fmaf(zi0, vr, ai));
        }
    }
    const double sr = warp_sum((double)ar), si = warp_sum((double)ai);
    if (lane == 0) {
        y[2 * row] = sr;
        y[2 * row + 1] = si;
    }
}

// r = b - Z x in FP64 (x, b, r complex128).  One warp per row.
__global__ void __launch_bounds__(256) residual_c128_kernel(const float* __restrict__ z,
                                                            const double* __restrict__ x,
                                                            const double* __restrict__ b, int64_t n,
                                                            double* __restrict__ r) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const float2* z2 = reinterpret_cast<const float2*>(z + 2 * row * n);
    const double2* x2 = reinterpret_cast<const double2*>(x);
    double ar = 0.0, ai = 0.0;
    for (int64_t j = lane; j < n; j += 32) {
        const float2 a = __ldcs(z2 + j);
        const double2 v = __ldg(x2 + j);
        ar = fma((double)a.x, v.x, fma(-(double)a.y, v.y, ar));
        ai = fma((double)a.x, v.y, fma((double)a.y, v.x, ai));
    }
    ar = warp_sum(ar);
    ai = warp_sum(ai);
    if (lane == 0) {
        r[2 * row] = b[2 * row] - ar;
        r[2 * row + 1] = b[2 * row + 1] - ai;
    }
}

// Real matrices (the Laplace collocation system): y = A v with A real [n, n] row-major and
// v complex (the Krylov vectors stay complex; for real data their imaginary parts stay 0).
// A float32: lane reads float4 (four entries) and the matching four complex64 of v.
__global__ void __launch_bounds__(256) matvec_r32_kernel(const float* __restrict__ a,
                                                         const float* __restrict__ v, int64_t n,
                                                         double* __restrict__ y) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const float* ar = a + row * n;
    float sr = 0.f, si = 0.f;
    int64_t done = 0;
    if ((reinterpret_cast<uintptr_t>(ar) & 15) == 0 && (reinterpret_cast<uintptr_t>(v) & 15) == 0) {
        const float4* a4 = reinterpret_cast<const float4*>(ar);
        const float4* v4 = reinterpret_cast<const float4*>(v);
        const int64_t nq = n >> 2;
#define MB_RMAC(A, P)                                                            \
    {                                                                            \
        const float4 u0 = __ldg(v4 + 2 * (P)), u1 = __ldg(v4 + 2 * (P) + 1);     \
        sr = fmaf(A.x, u0.x, fmaf(A.y, u0.z, fmaf(A.z, u1.x, fmaf(A.w, u1.z, sr)))); \
        si = fmaf(A.x, u0.y, fmaf(A.y, u0.w, fmaf(A.z, u1.y, fmaf(A.w, u1.w, si)))); \
    }
        int64_t p = lane;
        for (; p + 96 < nq; p += 128) {
            const float4 a0 = __ldcs(a4 + p), a1 = __ldcs(a4 + p + 32), a2 = __ldcs(a4 + p + 64),
                         a3 = __ldcs(a4 + p + 96);
            MB_RMAC(a0, p) MB_RMAC(a1, p + 32) MB_RMAC(a2, p + 64) MB_RMAC(a3, p + 96)
        }
        for (; p < nq; p += 32) {
            const float4 a0 = __ldcs(a4 + p);
            MB_RMAC(a0, p)
        }
#undef MB_RMAC
        done = nq << 2;
    }
    for (int64_t j = done + lane; j < n; j += 32) {
        sr = fmaf(ar[j], v[2 * j], sr);
        si = fmaf(ar[j], v[2 * j + 1], si);
    }
    const double tr = warp_sum((double)sr), ti = warp_sum((double)si);
    if (lane == 0) {
        y[2 * row] = tr;
        y[2 * row + 1] = ti;
    }
}

// A float64, v complex128 (the FP64 basis vector itself).
__global__ void __launch_bounds__(256) matvec_r64_kernel(const double* __restrict__ a,
                                                         const double* __restrict__ v, int64_t n,
                                                         double* __restrict__ y) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const double* ar = a + row * n;
    const double2* v2 = reinterpret_cast<const double2*>(v);
    double sr = 0.0, si = 0.0;
    int64_t j = lane;
    for (; j + 96 < n; j += 128) {
        const double a0 = __ldcs(ar + j), a1 = __ldcs(ar + j + 32), a2 = __ldcs(ar + j + 64), a3 = __ldcs(ar + j + 96);
        const double2 u0 = __ldg(v2 + j), u1 = __ldg(v2 + j + 32), u2 = __ldg(v2 + j + 64), u3 = __ldg(v2 + j + 96);
        sr = fma(a0, u0.x, fma(a1, u1.x, fma(a2, u2.x, fma(a3, u3.x, sr))));
        si = fma(a0, u0.y, fma(a1, u1.y, fma(a2, u2.y, fma(a3, u3.y, si))));
    }
    for (; j < n; j += 32) {
        const double a0 = __ldcs(ar + j);
        const double2 u0 = __ldg(v2 + j);
        sr = fma(a0, u0.x, sr);
        si = fma(a0, u0.y, si);
    }
    sr = warp_sum(sr);
    si = warp_sum(si);
    if (lane == 0) {
        y[2 * row] = sr;
        y[2 * row + 1] = si;
    }
}

// r = b - A x in FP64 for real A (float32 or float64), x, b, r complex128.
template <typename T>
__global__ void __launch_bounds__(256) residual_real_kernel(const T* __restrict__ a, const double* __restrict__ x,
                                                            const double* __restrict__ b, int64_t n,
                                                            double* __restrict__ r) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const T* ar = a + row * n;
    const double2* x2 = reinterpret_cast<const double2*>(x);
    double sr = 0.0, si = 0.0;
    for (int64_t j = lane; j < n; j += 32) {
        const double aj = (double)__ldcs(ar + j);
        const double2 u = __ldg(x2 + j);
        sr = fma(aj, u.x, sr);
        si = fma(aj, u.y, si);
    }
    sr = warp_sum(sr);
    si = warp_sum(si);
    if (lane == 0) {
        r[2 * row] = b[2 * row] - sr;
        r[2 * row + 1] = b[2 * row + 1] - si;
    }
}

// dst complex128 = (src, 0); and back: dst real = Re(src).
__global__ void real_to_c128_kernel(const double* __restrict__ src, int64_t n, double* __restrict__ dst) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dst[2 * k] = src ? src[k] : 0.0;
    dst[2 * k + 1] = 0.0;
}
__global__ void c128_real_part_kernel(const double* __restrict__ src, int64_t n, double* __restrict__ dst) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dst[k] = src[2 * k];
}

// h[i] += sum_k conj(V[i, k]) w[k] for i < m (FP64); h is interleaved complex, pre-zeroed.
__global__ void __launch_bounds__(256) dots_kernel(const double* __restrict__ V, const double* __restrict__ w,
                                                   int64_t n, int m, double* __restrict__ h) {
    __shared__ double s_re[kGmresMaxRestart + 1][8], s_im[kGmresMaxRestart + 1][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int i = 0; i < m; ++i) {
        const double* vi = V + 2 * (int64_t)i * n;
        double ar = 0.0, ai = 0.0;
        for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
            const double vr = vi[2 * k], vim = vi[2 * k + 1], wr = w[2 * k], wi = w[2 * k + 1];
            ar = fma(vr, wr, fma(vim, wi, ar));
            ai = fma(vr, wi, fma(-vim, wr, ai));
        }
        ar = warp_sum(ar);
        ai = warp_sum(ai);
        if (lane == 0) {
            s_re[i][warp] = ar;
            s_im[i][warp] = ai;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        double sr = 0.0, si = 0.0;
        for (int q = 0; q < 8; ++q) {
            sr += s_re[i][q];
            si += s_im[i][q];
        }
        atomicAdd(h + 2 * i, sr);
        atomicAdd(h + 2 * i + 1, si);
    }
}

// w -= sum_i V[i] h[i]  (h complex128, m entries)
__global__ void subtract_basis_kernel(const double* __restrict__ V, const double* __restrict__ h, int64_t n,
                                      int m, double* __restrict__ w) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double wr = w[2 * k], wi = w[2 * k + 1];
    for (int i = 0; i < m; ++i) {
        const double hr = h[2 * i], hi = h[2 * i + 1];
        const double vr = V[2 * ((int64_t)i * n + k)], vi = V[2 * ((int64_t)i * n + k) + 1];
        wr -= hr * vr - hi * vi;
        wi -= hr * vi + hi * vr;
    }
    w[2 * k] = wr;
    w[2 * k + 1] = wi;
}

// out = sum_i V[i] y[i] added into x (x complex128)
__global__ void add_basis_kernel(const double* __restrict__ V, const double* __restrict__ y, int64_t n, int m,
                                 double* __restrict__ x) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double xr = x[2 * k], xi = x[2 * k + 1];
    for (int i = 0; i < m; ++i) {
        const double yr = y[2 * i], yi = y[2 * i + 1];
        const double vr = V[2 * ((int64_t)i * n + k)], vi = V[2 * ((int64_t)i * n + k) + 1];
        xr += yr * vr - yi * vi;
        xi += yr * vi + yi * vr;
    }
    x[2 * k] = xr;
    x[2 * k + 1] = xi;
}

// sum |w|^2 into *out (pre-zeroed, FP64 atomics)
__global__ void __launch_bounds__(256) norm2_kernel(const double* __restrict__ w, int64_t n, double* __restrict__ out) {
    __shared__ double s[8];
    double a = 0.0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        a = fma(w[2 * k], w[2 * k], fma(w[2 * k + 1], w[2 * k + 1], a));
    a = warp_sum(a);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += s[q];
        atomicAdd(out, t);
    }
}

// dst (complex128) = src * scale; optional complex64 copy
__global__ void scale_kernel(const double* __restrict__ src, double scale, int64_t n, double* __restrict__ dst,
                             float* __restrict__ dst32) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double r = src[2 * k] * scale, i = src[2 * k + 1] * scale;
    if (dst) {
        dst[2 * k] = r;
        dst[2 * k + 1] = i;
    }
    if (dst32) {
        dst32[2 * k] = (float)r;
        dst32[2 * k + 1] = (float)i;
    }
}

// ---------------------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------------------
struct GmresWork {
    double* V;      // [(m+1), n] complex128
    double* w;      // [n] complex128
    double* r;      // [n] complex128
    float* v32;     // [n] complex64
    double* h;      // [2 (m+1)] complex128 (dots), then [1] for norms
    double* nrm;    // [2]
};

constexpr size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

constexpr size_t gmres_ws_bytes(int64_t n, int m) {
    return al256(sizeof(double) * 2 * (size_t)(m + 1) * n) + 2 * al256(sizeof(double) * 2 * n) +
           al256(sizeof(float) * 2 * n) + al256(sizeof(double) * 2 * (m + 2)) + al256(sizeof(double) * 4);
}

size_t gmres_workspace_bytes(int64_t n, int m) { return gmres_ws_bytes(n, m); }

static GmresWork carve(void* ws, int64_t n, int m) {
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    char* p = static_cast<char*>(ws);
    GmresWork g;
    g.V = reinterpret_cast<double*>(p);
    p += al(sizeof(double) * 2 * (size_t)(m + 1) * n);
    g.w = reinterpret_cast<double*>(p);
    p += al(sizeof(double) * 2 * n);
    g.r = reinterpret_cast<double*>(p);
    p += al(sizeof(double) * 2 * n);
    g.v32 = reinterpret_cast<float*>(p);
    p += al(sizeof(float) * 2 * n);
    g.h = reinterpret_cast<double*>(p);
    p += al(sizeof(double) * 2 * (m + 2));
    g.nrm = reinterpret_cast<double*>(p);
    return g;
}

static int sync_check(cudaStream_t s, const char* what) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return check_launch(what);
}

static int norm_of(const double* w, int64_t n, double* d_out, double* h_out, cudaStream_t s) {
    cudaMemsetAsync(d_out, 0, sizeof(double), s);
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    norm2_kernel<<<blocks, 256, 0, s>>>(w, n, d_out);
    cudaMemcpyAsync(h_out, d_out, sizeof(double), cudaMemcpyDeviceToHost, s);
    int rc = sync_check(s, "gmres norm");
    *h_out = std::sqrt(*h_out);
    return rc;
}

// Host-side bookkeeping of one GMRES(m) run (Hessenberg columns, rotations, rhs), sized for m.
struct GmresHost {
    std::complex<double>* H;     // [(m+1) * m]
    std::complex<double>* cs;    // [m]
    std::complex<double>* sn;    // [m]
    std::complex<double>* gvec;  // [m+1]
    std::complex<double>* hcol;  // [m+2]
    std::complex<double>* yv;    // [m]
    double* hbuf;                // [2 (m+1)]
};

// The system matrix: complex64 (kind 0, the RWG impedance matrix), real float32 (1) or real
// float64 (2).
struct GmresMatrix {
    int kind;
    const void* a;
};

static int gmres_core(const GmresMatrix& A, int64_t n, const double* b, double* x, int m, int max_iters,
                      double tol, void* workspace, const GmresHost& hs, int64_t* iters_out,
                      int64_t* cycles_out, double* relres_out, int* status_out, cudaStream_t s);

int gmres_c64(const float* z, int64_t n, const double* b, double* x, int m, int max_iters, double tol,
              void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out,
              double* relres_out, int* status_out, cudaStream_t s) {
    if (n <= 0) return set_error(MB_ERR_ARG, "n must be > 0");
    if (m < 1 || m > kGmresMaxRestart) return set_error(MB_ERR_ARG, "restart must be in [1, %d]", kGmresMaxRestart);
    if (max_iters < 1) return set_error(MB_ERR_ARG, "max_iters must be >= 1");
    if (!(tol > 0)) return set_error(MB_ERR_ARG, "tol must be > 0");
    if (ws_bytes < gmres_workspace_bytes(n, m)) return set_error(MB_ERR_ARG, "workspace too small");
    std::vector<std::complex<double>> H((size_t)(m + 1) * m), cs(m), sn(m), gvec(m + 1), hcol(m + 2), yv(m);
    std::vector<double> hbuf(2 * (m + 1));
    const GmresHost hs{H.data(), cs.data(), sn.data(), gvec.data(), hcol.data(), yv.data(), hbuf.data()};
    return gmres_core(GmresMatrix{0, z}, n, b, x, m, max_iters, tol, workspace, hs, iters_out, cycles_out,
                      relres_out, status_out, s);
}

// Real system A x = b (A float32 or float64 [n, n]; b, x float64 [n]).  The complex core
// runs on complex copies of b and x kept after the complex workspace.
size_t gmres_real_workspace_bytes(int64_t n, int m) { return gmres_ws_bytes(n, m) + 2 * al256(16 * (size_t)n); }

int gmres_real(int kind, const void* a, int64_t n, const double* b, double* x, int m, int max_iters, double tol,
               void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out, double* relres_out,
               int* status_out, cudaStream_t s) {
    if (n <= 0) return set_error(MB_ERR_ARG, "n must be > 0");
    if (m < 1 || m > kGmresMaxRestart) return set_error(MB_ERR_ARG, "restart must be in [1, %d]", kGmresMaxRestart);
    if (max_iters < 1) return set_error(MB_ERR_ARG, "max_iters must be >= 1");
    if (!(tol > 0)) return set_error(MB_ERR_ARG, "tol must be > 0");
    if (ws_bytes < gmres_real_workspace_bytes(n, m)) return set_error(MB_ERR_ARG, "workspace too small");
    char* extra = static_cast<char*>(workspace) + gmres_ws_bytes(n, m);
    double* bc = reinterpret_cast<double*>(extra);
    double* xc = reinterpret_cast<double*>(extra + al256(16 * (size_t)n));
    const unsigned vb = (unsigned)((n + 255) / 256);
    real_to_c128_kernel<<<vb, 256, 0, s>>>(b, n, bc);
    real_to_c128_kernel<<<vb, 256, 0, s>>>(x, n, xc);
    std::vector<std::complex<double>> H((size_t)(m + 1) * m), cs(m), sn(m), gvec(m + 1), hcol(m + 2), yv(m);
    std::vector<double> hbuf(2 * (m + 1));
    const GmresHost hs{H.data(), cs.data(), sn.data(), gvec.data(), hcol.data(), yv.data(), hbuf.data()};
    int rc = gmres_core(GmresMatrix{kind, a}, n, bc, xc, m, max_iters, tol, workspace, hs, iters_out, cycles_out,
                        relres_out, status_out, s);
    if (rc) return rc;
    c128_real_part_kernel<<<vb, 256, 0, s>>>(xc, n, x);
    return sync_check(s, "gmres real result");
}

static int gmres_core(const GmresMatrix& A, int64_t n, const double* b, double* x, int m, int max_iters,
                      double tol, void* workspace, const GmresHost& hs, int64_t* iters_out,
                      int64_t* cycles_out, double* relres_out, int* status_out, cudaStream_t s) {
    GmresWork g = carve(workspace, n, m);
    std::complex<double>* H = hs.H;
    std::complex<double>* cs = hs.cs;
    std::complex<double>* sn = hs.sn;
    std::complex<double>* gvec = hs.gvec;
    double* hbuf = hs.hbuf;
    const int tb = 256;
    const unsigned vblocks = (unsigned)((n + tb - 1) / tb);
    const unsigned rblocks = (unsigned)((n + 7) / 8);
    const int dblocks = (int)std::min<int64_t>((n + 255) / 256, 512);
    int rc;
    double bnorm;
    if ((rc = norm_of(b, n, g.nrm, &bnorm, s))) return rc;
    if (bnorm == 0.0) bnorm = 1.0;
    int64_t iters = 0, cycles = 0;
    double relres = 0.0;
    int status = 1;
    while (true) {
        // FP64 residual of the current iterate
        if (A.kind == 0)
            residual_c128_kernel<<<rblocks, 256, 0, s>>>(static_cast<const float*>(A.a), x, b, n, g.r);
        else if (A.kind == 1)
            residual_real_kernel<float><<<rblocks, 256, 0, s>>>(static_cast<const float*>(A.a), x, b, n, g.r);
        else
            residual_real_kernel<double><<<rblocks, 256, 0, s>>>(static_cast<const double*>(A.a), x, b, n, g.r);
        double beta;
        if ((rc = norm_of(g.r, n, g.nrm, &beta, s))) return rc;
        relres = beta / bnorm;
        if (relres <= tol) {
            status = 0;
            break;
        }
        if (iters >= max_iters) break;
        ++cycles;
        scale_kernel<<<vblocks, tb, 0, s>>>(g.r, 1.0 / beta, n, g.V, g.v32);
        for (int i = 0; i <= m; ++i) gvec[i] = 0.0;
        gvec[0] = beta;
        int j = 0;
        for (; j < m && iters < max_iters; ++j, ++iters) {
            if (A.kind == 0)
                matvec_c64_kernel<<<rblocks, 256, 0, s>>>(static_cast<const float*>(A.a), g.v32, n, g.w);
            else if (A.kind == 1)
                matvec_r32_kernel<<<rblocks, 256, 0, s>>>(static_cast<const float*>(A.a), g.v32, n, g.w);
            else
                matvec_r64_kernel<<<rblocks, 256, 0, s>>>(static_cast<const double*>(A.a),
                                                          g.V + 2 * (int64_t)j * n, n, g.w);
            // CGS2: two passes of h = V^H w; w -= V h
            std::complex<double>* hcol = hs.hcol;
            for (int i = 0; i < j + 2; ++i) hcol[i] = 0.0;
            for (int pass = 0; pass < 2; ++pass) {
                cudaMemsetAsync(g.h, 0, sizeof(double) * 2 * (j + 1), s);
                dots_kernel<<<dblocks, 256, 0, s>>>(g.V, g.w, n, j + 1, g.h);
                subtract_basis_kernel<<<vblocks, tb, 0, s>>>(g.V, g.h, n, j + 1, g.w);
                cudaMemcpyAsync(hbuf, g.h, sizeof(double) * 2 * (j + 1), cudaMemcpyDeviceToHost, s);
                if ((rc = sync_check(s, "gmres arnoldi"))) return rc;
                for (int i = 0; i <= j; ++i) hcol[i] += std::complex<double>(hbuf[2 * i], hbuf[2 * i + 1]);
            }
            double hn;
            if ((rc = norm_of(g.w, n, g.nrm, &hn, s))) return rc;
            hcol[j + 1] = hn;
            // apply previous rotations, then a new one for row j+1
            for (int i = 0; i < j; ++i) {
                const std::complex<double> t = std::conj(cs[i]) * hcol[i] + std::conj(sn[i]) * hcol[i + 1];
                hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
                hcol[i] = t;
            }
            const double a = std::abs(hcol[j]), bb = std::abs(hcol[j + 1]);
            const double rr = std::hypot(a, bb);
            if (rr == 0.0) {
                cs[j] = 1.0;
                sn[j] = 0.0;
            } else {
                cs[j] = hcol[j] / rr;
                sn[j] = hcol[j + 1] / rr;
            }
            hcol[j] = rr;
            hcol[j + 1] = 0.0;
            gvec[j + 1] = -sn[j] * gvec[j];
            gvec[j] = std::conj(cs[j]) * gvec[j];
            for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hcol[i];
            const double est = std::abs(gvec[j + 1]) / bnorm;
            const bool breakdown = hn <= 1e-300;
            if (!breakdown) scale_kernel<<<vblocks, tb, 0, s>>>(g.w, 1.0 / hn, n, g.V + 2 * (int64_t)(j + 1) * n, g.v32);
            if (est <= 0.5 * tol || breakdown) {
                ++j;
                ++iters;
                break;
            }
        }
        // back substitution H y = g (upper triangular j x j), then x += V y
        std::complex<double>* yv = hs.yv;
        for (int i = j - 1; i >= 0; --i) {
            std::complex<double> acc = gvec[i];
            for (int q = i + 1; q < j; ++q) acc -= H[(size_t)i * m + q] * yv[q];
            yv[i] = acc / H[(size_t)i * m + i];
        }
        for (int i = 0; i < j; ++i) {
            hbuf[2 * i] = yv[i].real();
            hbuf[2 * i + 1] = yv[i].imag();
        }
        cudaMemcpyAsync(g.h, hbuf, sizeof(double) * 2 * j, cudaMemcpyHostToDevice, s);
        add_basis_kernel<<<vblocks, tb, 0, s>>>(g.V, g.h, n, j, x);
        if ((rc = sync_check(s, "gmres update"))) return rc;
    }
    if (iters_out) *iters_out = iters;
    if (cycles_out) *cycles_out = cycles;
    if (relres_out) *relres_out = relres;
    if (status_out) *status_out = status;
    return MB_OK;
}

// ---------------------------------------------------------------------------------------
// GMRES without any allocation, for callers that cannot allocate device memory.
//
// The device scratch is a fixed array in this library's own device memory: every GPU
// that loads the library holds it (about 7 MB) until the process exits.  The host-side
// bookkeeping uses per-thread static storage.  Limits: n <= kNoAllocMaxN unknowns,
// restart <= kNoAllocMaxRestart.
// The first call on each device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it for the life of the
// process; make that first call before any stream capture.  Calls after cudaDeviceReset()
// on that device are not supported: the module is loaded again and the cached address
// would be stale.  All calls on a device share the one array and it keeps the
// previous call's contents; the solver writes every scratch value before reading it.
// Calls that overlap on the GPU (other streams, other host threads) race on the array.
// ---------------------------------------------------------------------------------------
constexpr int64_t kNoAllocMaxN = 8192;
constexpr int kNoAllocMaxRestart = 50;
constexpr size_t kNoAllocScratchBytes = gmres_ws_bytes(kNoAllocMaxN, kNoAllocMaxRestart);
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_gmres_scratch[kNoAllocScratchBytes];

static thread_local double tl_H[2 * (kNoAllocMaxRestart + 1) * kNoAllocMaxRestart];
static thread_local double tl_cs[2 * kNoAllocMaxRestart];
static thread_local double tl_sn[2 * kNoAllocMaxRestart];
static thread_local double tl_g[2 * (kNoAllocMaxRestart + 1)];
static thread_local double tl_hcol[2 * (kNoAllocMaxRestart + 2)];
static thread_local double tl_y[2 * kNoAllocMaxRestart];
static thread_local double tl_hbuf[2 * (kNoAllocMaxRestart + 1)];

static std::mutex g_scratch_mu;
static void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_gmres_scratch on the current device (looked up once per device).
static int scratch_for_current_device(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(MB_ERR_UNSUPPORTED, "device ordinal %d too large", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (g_scratch_ptr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_gmres_scratch);
        if (e != cudaSuccess || p == nullptr)
            return set_error(MB_ERR_CUDA, "cudaGetSymbolAddress(gmres scratch): %s", cudaGetErrorString(e));
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return MB_OK;
}

int gmres_c64_noalloc(const float* z, int64_t n, const double* b, double* x, int m, int max_iters, double tol,
                      int64_t* iters_out, int64_t* cycles_out, double* relres_out, int* status_out,
                      cudaStream_t s) {
    if (n <= 0) return set_error(MB_ERR_ARG, "n must be > 0");
    if (n > kNoAllocMaxN)
        return set_error(MB_ERR_SIZE,
                         "mb_gmres_c64_noalloc: n = %lld unknowns exceeds the built-in scratch limit of %lld; "
                         "use mb_gmres_c64 with a caller-owned workspace",
                         (long long)n, (long long)kNoAllocMaxN);
    if (m < 1 || m > kNoAllocMaxRestart)
        return set_error(MB_ERR_SIZE, "mb_gmres_c64_noalloc: restart = %d outside [1, %d]", m, kNoAllocMaxRestart);
    if (max_iters < 1) return set_error(MB_ERR_ARG, "max_iters must be >= 1");
    if (!(tol > 0)) return set_error(MB_ERR_ARG, "tol must be > 0");
    void* ws = nullptr;
    int rc = scratch_for_current_device(&ws);
    if (rc) return rc;
    using cd = std::complex<double>;
    const GmresHost hs{reinterpret_cast<cd*>(tl_H), reinterpret_cast<cd*>(tl_cs), reinterpret_cast<cd*>(tl_sn),
                       reinterpret_cast<cd*>(tl_g), reinterpret_cast<cd*>(tl_hcol), reinterpret_cast<cd*>(tl_y),
                       tl_hbuf};
    return gmres_core(GmresMatrix{0, z}, n, b, x, m, max_iters, tol, ws, hs, iters_out, cycles_out, relres_out,
                      status_out, s);
}

int launch_matvec_c64(const float* z, const float* v, int64_t n, double* y, cudaStream_t s) {
    if (n <= 0) return MB_OK;
    matvec_c64_kernel<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(z, v, n, y);
    return check_launch("matvec_c64");
}

int launch_residual_c128(const float* z, const double* x, const double* b, int64_t n, double* r, cudaStream_t s) {
    if (n <= 0) return MB_OK;
    residual_c128_kernel<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(z, x, b, n, r);
    return check_launch("residual_c128");
}

// ---------------------------------------------------------------------------------------
// Preconditioned GMRES(m) with the whole restart cycle on the device.
//
// Right preconditioning with the sparse approximate inverse M (spai.cu): each cycle solves
// (Z M) u = r0 and updates x += M u, so the residual GMRES minimises is the residual of
// Z x = b itself.  Every cycle starts from the refinement residual b - Z x; the Hessenberg
// matrix, the Givens rotations, the residual estimate, the stopping test, the back
// substitution and x stay in FP64, in one-warp kernels on a device state record.  Sums over
// the vector run as block partials that the last block to finish adds in a fixed order
// (deterministic, no FP64 atomics).  A cycle is a fixed sequence of launches: once the state
// says the cycle has ended, the remaining steps' launches return at once.  With use_graph the
// cycle is captured once as a CUDA graph and replayed; the host reads the state once per
// cycle.
//
// Three matrix kinds:
//   0  complex64 Z: FP32 products; the Krylov basis is complex64 and the Gram-Schmidt
//      products run in FP32 with FP64 sums across lanes and blocks (GB300's FP64 rate would
//      make FP64 Gram-Schmidt a third of a step); the refinement residual is a compensated
//      FP32 dot product -- x split into FP32 hi + lo parts, each product Z_ij x_hi,j made
//      exact by TwoProduct (mul + fma), running sums kept exact by TwoSum, the rounding terms
//      and the x_lo products summed beside them, lane sums combined in FP64 -- accurate to
//      ~1e-13 of sum |Z_ij x_j| at FP32 instruction speed.
//   1  complex128 Z: FP64 products, basis and residual (the FP64 reference solution of the
//      same discretisation).
//   2  as 0, but the Arnoldi products read a half-precision copy of Z (complex FP16 scaled by
//      max |Re, Im Z|, half the bytes of complex64): each inner cycle stops once its residual
//      estimate has dropped by inner_rtol (the copy's ~2e-4 relative error bounds what one
//      cycle can gain) and the next cycle restarts from the complex64 refinement residual.
// ---------------------------------------------------------------------------------------
constexpr int kPgMaxBlocks = 256;
constexpr int kPgRowsPerBlock = 8;   // warps per block in the one-warp-per-row kernels

struct PgState {
    double bn2, bnorm, rn2, beta, relres, tol, hn2, hn, inner_rtol;
    long long iters, max_iters, cycles;
    int m, jdone, active, converged;
    unsigned int cnt;
    int pad;
};

struct PgWork {
    void* V;        // [(m+1), n] basis (complex64 for kinds 0 and 2, complex128 for kind 1)
    void* w;        // [n] product / new basis vector (same type as V)
    double2* r;     // [n] residual, then the cycle's update V y
    double2* z;     // [n] M v (float2 view for kinds 0, 2); x split (float4) at cycle start
    double2* part;  // [blocks, m+1] block partials
    double* npart;  // [blocks]
    PgState* st;
    double2* g;     // [m+1]
    double2* cs;    // [m]
    double2* sn;    // [m]
    double2* H;     // [m, m+1], column j at H[j (m+1) + i]
    double2* y;     // [m]
    double2* h1;    // [m+1] pass-1 projections
    double2* h2;    // [m+1] pass-2 projections
};

static size_t pg_state_bytes(int m) { return al256(sizeof(PgState) + 16 * (size_t)(5 * m + 3 + m * (m + 1))); }

size_t pgmres_workspace_bytes(int64_t n, int m) {
    return al256(16 * (size_t)(m + 1) * n) + 3 * al256(16 * (size_t)n) + al256(16 * (size_t)kPgMaxBlocks * (m + 1)) +
           al256(8 * (size_t)kPgMaxBlocks) + pg_state_bytes(m);
}

static PgWork pg_carve(void* ws, int64_t n, int m) {
    char* p = static_cast<char*>(ws);
    PgWork w;
    w.V = p;
    p += al256(16 * (size_t)(m + 1) * n);
    w.w = p;
    p += al256(16 * (size_t)n);
    w.r = reinterpret_cast<double2*>(p);
    p += al256(16 * (size_t)n);
    w.z = reinterpret_cast<double2*>(p);
    p += al256(16 * (size_t)n);
    w.part = reinterpret_cast<double2*>(p);
    p += al256(16 * (size_t)kPgMaxBlocks * (m + 1));
    w.npart = reinterpret_cast<double*>(p);
    p += al256(8 * (size_t)kPgMaxBlocks);
    w.st = reinterpret_cast<PgState*>(p);
    double2* a = reinterpret_cast<double2*>(p + ((sizeof(PgState) + 15) & ~size_t(15)));
    w.g = a;
    a += m + 1;
    w.cs = a;
    a += m;
    w.sn = a;
    a += m;
    w.H = a;
    a += (size_t)m * (m + 1);
    w.y = a;
    a += m;
    w.h1 = a;
    a += m + 1;
    w.h2 = a;
    return w;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconjmul(double2 a, double2 b) {  // conj(a) b
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 d) {
    const double dd = d.x * d.x + d.y * d.y;
    return make_double2((a.x * d.x + a.y * d.y) / dd, (a.y * d.x - a.x * d.y) / dd);
}
__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }

// basis element type helpers: B = float2 (FP32 arithmetic) or double2 (FP64)
template <typename B>
struct PgB;
template <>
struct PgB<float2> {
    using S = float;
    static __device__ __forceinline__ float2 make(double re, double im) { return make_float2((float)re, (float)im); }
};
template <>
struct PgB<double2> {
    using S = double;
    static __device__ __forceinline__ double2 make(double re, double im) { return make_double2(re, im); }
};

// Adds the blocks' partials npart[0..nblocks) in a fixed order into *out once every block
// has written its own; the counter is left at zero for the next launch.
__device__ __forceinline__ void pg_last_block_sum(double* npart, unsigned* cnt, double* out, unsigned nblocks) {
    __shared__ bool s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(cnt, 1u) == nblocks - 1;
    __syncthreads();
    if (s_last && threadIdx.x < 32) {
        double a = 0.0;
        for (unsigned b = threadIdx.x; b < nblocks; b += 32) a += __ldcg(npart + b);
        a = warp_sum(a);
        if (threadIdx.x == 0) {
            *out = a;
            *cnt = 0;
        }
    }
}

// *out = sum |v_k|^2 (FP64), grid-stride over at most kPgMaxBlocks blocks
__global__ void __launch_bounds__(256) pg_norm2_kernel(const double2* __restrict__ v, int64_t n,
                                                      double* __restrict__ npart, unsigned* cnt, double* out) {
    __shared__ double s[8];
    double a = 0.0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        a += cabs2(v[k]);
    a = warp_sum(a);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += s[q];
        npart[blockIdx.x] = t;
    }
    pg_last_block_sum(npart, cnt, out, gridDim.x);
}

__global__ void pg_init_kernel(PgState* st, double tol, long long max_iters, int m, double inner_rtol) {
    const double b = sqrt(st->bn2);
    st->bnorm = b > 0.0 ? b : 1.0;
    st->tol = tol;
    st->inner_rtol = inner_rtol;
    st->max_iters = max_iters;
    st->m = m;
    st->iters = 0;
    st->cycles = 0;
    st->converged = 0;
    st->active = 0;
    st->jdone = 0;
    st->relres = 0.0;
}

__global__ void pg_cycle_start_kernel(PgState* st, double2* g) {
    const double beta = sqrt(st->rn2);
    st->beta = beta;
    st->relres = beta / st->bnorm;
    st->jdone = 0;
    st->active = 0;
    if (st->relres <= st->tol) {
        st->converged = 1;
        return;
    }
    if (st->iters >= st->max_iters || !(beta > 0.0)) return;
    st->active = 1;
    st->cycles += 1;
    g[0] = make_double2(beta, 0.0);
    for (int i = 1; i <= st->m; ++i) g[i] = make_double2(0.0, 0.0);
}

// V_0 = r / beta (r complex128)
template <typename B>
__global__ void pg_start_basis_kernel(const double2* __restrict__ r, int64_t n, const PgState* __restrict__ st,
                                      B* __restrict__ v0) {
    if (!st->active) return;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double s = 1.0 / st->beta;
    v0[k] = PgB<B>::make(r[k].x * s, r[k].y * s);
}

// V_{j+1} = w / h_{j+1,j}
template <typename B>
__global__ void pg_scale_kernel(const B* __restrict__ w, int64_t n, const PgState* __restrict__ st,
                                B* __restrict__ dst) {
    if (!st->active) return;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    using S = typename PgB<B>::S;
    const S s = (S)(1.0 / st->hn);
    const B v = w[k];
    B o;
    o.x = v.x * s;
    o.y = v.y * s;
    dst[k] = o;
}

// z = M v, one warp per row (lanes over the row's pattern), in the basis' precision (lane
// sums too); z has the basis' type.
template <typename B>
__global__ void __launch_bounds__(256) pg_precond_kernel(const int32_t* __restrict__ cols,
                                                         const float2* __restrict__ vals, int64_t n,
                                                         const B* __restrict__ v, B* __restrict__ z,
                                                         const PgState* __restrict__ st) {
    if (!st->active) return;
    using S = typename PgB<B>::S;
    const int64_t row = (int64_t)blockIdx.x * kPgRowsPerBlock + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    if (!cols) {
        if (lane == 0) z[row] = v[row];
        return;
    }
    S ar = 0, ai = 0;
#pragma unroll
    for (int q = lane; q < MB_SPAI_WIDTH; q += 32) {
        const int32_t c = __ldg(cols + row * MB_SPAI_WIDTH + q);
        if (c >= 0) {
            const float2 mq = __ldg(vals + row * MB_SPAI_WIDTH + q);
            const B x = v[c];
            ar += (S)mq.x * x.x - (S)mq.y * x.y;
            ai += (S)mq.x * x.y + (S)mq.y * x.x;
        }
    }
    // lane sums in the basis' precision: an FP64 shuffle-add tree per row cost ~15 us per
    // apply at 30 720 rows on GB300's FP64 rate
    const S sr = warp_sum(ar), si = warp_sum(ai);
    if (lane == 0) z[row] = PgB<B>::make(sr, si);
}

// w = Z v with Z complex64, v complex64: FP32 products, FP64 lane combination, complex64 w
__global__ void __launch_bounds__(256) pg_matvec_c64_kernel(const float* __restrict__ z, const float2* __restrict__ v,
                                                            int64_t n, float2* __restrict__ w,
                                                            const int* __restrict__ active) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n || !*active) return;
    const float* zr = z + 2 * row * n;
    float ar = 0.f, ai = 0.f;
    if ((n & 1) == 0 && (reinterpret_cast<uintptr_t>(zr) & 15) == 0) {
        const float4* z4 = reinterpret_cast<const float4*>(zr);
        const float4* v4 = reinterpret_cast<const float4*>(v);
        const int64_t npair = n >> 1;
        int64_t p = lane;
#define MB_PGMAC(A, B)                         \
    ar = fmaf(A.x, B.x, fmaf(-A.y, B.y, ar));  \
    ai = fmaf(A.x, B.y, fmaf(A.y, B.x, ai));   \
    ar = fmaf(A.z, B.z, fmaf(-A.w, B.w, ar));  \
    ai = fmaf(A.z, B.w, fmaf(A.w, B.z, ai));
        for (; p + 96 < npair; p += 128) {
            const float4 a0 = __ldcs(z4 + p), a1 = __ldcs(z4 + p + 32), a2 = __ldcs(z4 + p + 64),
                         a3 = __ldcs(z4 + p + 96);
            const float4 b0 = __ldg(v4 + p), b1 = __ldg(v4 + p + 32), b2 = __ldg(v4 + p + 64),
                         b3 = __ldg(v4 + p + 96);
            MB_PGMAC(a0, b0) MB_PGMAC(a1, b1) MB_PGMAC(a2, b2) MB_PGMAC(a3, b3)
        }
        for (; p < npair; p += 32) {
            const float4 a0 = __ldcs(z4 + p), b0 = __ldg(v4 + p);
            MB_PGMAC(a0, b0)
        }
#undef MB_PGMAC
    } else {
        const float2* z2 = reinterpret_cast<const float2*>(zr);
        for (int64_t j = lane; j < n; j += 32) {
            const float2 a = __ldcs(z2 + j), b = __ldg(v + j);
            ar = fmaf(a.x, b.x, fmaf(-a.y, b.y, ar));
            ai = fmaf(a.x, b.y, fmaf(a.y, b.x, ai));
        }
    }
    const double sr = warp_sum((double)ar), si = warp_sum((double)ai);
    if (lane == 0) w[row] = make_float2((float)sr, (float)si);
}

// w = scale * Zh v with Zh the complex FP16 copy (interleaved half pairs), v complex64
__global__ void __launch_bounds__(256) pg_matvec_h16_kernel(const __half2* __restrict__ zh,
                                                            const float* __restrict__ scale,
                                                            const float2* __restrict__ v, int64_t n,
                                                            float2* __restrict__ w, const int* __restrict__ active) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n || !*active) return;
    const __half2* zr = zh + row * n;
    float ar = 0.f, ai = 0.f;
    if ((n & 3) == 0 && (reinterpret_cast<uintptr_t>(zr) & 15) == 0) {
        // four complex entries per 16-byte load
        const uint4* z16 = reinterpret_cast<const uint4*>(zr);
        const float4* v4 = reinterpret_cast<const float4*>(v);
        const int64_t nq = n >> 2;
        for (int64_t p = lane; p < nq; p += 32) {
            const uint4 a = __ldcs(z16 + p);
            const float4 b0 = __ldg(v4 + 2 * p), b1 = __ldg(v4 + 2 * p + 1);
            const float2 z0 = __half22float2(*reinterpret_cast<const __half2*>(&a.x));
            const float2 z1 = __half22float2(*reinterpret_cast<const __half2*>(&a.y));
            const float2 z2 = __half22float2(*reinterpret_cast<const __half2*>(&a.z));
            const float2 z3 = __half22float2(*reinterpret_cast<const __half2*>(&a.w));
            ar = fmaf(z0.x, b0.x, fmaf(-z0.y, b0.y, ar));
            ai = fmaf(z0.x, b0.y, fmaf(z0.y, b0.x, ai));
            ar = fmaf(z1.x, b0.z, fmaf(-z1.y, b0.w, ar));
            ai = fmaf(z1.x, b0.w, fmaf(z1.y, b0.z, ai));
            ar = fmaf(z2.x, b1.x, fmaf(-z2.y, b1.y, ar));
            ai = fmaf(z2.x, b1.y, fmaf(z2.y, b1.x, ai));
            ar = fmaf(z3.x, b1.z, fmaf(-z3.y, b1.w, ar));
            ai = fmaf(z3.x, b1.w, fmaf(z3.y, b1.z, ai));
        }
    } else {
        for (int64_t j = lane; j < n; j += 32) {
            const float2 a = __half22float2(zr[j]), b = __ldg(v + j);
            ar = fmaf(a.x, b.x, fmaf(-a.y, b.y, ar));
            ai = fmaf(a.x, b.y, fmaf(a.y, b.x, ai));
        }
    }
    const double s = (double)*scale;
    const double sr = warp_sum((double)ar), si = warp_sum((double)ai);
    if (lane == 0) w[row] = make_float2((float)(sr * s), (float)(si * s));
}

// y = Z v in FP64 with Z complex128 [n, n]; one warp per row
__global__ void __launch_bounds__(256) matvec_z128_kernel(const double2* __restrict__ z,
                                                          const double2* __restrict__ v, int64_t n,
                                                          double2* __restrict__ y, const int* __restrict__ active) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n || (active && !*active)) return;
    const double2* zr = z + row * n;
    double ar = 0.0, ai = 0.0;
    int64_t j = lane;
    for (; j + 32 < n; j += 64) {
        const double2 a0 = __ldcs(zr + j), a1 = __ldcs(zr + j + 32);
        const double2 b0 = __ldg(v + j), b1 = __ldg(v + j + 32);
        ar = fma(a0.x, b0.x, fma(-a0.y, b0.y, ar));
        ai = fma(a0.x, b0.y, fma(a0.y, b0.x, ai));
        ar = fma(a1.x, b1.x, fma(-a1.y, b1.y, ar));
        ai = fma(a1.x, b1.y, fma(a1.y, b1.x, ai));
    }
    for (; j < n; j += 32) {
        const double2 a0 = __ldcs(zr + j), b0 = __ldg(v + j);
        ar = fma(a0.x, b0.x, fma(-a0.y, b0.y, ar));
        ai = fma(a0.x, b0.y, fma(a0.y, b0.x, ai));
    }
    ar = warp_sum(ar);
    ai = warp_sum(ai);
    if (lane == 0) y[row] = make_double2(ar, ai);
}

// r = b - Z x, Z complex128
__global__ void __launch_bounds__(256) residual_z128_kernel(const double2* __restrict__ z,
                                                            const double2* __restrict__ x,
                                                            const double2* __restrict__ b, int64_t n,
                                                            double2* __restrict__ r) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const double2* zr = z + row * n;
    double ar = 0.0, ai = 0.0;
    for (int64_t j = lane; j < n; j += 32) {
        const double2 a = __ldcs(zr + j), v = __ldg(x + j);
        ar = fma(a.x, v.x, fma(-a.y, v.y, ar));
        ai = fma(a.x, v.y, fma(a.y, v.x, ai));
    }
    ar = warp_sum(ar);
    ai = warp_sum(ai);
    if (lane == 0) r[row] = make_double2(b[row].x - ar, b[row].y - ai);
}

// x (complex128) -> (hi, lo) FP32 parts: xs[k] = (Re hi, Im hi, Re lo, Im lo)
__global__ void pg_split_kernel(const double2* __restrict__ x, int64_t n, float4* __restrict__ xs) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double2 v = x[k];
    const float hr = (float)v.x, hi = (float)v.y;
    xs[k] = make_float4(hr, hi, (float)(v.x - (double)hr), (float)(v.y - (double)hi));
}

// s + t exactly as s' + e on both lanes of a packed pair (Knuth's TwoSum; the explicit
// add / sub .rn.f32x2 instructions keep the compiler from contracting or reordering it)
__device__ __forceinline__ void two_sum2(float2& s, float2 t, float2& e) {
    const float2 u = add2(s, t);
    const float2 bb = sub2(u, s);
    e = add2(sub2(s, sub2(u, bb)), sub2(t, bb));
    s = u;
}

// r = b - Z x with Z complex64 and x given by its FP32 split: compensated FP32 dot products
// (exact products by TwoProduct, exact running sums by TwoSum), lane sums combined in FP64.
__global__ void __launch_bounds__(256) residual_c64x_kernel(const float2* __restrict__ z,
                                                            const float4* __restrict__ xs,
                                                            const double2* __restrict__ b, int64_t n,
                                                            double2* __restrict__ r) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const float2* zr = z + row * n;
    // real and imaginary chains side by side in packed f32x2 instructions (lane x: real,
    // lane y: imaginary), the same operations in the same order as two scalar chains:
    // p1 = a.x (x_r, x_i), p2 = (-a.y x_i, a.y x_r); en = -(rounding error of p), exact
    float2 s = bc(0.f), c = bc(0.f);
    for (int64_t j = lane; j < n; j += 32) {
        const float2 a = __ldcs(zr + j);
        const float4 x = __ldg(xs + j);
        const float2 xh = make_float2(x.x, x.y), xhs = make_float2(x.y, x.x);
        const float2 xl = make_float2(x.z, x.w), xls = make_float2(x.w, x.z);
        const float2 A1 = bc(a.x), A1n = bc(-a.x), A2 = make_float2(-a.y, a.y), A2n = make_float2(a.y, -a.y);
        const float2 p1 = mul2(A1, xh), en1 = fma2(A1n, xh, p1);
        const float2 p2 = mul2(A2, xhs), en2 = fma2(A2n, xhs, p2);
        float2 t1, t2;
        two_sum2(s, p1, t1);
        two_sum2(s, p2, t2);
        c = add2(c, add2(sub2(add2(t1, t2), add2(en1, en2)), fma2(A1, xl, mul2(A2, xls))));
    }
    const double ar = warp_sum((double)s.x + (double)c.x), ai = warp_sum((double)s.y + (double)c.y);
    if (lane == 0) r[row] = make_double2(b[row].x - ar, b[row].y - ai);
}

// h[i] = sum_k conj(V_i[k]) w[k] for i < nb: block (c, g) has warp w on row i = 8 g + w over
// chunk c (products and the warp's lane sums in the basis' precision); the last block to
// finish adds the chunks of every row in FP64 in a fixed order (a warp per row, lanes over
// chunks).
template <typename B>
__global__ void __launch_bounds__(256) pg_dots_kernel(const B* __restrict__ V, const B* __restrict__ w, int64_t n,
                                                      int nb, int64_t chunk, double2* __restrict__ part, int ldp,
                                                      unsigned* cnt, double2* __restrict__ h,
                                                      const int* __restrict__ active) {
    if (!*active) return;
    using S = typename PgB<B>::S;
    __shared__ bool s_last;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.y * 8 + warp;
    const int64_t k0 = (int64_t)blockIdx.x * chunk;
    const int64_t k1 = k0 + chunk < n ? k0 + chunk : n;
    if (i < nb) {
        const B* vi = V + (int64_t)i * n;
        S ar0 = 0, ai0 = 0, ar1 = 0, ai1 = 0;
        int64_t k = k0 + lane;
        for (; k + 32 < k1; k += 64) {
            const B a0 = vi[k], a1 = vi[k + 32], b0 = w[k], b1 = w[k + 32];
            ar0 += a0.x * b0.x + a0.y * b0.y;
            ai0 += a0.x * b0.y - a0.y * b0.x;
            ar1 += a1.x * b1.x + a1.y * b1.y;
            ai1 += a1.x * b1.y - a1.y * b1.x;
        }
        if (k < k1) {
            const B a0 = vi[k], b0 = w[k];
            ar0 += a0.x * b0.x + a0.y * b0.y;
            ai0 += a0.x * b0.y - a0.y * b0.x;
        }
        // lane sums in the basis' precision, chunk partials added in FP64 below
        const double ar = (double)warp_sum(ar0 + ar1), ai = (double)warp_sum(ai0 + ai1);
        if (lane == 0) part[(int64_t)blockIdx.x * ldp + i] = make_double2(ar, ai);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(cnt, 1u) == gridDim.x * gridDim.y - 1;
    __syncthreads();
    if (!s_last) return;
    for (int ii = warp; ii < nb; ii += 8) {
        double sr = 0.0, si = 0.0;
        for (unsigned c = lane; c < gridDim.x; c += 32) {
            const double2 p = __ldcg(part + (int64_t)c * ldp + ii);
            sr += p.x;
            si += p.y;
        }
        sr = warp_sum(sr);
        si = warp_sum(si);
        if (lane == 0) h[ii] = make_double2(sr, si);
    }
    if (threadIdx.x == 0) *cnt = 0;
}

// w -= sum_{i<nb} V_i h_i in the basis' precision (one element per thread, the sum over i
// unrolled by four); with npart, also |w|^2 into *hn2 (FP64 block partials + last block).
template <typename B>
__global__ void __launch_bounds__(128) pg_sub_kernel(const B* __restrict__ V, const double2* __restrict__ h, int64_t n,
                                                     int nb, B* __restrict__ w, double* __restrict__ npart,
                                                     unsigned* cnt, double* hn2, const int* __restrict__ active) {
    if (!*active) return;
    using S = typename PgB<B>::S;
    __shared__ B sh[kGmresMaxRestart + 1];
    __shared__ double s[4];
    for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = PgB<B>::make(h[i].x, h[i].y);
    __syncthreads();
    double a = 0.0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        B x = w[k];
        int i = 0;
        for (; i + 4 <= nb; i += 4) {
            const B v0 = V[(int64_t)i * n + k], v1 = V[(int64_t)(i + 1) * n + k];
            const B v2 = V[(int64_t)(i + 2) * n + k], v3 = V[(int64_t)(i + 3) * n + k];
            const B c0 = sh[i], c1 = sh[i + 1], c2 = sh[i + 2], c3 = sh[i + 3];
            const S pr = (v0.x * c0.x - v0.y * c0.y) + (v1.x * c1.x - v1.y * c1.y) + (v2.x * c2.x - v2.y * c2.y) +
                         (v3.x * c3.x - v3.y * c3.y);
            const S pi = (v0.x * c0.y + v0.y * c0.x) + (v1.x * c1.y + v1.y * c1.x) + (v2.x * c2.y + v2.y * c2.x) +
                         (v3.x * c3.y + v3.y * c3.x);
            x.x -= pr;
            x.y -= pi;
        }
        for (; i < nb; ++i) {
            const B v0 = V[(int64_t)i * n + k], c0 = sh[i];
            x.x -= v0.x * c0.x - v0.y * c0.y;
            x.y -= v0.x * c0.y + v0.y * c0.x;
        }
        w[k] = x;
        a += (double)(x.x * x.x + x.y * x.y);
    }
    if (!npart) return;
    a = warp_sum(a);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) npart[blockIdx.x] = (s[0] + s[1]) + (s[2] + s[3]);
    pg_last_block_sum(npart, cnt, hn2, gridDim.x);
}

// One Arnoldi step's Hessenberg column (one warp): h = h1 + h2 and |w| staged in shared
// memory with the previous rotations; lane 0 applies them, forms the new rotation, updates
// the residual estimate and decides whether the cycle ends.
__global__ void __launch_bounds__(32) pg_givens_kernel(PgState* st, double2* g, double2* cs, double2* sn,
                                                       double2* H, const double2* h1, const double2* h2, int j) {
    if (!st->active) return;
    __shared__ double2 col[kGmresMaxRestart + 1], scs[kGmresMaxRestart], ssn[kGmresMaxRestart];
    const int lane = threadIdx.x;
    const int m = st->m;
    for (int i = lane; i <= j; i += 32) col[i] = make_double2(h1[i].x + h2[i].x, h1[i].y + h2[i].y);
    for (int i = lane; i < j; i += 32) {
        scs[i] = cs[i];
        ssn[i] = sn[i];
    }
    __syncwarp();
    if (lane == 0) {
        const double hn = sqrt(st->hn2);
        st->hn = hn;
        for (int i = 0; i < j; ++i) {
            const double2 a = col[i], b = col[i + 1];
            // t = conj(cs) a + conj(sn) b; b' = -sn a + cs b
            const double2 t1 = cconjmul(scs[i], a), t2 = cconjmul(ssn[i], b);
            const double2 u1 = cmul(ssn[i], a), u2 = cmul(scs[i], b);
            col[i] = make_double2(t1.x + t2.x, t1.y + t2.y);
            col[i + 1] = make_double2(u2.x - u1.x, u2.y - u1.y);
        }
        const double rr = hypot(sqrt(cabs2(col[j])), hn);
        double2 c, sv;
        if (rr == 0.0) {
            c = make_double2(1.0, 0.0);
            sv = make_double2(0.0, 0.0);
        } else {
            c = make_double2(col[j].x / rr, col[j].y / rr);
            sv = make_double2(hn / rr, 0.0);
        }
        cs[j] = c;
        sn[j] = sv;
        col[j] = make_double2(rr, 0.0);
        const double2 gj = g[j];
        const double2 ng = cmul(sv, gj);
        g[j + 1] = make_double2(-ng.x, -ng.y);
        g[j] = cconjmul(c, gj);
        st->iters += 1;
        st->jdone = j + 1;
        const double gres = sqrt(cabs2(g[j + 1]));
        const double stop = fmax(0.5 * st->tol * st->bnorm, st->inner_rtol * st->beta);
        if (gres <= stop || hn <= 1e-300 || st->iters >= st->max_iters || j + 1 == m) st->active = 0;
    }
    __syncwarp();
    for (int i = lane; i <= j; i += 32) H[(int64_t)j * (m + 1) + i] = col[i];
}

// y = R^{-1} g over the cycle's steps, column by column (one warp; g kept in shared memory)
__global__ void __launch_bounds__(32) pg_backsub_kernel(const PgState* st, const double2* H, const double2* g,
                                                        double2* y) {
    __shared__ double2 sg[kGmresMaxRestart + 1];
    const int jd = st->jdone, m = st->m, lane = threadIdx.x;
    for (int r = lane; r < jd; r += 32) sg[r] = g[r];
    __syncwarp();
    for (int i = jd - 1; i >= 0; --i) {
        const double2 yi = cdiv(sg[i], H[(int64_t)i * (m + 1) + i]);
        if (lane == 0) y[i] = yi;
        for (int r = lane; r < i; r += 32) {
            const double2 p = cmul(H[(int64_t)i * (m + 1) + r], yi);
            sg[r].x -= p.x;
            sg[r].y -= p.y;
        }
        __syncwarp();
    }
}

// u = sum_{i < jdone} V_i y_i (FP64)
template <typename B>
__global__ void pg_combine_kernel(const B* __restrict__ V, const double2* __restrict__ y,
                                  const PgState* __restrict__ st, int64_t n, double2* __restrict__ u) {
    const int jd = st->jdone;
    if (jd == 0) return;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double2 a = make_double2(0.0, 0.0);
    for (int i = 0; i < jd; ++i) {
        const B v = V[(int64_t)i * n + k];
        const double2 p = cmul(make_double2(v.x, v.y), y[i]);
        a.x += p.x;
        a.y += p.y;
    }
    u[k] = a;
}

// x += M u (FP64)
__global__ void pg_update_kernel(const int32_t* __restrict__ cols, const float2* __restrict__ vals,
                                 const double2* __restrict__ u, const PgState* __restrict__ st, int64_t n,
                                 double2* __restrict__ x) {
    if (st->jdone == 0) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 d = cols ? spai_row_f64(cols, vals, i, u) : u[i];
    x[i] = make_double2(x[i].x + d.x, x[i].y + d.y);
}

struct PgMatrix {
    int kind;            // 0: complex64, 1: complex128, 2: complex64 + half copy for the products
    const void* z;       // the matrix of the refinement residual
    const __half2* zh;   // kind 2: the half copy
    const float* scale;  // kind 2: its scale (device)
};

template <typename B>
static void pg_cycle_t(const PgMatrix& A, int64_t n, const int32_t* cols, const float2* vals, const double2* b,
                       double2* x, int m, const PgWork& W, unsigned* cnt, cudaStream_t s) {
    const unsigned vb = (unsigned)((n + 255) / 256), rb = (unsigned)((n + 7) / 8);
    const int nblk = (int)std::min<int64_t>(vb, kPgMaxBlocks);
    const int sblk = (int)std::min<int64_t>((n + 127) / 128, kPgMaxBlocks);
    // dot-product chunks: at least 1024 elements, at most kPgMaxBlocks chunks
    int64_t chunk = 1024;
    while ((n + chunk - 1) / chunk > kPgMaxBlocks) chunk *= 2;
    const unsigned nchunk = (unsigned)((n + chunk - 1) / chunk);
    const int* act = &W.st->active;
    B* V = static_cast<B*>(W.V);
    B* w = static_cast<B*>(W.w);
    B* z = reinterpret_cast<B*>(W.z);
    if (A.kind == 1) {
        residual_z128_kernel<<<rb, 256, 0, s>>>(static_cast<const double2*>(A.z), x, b, n, W.r);
    } else {
        pg_split_kernel<<<vb, 256, 0, s>>>(x, n, reinterpret_cast<float4*>(W.z));
        residual_c64x_kernel<<<rb, 256, 0, s>>>(static_cast<const float2*>(A.z),
                                                reinterpret_cast<const float4*>(W.z), b, n, W.r);
    }
    pg_norm2_kernel<<<nblk, 256, 0, s>>>(W.r, n, W.npart, cnt, &W.st->rn2);
    pg_cycle_start_kernel<<<1, 1, 0, s>>>(W.st, W.g);
    pg_start_basis_kernel<B><<<vb, 256, 0, s>>>(W.r, n, W.st, V);
    for (int j = 0; j < m; ++j) {
        const B* vj = V + (int64_t)j * n;
        const dim3 dgrid(nchunk, (unsigned)((j + 1 + 7) / 8));
        pg_precond_kernel<B><<<rb, 256, 0, s>>>(cols, vals, n, vj, z, W.st);
        if constexpr (sizeof(B) == 8) {
            if (A.kind == 2)
                pg_matvec_h16_kernel<<<rb, 256, 0, s>>>(A.zh, A.scale, reinterpret_cast<const float2*>(z), n,
                                                        reinterpret_cast<float2*>(w), act);
            else
                pg_matvec_c64_kernel<<<rb, 256, 0, s>>>(static_cast<const float*>(A.z),
                                                        reinterpret_cast<const float2*>(z), n,
                                                        reinterpret_cast<float2*>(w), act);
        } else {
            matvec_z128_kernel<<<rb, 256, 0, s>>>(static_cast<const double2*>(A.z),
                                                  reinterpret_cast<const double2*>(z), n,
                                                  reinterpret_cast<double2*>(w), act);
        }
        pg_dots_kernel<B><<<dgrid, 256, 0, s>>>(V, w, n, j + 1, chunk, W.part, m + 1, cnt, W.h1, act);
        pg_sub_kernel<B><<<sblk, 128, 0, s>>>(V, W.h1, n, j + 1, w, nullptr, cnt, nullptr, act);
        pg_dots_kernel<B><<<dgrid, 256, 0, s>>>(V, w, n, j + 1, chunk, W.part, m + 1, cnt, W.h2, act);
        pg_sub_kernel<B><<<sblk, 128, 0, s>>>(V, W.h2, n, j + 1, w, W.npart, cnt, &W.st->hn2, act);
        pg_givens_kernel<<<1, 32, 0, s>>>(W.st, W.g, W.cs, W.sn, W.H, W.h1, W.h2, j);
        pg_scale_kernel<B><<<vb, 256, 0, s>>>(w, n, W.st, V + (int64_t)(j + 1) * n);
    }
    pg_backsub_kernel<<<1, 32, 0, s>>>(W.st, W.H, W.g, W.y);
    pg_combine_kernel<B><<<vb, 256, 0, s>>>(V, W.y, W.st, n, W.r);
    pg_update_kernel<<<vb, 256, 0, s>>>(cols, vals, W.r, W.st, n, x);
}

static void pg_cycle(const PgMatrix& A, int64_t n, const int32_t* cols, const float2* vals, const double2* b,
                     double2* x, int m, const PgWork& W, unsigned* cnt, cudaStream_t s) {
    if (A.kind == 1) pg_cycle_t<double2>(A, n, cols, vals, b, x, m, W, cnt, s);
    else pg_cycle_t<float2>(A, n, cols, vals, b, x, m, W, cnt, s);
}

int pgmres(int kind, const void* z, const void* z_half, const float* half_scale, double inner_rtol, int64_t n,
           const int32_t* m_cols, const float* m_vals, const double* b, double* x, int m, int max_iters, double tol,
           bool use_graph, void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out,
           double* relres_out, int* status_out, cudaStream_t s) {
    if (!z || !b || !x || !workspace) return set_error(MB_ERR_ARG, "pgmres: null pointer");
    if (n <= 0) return set_error(MB_ERR_ARG, "n must be > 0");
    if (m < 1 || m > kGmresMaxRestart) return set_error(MB_ERR_ARG, "restart must be in [1, %d]", kGmresMaxRestart);
    if (max_iters < 1) return set_error(MB_ERR_ARG, "max_iters must be >= 1");
    if (!(tol > 0)) return set_error(MB_ERR_ARG, "tol must be > 0");
    if (!(inner_rtol >= 0 && inner_rtol < 1)) return set_error(MB_ERR_ARG, "inner_rtol must be in [0, 1)");
    if ((m_cols == nullptr) != (m_vals == nullptr))
        return set_error(MB_ERR_ARG, "pgmres: give both m_cols and m_vals, or neither");
    if ((z_half == nullptr) != (half_scale == nullptr))
        return set_error(MB_ERR_ARG, "pgmres: give both z_half and half_scale, or neither");
    if (kind == 1 && z_half) return set_error(MB_ERR_ARG, "pgmres: the half copy applies to a complex64 matrix");
    if (ws_bytes < pgmres_workspace_bytes(n, m)) return set_error(MB_ERR_ARG, "workspace too small");
    if (((reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(z)) & 15) != 0)
        return set_error(MB_ERR_ARG, "pgmres: z, b and x must be 16-byte aligned");
    if (z_half && (reinterpret_cast<uintptr_t>(z_half) & 15) != 0)
        return set_error(MB_ERR_ARG, "pgmres: z_half must be 16-byte aligned");
    const PgMatrix A{z_half ? 2 : kind, z, static_cast<const __half2*>(z_half), half_scale};
    PgWork W = pg_carve(workspace, n, m);
    const unsigned vb = (unsigned)((n + 255) / 256);
    const int nblk = (int)std::min<int64_t>(vb, kPgMaxBlocks);
    const float2* vals = reinterpret_cast<const float2*>(m_vals);
    const double2* b2 = reinterpret_cast<const double2*>(b);
    double2* x2 = reinterpret_cast<double2*>(x);
    unsigned* cnt = &W.st->cnt;
    cudaMemsetAsync(W.st, 0, sizeof(PgState), s);
    pg_norm2_kernel<<<nblk, 256, 0, s>>>(b2, n, W.npart, cnt, &W.st->bn2);
    pg_init_kernel<<<1, 1, 0, s>>>(W.st, tol, max_iters, m, z_half ? inner_rtol : 0.0);
    int rc = check_launch("pgmres init");
    if (rc) return rc;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
    };
    if (use_graph) {
        if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return cleanup(), set_error(MB_ERR_CUDA, "pgmres: stream capture failed");
        pg_cycle(A, n, m_cols, vals, b2, x2, m, W, cnt, cap);
        cudaError_t ce = cudaStreamEndCapture(cap, &graph);
        if (ce != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
            return cleanup(), set_error(MB_ERR_CUDA, "pgmres: graph capture / instantiate failed");
    }
    PgState hs{};
    const long long max_cycles = (long long)max_iters + 2;
    for (long long c = 0; c < max_cycles; ++c) {
        if (use_graph) {
            if (cudaGraphLaunch(exec, s) != cudaSuccess)
                return cleanup(), set_error(MB_ERR_CUDA, "pgmres: graph launch failed");
        } else {
            pg_cycle(A, n, m_cols, vals, b2, x2, m, W, cnt, s);
        }
        cudaMemcpyAsync(&hs, W.st, sizeof(PgState), cudaMemcpyDeviceToHost, s);
        if ((rc = sync_check(s, "pgmres cycle"))) return cleanup(), rc;
        if (hs.converged || hs.jdone == 0) break;
    }
    cleanup();
    if (iters_out) *iters_out = hs.iters;
    if (cycles_out) *cycles_out = hs.cycles;
    if (relres_out) *relres_out = hs.relres;
    if (status_out) *status_out = hs.converged ? 0 : 1;
    return MB_OK;
}

// ---------------------------------------------------------------------------------------
// half-precision copy of a complex64 matrix for the Arnoldi products of kind 2
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) half_scale_kernel(const float4* __restrict__ z, int64_t n4,
                                                         unsigned* __restrict__ amax_bits) {
    float a = 0.f;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = __ldcs(z + k);
        a = fmaxf(a, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
    if ((threadIdx.x & 31) == 0) atomicMax(amax_bits, __float_as_uint(a));  // a >= 0: bits order as values
}

__global__ void __launch_bounds__(256) half_copy_kernel(const float4* __restrict__ z, int64_t n4,
                                                        const float* __restrict__ scale, uint2* __restrict__ zh) {
    const float s = *scale;
    const float inv = s > 0.f ? 1.f / s : 0.f;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = __ldcs(z + k);
        const __half2 a = __floats2half2_rn(v.x * inv, v.y * inv), b = __floats2half2_rn(v.z * inv, v.w * inv);
        zh[k] = make_uint2(*reinterpret_cast<const unsigned*>(&a), *reinterpret_cast<const unsigned*>(&b));
    }
}

int half_copy_c64(const float* z, int64_t count, void* zh, float* scale, cudaStream_t s) {
    if (!z || !zh || !scale) return set_error(MB_ERR_ARG, "half copy: null pointer");
    if (count <= 0) return set_error(MB_ERR_ARG, "half copy: count must be > 0");
    if (count & 1) return set_error(MB_ERR_ARG, "half copy: count must be even (pairs of complex entries)");
    if (((reinterpret_cast<uintptr_t>(z) & 15) | (reinterpret_cast<uintptr_t>(zh) & 7)) != 0)
        return set_error(MB_ERR_ARG, "half copy: z must be 16-byte and z_half 8-byte aligned");
    const int64_t n4 = count / 2;  // float4 = two complex entries
    const unsigned blocks = (unsigned)std::min<int64_t>((n4 + 255) / 256, 152 * 16);
    cudaMemsetAsync(scale, 0, sizeof(float), s);
    half_scale_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const float4*>(z), n4,
                                             reinterpret_cast<unsigned*>(scale));
    half_copy_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const float4*>(z), n4, scale, static_cast<uint2*>(zh));
    return check_launch("half_copy_c64");
}

}  // namespace mb
