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
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <complex>
#include <mutex>
#include <vector>

#include "common.cuh"

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

// y[row] = sum_j Z[row, j] v[j]; Z, v interleaved complex64; y complex128.
// One warp per row; lane l reads float4 (two complex) at 16-byte granularity when both the
// Z row and v start on a 16-byte boundary, else one complex at a time (v may be an
// 8-byte-aligned view such as X[1:n+1] of a complex64 array).
__global__ void __launch_bounds__(256) matvec_c64_kernel(const float* __restrict__ z,
                                                         const float* __restrict__ v, int64_t n,
                                                         double* __restrict__ y) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
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

}  // namespace mb
