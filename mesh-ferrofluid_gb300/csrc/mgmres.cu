// mgmres.cu -- GMRES(restart) for many right-hand sides in lockstep, Z X = B, with every
// Arnoldi step's m matrix-vector products done as one tensor-core product Z [v_1 .. v_m]
// (mb_cgemm_tf32x3, FP32-class accuracy) instead of m HBM-bound matvecs.
//
// Each column is an independent GMRES process (its own Hessenberg matrix, Givens rotations
// and residual estimate); only the product with Z is shared.  The Krylov basis, the
// Gram-Schmidt coefficients (CGS2, two passes) and the Givens rotations are FP64 / complex128
// on the device; a column whose estimate reaches tol / 2, or whose new basis vector
// vanishes, stops (its later basis vectors are zero) while the others continue.  Every
// restart cycle starts from the residual B - Z X computed with the same product on the
// complex64 rounding of X, so the attainable relative residual is that product's accuracy
// (~1e-6).  The host loop synchronises once per Arnoldi step (the active-column count).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace mb {

size_t cgemm_workspace_bytes(int64_t n, int64_t m);
int cgemm_tf32x3(const float* z_hi, const float* z_lo, int64_t n, const float* x, int64_t m, float* y, void* ws,
                 size_t ws_bytes, cudaStream_t s);

constexpr int kMgMaxRestart = 128;

struct MgWork {
    double* V;      // [(r+1), n, m] complex128
    double* w;      // [n, m] complex128
    float* v32;     // [n, m] complex64 (GEMM input)
    float* y32;     // [n, m] complex64 (GEMM output)
    void* gemm_ws;  // cgemm workspace
    double* H;      // [(r+1), r, m] complex128: H[i][j][c]
    double* hc;     // [(r+1), m] complex128 (one CGS pass)
    double* cs;     // [r, m] complex128
    double* sn;     // [r, m] complex128
    double* g;      // [(r+1), m] complex128
    double* yv;     // [r, m] complex128
    double* beta;   // [m]
    double* bnorm;  // [m]
    double* hn;     // [m]
    int* active;    // [m]
    int* jend;      // [m]
    int* count;     // [4]
};

static size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

static size_t mg_layout(int64_t n, int64_t m, int r, void* base, MgWork* W) {
    const size_t nm = (size_t)n * m;
    size_t off = 0;
    char* p = static_cast<char*>(base);
    auto take = [&](size_t bytes) {
        void* at = p ? p + off : nullptr;
        off += a256(bytes);
        return at;
    };
    W->V = static_cast<double*>(take(16 * nm * (r + 1)));
    W->w = static_cast<double*>(take(16 * nm));
    W->v32 = static_cast<float*>(take(8 * nm));
    W->y32 = static_cast<float*>(take(8 * nm));
    W->gemm_ws = take(cgemm_workspace_bytes(n, m));
    W->H = static_cast<double*>(take(16 * (size_t)(r + 1) * r * m));
    W->hc = static_cast<double*>(take(16 * (size_t)(r + 1) * m));
    W->cs = static_cast<double*>(take(16 * (size_t)r * m));
    W->sn = static_cast<double*>(take(16 * (size_t)r * m));
    W->g = static_cast<double*>(take(16 * (size_t)(r + 1) * m));
    W->yv = static_cast<double*>(take(16 * (size_t)r * m));
    W->beta = static_cast<double*>(take(8 * m));
    W->bnorm = static_cast<double*>(take(8 * m));
    W->hn = static_cast<double*>(take(8 * m));
    W->active = static_cast<int*>(take(4 * m));
    W->jend = static_cast<int*>(take(4 * m));
    W->count = static_cast<int*>(take(16));
    return off;
}

size_t gmres_multi_workspace_bytes(int64_t n, int64_t m, int r) {
    MgWork W;
    return mg_layout(n, m, r, nullptr, &W);
}

// ---- kernels ---------------------------------------------------------------------------
__global__ void mg_to_c64(const double* __restrict__ src, int64_t count, float* __restrict__ dst) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

__global__ void mg_widen(const float* __restrict__ src, int64_t count, double* __restrict__ dst) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

// R = B - Y (Y complex64 from the product), written into V_0; per-column |R|^2 into beta.
__global__ void mg_residual(const double* __restrict__ b, const float* __restrict__ y, int64_t n, int64_t m,
                            double* __restrict__ r, double* __restrict__ sq) {
    const int64_t c = (int64_t)blockIdx.x * 32 + threadIdx.x;
    double acc = 0.0;
    if (c < m) {
        for (int64_t k = blockIdx.y * blockDim.y + threadIdx.y; k < n; k += (int64_t)gridDim.y * blockDim.y) {
            const int64_t e = 2 * (k * m + c);
            const double re = b[e] - (double)y[e], im = b[e + 1] - (double)y[e + 1];
            r[e] = re;
            r[e + 1] = im;
            acc += re * re + im * im;
        }
    }
    __shared__ double s[8][33];
    s[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && c < m) {
        double t = 0.0;
        for (int q = 0; q < (int)blockDim.y; ++q) t += s[q][threadIdx.x];
        atomicAdd(sq + c, t);
    }
}

// per-column |x|^2 of a complex128 [n, m] block into sq (pre-zeroed)
__global__ void mg_colnorm2(const double* __restrict__ x, int64_t n, int64_t m, double* __restrict__ sq) {
    const int64_t c = (int64_t)blockIdx.x * 32 + threadIdx.x;
    double acc = 0.0;
    if (c < m) {
        for (int64_t k = blockIdx.y * blockDim.y + threadIdx.y; k < n; k += (int64_t)gridDim.y * blockDim.y) {
            const int64_t e = 2 * (k * m + c);
            acc += x[e] * x[e] + x[e + 1] * x[e + 1];
        }
    }
    __shared__ double s[8][33];
    s[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && c < m) {
        double t = 0.0;
        for (int q = 0; q < (int)blockDim.y; ++q) t += s[q][threadIdx.x];
        atomicAdd(sq + c, t);
    }
}

// hc[i][c] += sum_k conj(V[i][k][c]) w[k][c] for i < nb (pre-zeroed); grid.z = i.
__global__ void mg_dots(const double* __restrict__ V, const double* __restrict__ w, int64_t n, int64_t m,
                        double* __restrict__ hc) {
    const int64_t c = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.z;
    double ar = 0.0, ai = 0.0;
    if (c < m) {
        const double* vi = V + 2 * (size_t)i * n * m;
        for (int64_t k = blockIdx.y * blockDim.y + threadIdx.y; k < n; k += (int64_t)gridDim.y * blockDim.y) {
            const int64_t e = 2 * (k * m + c);
            const double vr = vi[e], vim = vi[e + 1], wr = w[e], wi = w[e + 1];
            ar = fma(vr, wr, fma(vim, wi, ar));
            ai = fma(vr, wi, fma(-vim, wr, ai));
        }
    }
    __shared__ double sr[8][33], si[8][33];
    sr[threadIdx.y][threadIdx.x] = ar;
    si[threadIdx.y][threadIdx.x] = ai;
    __syncthreads();
    if (threadIdx.y == 0 && c < m) {
        double tr = 0.0, ti = 0.0;
        for (int q = 0; q < (int)blockDim.y; ++q) {
            tr += sr[q][threadIdx.x];
            ti += si[q][threadIdx.x];
        }
        atomicAdd(hc + 2 * ((int64_t)i * m + c), tr);
        atomicAdd(hc + 2 * ((int64_t)i * m + c) + 1, ti);
    }
}

// w[k][c] -= sum_{i<nb} V[i][k][c] hc[i][c]
__global__ void mg_subtract(const double* __restrict__ V, const double* __restrict__ hc, int64_t n, int64_t m, int nb,
                            double* __restrict__ w) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * m) return;
    const int64_t c = idx % m;
    double wr = w[2 * idx], wi = w[2 * idx + 1];
    for (int i = 0; i < nb; ++i) {
        const double hr = hc[2 * ((int64_t)i * m + c)], hi = hc[2 * ((int64_t)i * m + c) + 1];
        const double vr = V[2 * ((int64_t)i * n * m + idx)], vi = V[2 * ((int64_t)i * n * m + idx) + 1];
        wr -= hr * vr - hi * vi;
        wi -= hr * vi + hi * vr;
    }
    w[2 * idx] = wr;
    w[2 * idx + 1] = wi;
}

// H[i][j][c] += hc[i][c] for i < nb (accumulates the two CGS passes)
__global__ void mg_accum_h(const double* __restrict__ hc, int nb, int j, int r, int64_t m, double* __restrict__ H) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)nb * m) return;
    const int i = (int)(idx / m);
    const int64_t c = idx % m;
    double* h = H + 2 * (((int64_t)i * r + j) * m + c);
    h[0] += hc[2 * idx];
    h[1] += hc[2 * idx + 1];
}

// One thread per column: H[j+1][j] = |w|, previous rotations applied to column j, a new
// rotation, the residual estimate; inactive columns are left untouched.
__global__ void mg_givens(double* __restrict__ H, double* __restrict__ cs, double* __restrict__ sn,
                          double* __restrict__ g, const double* __restrict__ hn2, const double* __restrict__ bnorm,
                          int j, int r, int64_t m, double tol, int* __restrict__ active, int* __restrict__ jend,
                          int* __restrict__ count) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m || !active[c]) return;
    auto hre = [&](int i) -> double& { return H[2 * (((int64_t)i * r + j) * m + c)]; };
    auto him = [&](int i) -> double& { return H[2 * (((int64_t)i * r + j) * m + c) + 1]; };
    const double hn = sqrt(hn2[c]);
    hre(j + 1) = hn;
    him(j + 1) = 0.0;
    for (int i = 0; i < j; ++i) {
        const double cr = cs[2 * ((int64_t)i * m + c)], ci = cs[2 * ((int64_t)i * m + c) + 1];
        const double sr = sn[2 * ((int64_t)i * m + c)], si = sn[2 * ((int64_t)i * m + c) + 1];
        const double ar = hre(i), ai = him(i), br = hre(i + 1), bi = him(i + 1);
        // t = conj(c) a + conj(s) b ;  b' = -s a + c b
        const double tr = cr * ar + ci * ai + sr * br + si * bi;
        const double ti = cr * ai - ci * ar + sr * bi - si * br;
        const double nbr = -(sr * ar - si * ai) + (cr * br - ci * bi);
        const double nbi = -(sr * ai + si * ar) + (cr * bi + ci * br);
        hre(i) = tr;
        him(i) = ti;
        hre(i + 1) = nbr;
        him(i + 1) = nbi;
    }
    const double ar = hre(j), ai = him(j), br = hre(j + 1), bi = him(j + 1);
    const double rr = sqrt(ar * ar + ai * ai + br * br + bi * bi);
    double cr = 1.0, ci = 0.0, sr = 0.0, si = 0.0;
    if (rr > 0.0) {
        cr = ar / rr;
        ci = ai / rr;
        sr = br / rr;
        si = bi / rr;
    }
    cs[2 * ((int64_t)j * m + c)] = cr;
    cs[2 * ((int64_t)j * m + c) + 1] = ci;
    sn[2 * ((int64_t)j * m + c)] = sr;
    sn[2 * ((int64_t)j * m + c) + 1] = si;
    hre(j) = rr;
    him(j) = 0.0;
    hre(j + 1) = 0.0;
    him(j + 1) = 0.0;
    // g[j+1] = -s g[j];  g[j] = conj(c) g[j]
    const double gr = g[2 * ((int64_t)j * m + c)], gi = g[2 * ((int64_t)j * m + c) + 1];
    g[2 * ((int64_t)(j + 1) * m + c)] = -(sr * gr - si * gi);
    g[2 * ((int64_t)(j + 1) * m + c) + 1] = -(sr * gi + si * gr);
    g[2 * ((int64_t)j * m + c)] = cr * gr + ci * gi;
    g[2 * ((int64_t)j * m + c) + 1] = cr * gi - ci * gr;
    const double e1 = g[2 * ((int64_t)(j + 1) * m + c)], e2 = g[2 * ((int64_t)(j + 1) * m + c) + 1];
    const double est = sqrt(e1 * e1 + e2 * e2) / bnorm[c];
    jend[c] = j + 1;
    if (est <= 0.5 * tol || hn <= 1e-300 || j + 1 == r) {
        active[c] = 0;
    } else {
        atomicAdd(count, 1);
    }
}

// V_{j+1} = w / |w| for columns still active (zero otherwise); complex64 copy for the product.
__global__ void mg_next_basis(const double* __restrict__ w, const double* __restrict__ hn2,
                              const int* __restrict__ active, int64_t n, int64_t m, double* __restrict__ vnext,
                              float* __restrict__ v32) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * m) return;
    const int64_t c = idx % m;
    const double s = active[c] ? 1.0 / sqrt(hn2[c]) : 0.0;
    const double re = w[2 * idx] * s, im = w[2 * idx + 1] * s;
    vnext[2 * idx] = re;
    vnext[2 * idx + 1] = im;
    v32[2 * idx] = (float)re;
    v32[2 * idx + 1] = (float)im;
}

// Start of a cycle: V_0 = R / beta, g = (beta, 0, ..), columns below tol inactive.
__global__ void mg_start(double* __restrict__ V0, float* __restrict__ v32, const double* __restrict__ beta2,
                         const double* __restrict__ bnorm, int64_t n, int64_t m, double tol, int* __restrict__ active) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * m) return;
    const int64_t c = idx % m;
    const double beta = sqrt(beta2[c]);
    const bool act = beta / bnorm[c] > tol;
    const double s = act ? 1.0 / beta : 0.0;
    const double re = V0[2 * idx] * s, im = V0[2 * idx + 1] * s;
    V0[2 * idx] = re;
    V0[2 * idx + 1] = im;
    v32[2 * idx] = (float)re;
    v32[2 * idx + 1] = (float)im;
    if (idx < m) active[idx] = act ? 1 : 0;
}

__global__ void mg_init_g(const double* __restrict__ beta2, const double* __restrict__ bnorm, int r, int64_t m,
                          double tol, double* __restrict__ g, int* __restrict__ jend, int* __restrict__ count) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m) return;
    for (int i = 0; i <= r; ++i) {
        g[2 * ((int64_t)i * m + c)] = 0.0;
        g[2 * ((int64_t)i * m + c) + 1] = 0.0;
    }
    const double beta = sqrt(beta2[c]);
    g[2 * c] = beta;
    jend[c] = 0;
    if (beta / bnorm[c] > tol) atomicAdd(count, 1);
}

// back substitution per column (upper-triangular jend x jend), then y into yv
__global__ void mg_backsolve(const double* __restrict__ H, const double* __restrict__ g, const int* __restrict__ jend,
                             int r, int64_t m, double* __restrict__ yv) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m) return;
    const int k = jend[c];
    for (int i = r - 1; i >= k; --i) {
        yv[2 * ((int64_t)i * m + c)] = 0.0;
        yv[2 * ((int64_t)i * m + c) + 1] = 0.0;
    }
    for (int i = k - 1; i >= 0; --i) {
        double ar = g[2 * ((int64_t)i * m + c)], ai = g[2 * ((int64_t)i * m + c) + 1];
        for (int q = i + 1; q < k; ++q) {
            const double hr = H[2 * (((int64_t)i * r + q) * m + c)], hi = H[2 * (((int64_t)i * r + q) * m + c) + 1];
            const double yr = yv[2 * ((int64_t)q * m + c)], yi = yv[2 * ((int64_t)q * m + c) + 1];
            ar -= hr * yr - hi * yi;
            ai -= hr * yi + hi * yr;
        }
        const double dr = H[2 * (((int64_t)i * r + i) * m + c)], di = H[2 * (((int64_t)i * r + i) * m + c) + 1];
        const double den = dr * dr + di * di;
        const double yr = den > 0.0 ? (ar * dr + ai * di) / den : 0.0;
        const double yi = den > 0.0 ? (ai * dr - ar * di) / den : 0.0;
        yv[2 * ((int64_t)i * m + c)] = yr;
        yv[2 * ((int64_t)i * m + c) + 1] = yi;
    }
}

// X += sum_i V_i y_i (per column)
__global__ void mg_update(const double* __restrict__ V, const double* __restrict__ yv, int64_t n, int64_t m, int nb,
                          double* __restrict__ x) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * m) return;
    const int64_t c = idx % m;
    double xr = x[2 * idx], xi = x[2 * idx + 1];
    for (int i = 0; i < nb; ++i) {
        const double yr = yv[2 * ((int64_t)i * m + c)], yi = yv[2 * ((int64_t)i * m + c) + 1];
        const double vr = V[2 * ((int64_t)i * n * m + idx)], vi = V[2 * ((int64_t)i * n * m + idx) + 1];
        xr += yr * vr - yi * vi;
        xi += yr * vi + yi * vr;
    }
    x[2 * idx] = xr;
    x[2 * idx + 1] = xi;
}

// ---- host driver -------------------------------------------------------------------------
static int mg_sync(cudaStream_t s, const char* what) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return check_launch(what);
}

int gmres_multi(const float* z_hi, const float* z_lo, int64_t n, const double* b, double* x, int64_t m, int r,
                int max_iters, double tol, void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out,
                double* max_relres_out, int* status_out, cudaStream_t s) {
    if (n <= 0 || m <= 0) return set_error(MB_ERR_ARG, "n and m must be > 0");
    if (r < 1 || r > kMgMaxRestart) return set_error(MB_ERR_ARG, "restart must be in [1, %d]", kMgMaxRestart);
    if (max_iters < 1 || !(tol > 0)) return set_error(MB_ERR_ARG, "bad max_iters / tol");
    if (ws_bytes < gmres_multi_workspace_bytes(n, m, r)) return set_error(MB_ERR_ARG, "workspace too small");
    MgWork W;
    mg_layout(n, m, r, workspace, &W);
    const int64_t nm = n * m;
    const unsigned eb = (unsigned)((nm + 255) / 256);
    const unsigned cb = (unsigned)((m + 127) / 128);
    const dim3 rblk(32, 8);
    // row blocks per column group: enough blocks to fill the GPU, few FP64 atomics per column
    const unsigned ky = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 63) / 64, (152 * 16 + (m + 31) / 32 - 1) /
                                                                                        ((m + 31) / 32)));
    const dim3 rgrid((unsigned)((m + 31) / 32), ky);
    const size_t gws = cgemm_workspace_bytes(n, m);
    std::vector<double> hb(m);
    int rc;
    // |b| per column
    cudaMemsetAsync(W.bnorm, 0, 8 * m, s);
    mg_colnorm2<<<rgrid, rblk, 0, s>>>(b, n, m, W.bnorm);
    cudaMemcpyAsync(hb.data(), W.bnorm, 8 * m, cudaMemcpyDeviceToHost, s);
    if ((rc = mg_sync(s, "gmres_multi |b|"))) return rc;
    for (auto& v : hb) v = v > 0 ? std::sqrt(v) : 1.0;
    cudaMemcpyAsync(W.bnorm, hb.data(), 8 * m, cudaMemcpyHostToDevice, s);
    int64_t iters = 0, cycles = 0;
    double worst = 0.0;
    int status = 1;
    std::vector<double> hbeta(m);
    while (true) {
        // residual of the current iterate through the tensor-core product
        mg_to_c64<<<eb, 256, 0, s>>>(x, 2 * nm, W.v32);
        if ((rc = cgemm_tf32x3(z_hi, z_lo, n, W.v32, m, W.y32, W.gemm_ws, gws, s))) return rc;
        cudaMemsetAsync(W.beta, 0, 8 * m, s);
        mg_residual<<<rgrid, rblk, 0, s>>>(b, W.y32, n, m, W.V, W.beta);
        cudaMemcpyAsync(hbeta.data(), W.beta, 8 * m, cudaMemcpyDeviceToHost, s);
        if ((rc = mg_sync(s, "gmres_multi residual"))) return rc;
        worst = 0.0;
        for (int64_t c = 0; c < m; ++c) worst = std::max(worst, std::sqrt(hbeta[c]) / hb[c]);
        if (worst <= tol) {
            status = 0;
            break;
        }
        if (iters >= max_iters) break;
        ++cycles;
        cudaMemsetAsync(W.count, 0, 16, s);
        mg_start<<<eb, 256, 0, s>>>(W.V, W.v32, W.beta, W.bnorm, n, m, tol, W.active);
        mg_init_g<<<cb, 128, 0, s>>>(W.beta, W.bnorm, r, m, tol, W.g, W.jend, W.count);
        cudaMemsetAsync(W.H, 0, 16 * (size_t)(r + 1) * r * m, s);
        int j = 0;
        for (; j < r && iters < max_iters; ++j, ++iters) {
            if ((rc = cgemm_tf32x3(z_hi, z_lo, n, W.v32, m, W.y32, W.gemm_ws, gws, s))) return rc;
            mg_widen<<<eb, 256, 0, s>>>(W.y32, 2 * nm, W.w);  // w (complex128) <- product
            for (int pass = 0; pass < 2; ++pass) {
                cudaMemsetAsync(W.hc, 0, 16 * (size_t)(j + 1) * m, s);
                mg_dots<<<dim3((unsigned)((m + 31) / 32), ky, (unsigned)(j + 1)), rblk, 0, s>>>(W.V, W.w, n, m, W.hc);
                mg_subtract<<<eb, 256, 0, s>>>(W.V, W.hc, n, m, j + 1, W.w);
                mg_accum_h<<<(unsigned)(((j + 1) * m + 255) / 256), 256, 0, s>>>(W.hc, j + 1, j, r, m, W.H);
            }
            cudaMemsetAsync(W.hn, 0, 8 * m, s);
            mg_colnorm2<<<rgrid, rblk, 0, s>>>(W.w, n, m, W.hn);
            cudaMemsetAsync(W.count, 0, 4, s);
            mg_givens<<<cb, 128, 0, s>>>(W.H, W.cs, W.sn, W.g, W.hn, W.bnorm, j, r, m, tol, W.active, W.jend,
                                         W.count);
            mg_next_basis<<<eb, 256, 0, s>>>(W.w, W.hn, W.active, n, m, W.V + 2 * (size_t)(j + 1) * nm, W.v32);
            int alive = 0;
            cudaMemcpyAsync(&alive, W.count, 4, cudaMemcpyDeviceToHost, s);
            if ((rc = mg_sync(s, "gmres_multi arnoldi"))) return rc;
            if (alive == 0) {
                ++j;
                ++iters;
                break;
            }
        }
        mg_backsolve<<<cb, 128, 0, s>>>(W.H, W.g, W.jend, r, m, W.yv);
        mg_update<<<eb, 256, 0, s>>>(W.V, W.yv, n, m, j, x);
        if ((rc = mg_sync(s, "gmres_multi update"))) return rc;
    }
    if (iters_out) *iters_out = iters;
    if (cycles_out) *cycles_out = cycles;
    if (max_relres_out) *max_relres_out = worst;
    if (status_out) *status_out = status;
    return MB_OK;
}

}  // namespace mb
