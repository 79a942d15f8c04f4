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

static size_t mg_layout(int64_t n, int64_t m, int r, size_t prod_ws, void* base, MgWork* W) {
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
    W->gemm_ws = prod_ws ? take(prod_ws) : nullptr;
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
    return mg_layout(n, m, r, cgemm_workspace_bytes(n, m), nullptr, &W);
}

size_t gmres_blockdiag_workspace_bytes(int64_t n, int64_t m, int r) {
    MgWork W;
    return mg_layout(n, m, r, 0, nullptr, &W);
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
#pragma unroll 4
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
#pragma unroll 4
    for (int i = 0; i < nb; ++i) {
        const double yr = yv[2 * ((int64_t)i * m + c)], yi = yv[2 * ((int64_t)i * m + c) + 1];
        const double vr = V[2 * ((int64_t)i * n * m + idx)], vi = V[2 * ((int64_t)i * n * m + idx) + 1];
        xr += yr * vr - yi * vi;
        xi += yr * vi + yi * vr;
    }
    x[2 * idx] = xr;
    x[2 * idx + 1] = xi;
}

// ---- block-diagonal product (many meshes) ------------------------------------------------
// desc[i] = (face offset, faces, edges E_i, offset of Z_i in the flat array (complex entries),
// -, first right-hand-side column); goff[i] = first warp of mesh i (each warp owns ROWS rows,
// goff[n_mesh] = total warps).  y[r, col + c] = sum_l Z_i[r, l] x[l, col + c] for the NC
// columns of mesh i; x, y: [rows_max, ld] interleaved complex64; FP32 products, FP32 lane
// sums, warp reduction.  Rows of the padded block beyond E_i are never written.
__device__ __forceinline__ int seg_of(const int64_t* __restrict__ off, int n, int64_t v) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int ROWS, int NC>
__global__ void __launch_bounds__(256) blockdiag_matvec_kernel(const float* __restrict__ z,
                                                               const int64_t* __restrict__ desc,
                                                               const int64_t* __restrict__ goff, int n_mesh,
                                                               const float* __restrict__ x, int64_t ld,
                                                               float* __restrict__ y) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= __ldg(goff + n_mesh)) return;
    const int i = seg_of(goff, n_mesh, w);
    const int64_t E = __ldg(desc + 6 * i + 2), zo = __ldg(desc + 6 * i + 3), co = __ldg(desc + 6 * i + 5);
    const int64_t r0 = (w - __ldg(goff + i)) * ROWS;
    const float2* zc = reinterpret_cast<const float2*>(z) + zo;
    const float2* xc = reinterpret_cast<const float2*>(x);
    float ar[ROWS][NC], ai[ROWS][NC];
#pragma unroll
    for (int q = 0; q < ROWS; ++q)
#pragma unroll
        for (int c = 0; c < NC; ++c) ar[q][c] = ai[q][c] = 0.f;
    // the NC complex64 of x[l, co ..] are contiguous: 16-byte loads when NC is even
    const bool vec = (NC % 2 == 0) && ((ld & 1) == 0) && ((co & 1) == 0);
#pragma unroll 2
    for (int64_t l = lane; l < E; l += 32) {
        float2 xv[NC];
        if (vec) {
            const float4* x4 = reinterpret_cast<const float4*>(xc + l * ld + co);
#pragma unroll
            for (int c = 0; c < NC / 2; ++c) {
                const float4 t = __ldg(x4 + c);
                xv[2 * c] = make_float2(t.x, t.y);
                xv[2 * c + 1] = make_float2(t.z, t.w);
            }
        } else {
#pragma unroll
            for (int c = 0; c < NC; ++c) xv[c] = __ldg(xc + l * ld + co + c);
        }
#pragma unroll
        for (int q = 0; q < ROWS; ++q) {
            if (r0 + q < E) {
                const float2 a = __ldcs(zc + (r0 + q) * E + l);
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    ar[q][c] = fmaf(a.x, xv[c].x, fmaf(-a.y, xv[c].y, ar[q][c]));
                    ai[q][c] = fmaf(a.x, xv[c].y, fmaf(a.y, xv[c].x, ai[q][c]));
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < ROWS; ++q)
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            float vr = ar[q][c], vi = ai[q][c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                vr += __shfl_xor_sync(0xffffffffu, vr, o);
                vi += __shfl_xor_sync(0xffffffffu, vi, o);
            }
            if (lane == 0 && r0 + q < E)
                reinterpret_cast<float2*>(y)[(r0 + q) * ld + co + c] = make_float2(vr, vi);
        }
}

int blockdiag_matvec(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                     const float* x, int64_t ld, int nc, int rows, float* y, cudaStream_t s) {
    if (n_mesh <= 0 || total_warps <= 0) return MB_OK;
    const int64_t blocks = (total_warps * 32 + 255) / 256;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "batch too large for one launch");
#define MB_BD(R, C)                                                                                           \
    if (rows == R && nc == C) {                                                                               \
        blockdiag_matvec_kernel<R, C><<<(unsigned)blocks, 256, 0, s>>>(z, desc, goff, n_mesh, x, ld, y);      \
        return check_launch("blockdiag_matvec");                                                              \
    }
    MB_BD(1, 1) MB_BD(2, 1) MB_BD(4, 1) MB_BD(8, 1)
    MB_BD(1, 2) MB_BD(2, 2) MB_BD(4, 2) MB_BD(8, 2)
    MB_BD(1, 4) MB_BD(2, 4) MB_BD(4, 4) MB_BD(8, 4)
    MB_BD(1, 8) MB_BD(2, 8) MB_BD(4, 8)
#undef MB_BD
    return set_error(MB_ERR_UNSUPPORTED, "block-diagonal product: rows per warp in {1, 2, 4, 8} (8 with up to 4 "
                                         "columns), columns per mesh in {1, 2, 4, 8}");
}

// ---- host driver -------------------------------------------------------------------------
static int mg_sync(cudaStream_t s, const char* what) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return check_launch(what);
}

// The lockstep driver.  prod(v32, y32, stream) computes Y = Z V for the [n, m] complex64 blocks.
// With use_graph, the r Arnoldi steps of a cycle are captured once as a CUDA graph and
// replayed every cycle (no host synchronisation inside a cycle; a cycle always runs its r
// steps, columns that converged early are inactive).
template <typename Prod>
static int gmres_lockstep(Prod prod, int64_t n, const double* b, double* x, int64_t m, int r, int max_iters,
                          double tol, size_t prod_ws, void* workspace, size_t ws_bytes, bool use_graph,
                          int64_t* iters_out, int64_t* cycles_out, double* max_relres_out, int* status_out,
                          cudaStream_t s) {
    if (n <= 0 || m <= 0) return set_error(MB_ERR_ARG, "n and m must be > 0");
    if (r < 1 || r > kMgMaxRestart) return set_error(MB_ERR_ARG, "restart must be in [1, %d]", kMgMaxRestart);
    if (max_iters < 1 || !(tol > 0)) return set_error(MB_ERR_ARG, "bad max_iters / tol");
    MgWork W;
    if (ws_bytes < mg_layout(n, m, r, prod_ws, nullptr, &W)) return set_error(MB_ERR_ARG, "workspace too small");
    mg_layout(n, m, r, prod_ws, workspace, &W);
    const int64_t nm = n * m;
    const unsigned eb = (unsigned)((nm + 255) / 256);
    const unsigned cb = (unsigned)((m + 127) / 128);
    const dim3 rblk(32, 8);
    // row blocks per column group: enough blocks to fill the GPU, few FP64 atomics per column
    const unsigned ky = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((n + 63) / 64, (152 * 16 + (m + 31) / 32 - 1) / ((m + 31) / 32)));
    const dim3 rgrid((unsigned)((m + 31) / 32), ky);
    std::vector<double> hb(m);
    int rc;
    cudaMemsetAsync(W.y32, 0, 8 * (size_t)nm, s);  // rows a product does not write stay 0
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
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;  // capture needs a stream other than the legacy default stream
    auto step = [&](int j, cudaStream_t st) -> int {
        int e;
        if ((e = prod(W.v32, W.y32, st))) return e;
        mg_widen<<<eb, 256, 0, st>>>(W.y32, 2 * nm, W.w);
        for (int pass = 0; pass < 2; ++pass) {
            cudaMemsetAsync(W.hc, 0, 16 * (size_t)(j + 1) * m, st);
            mg_dots<<<dim3((unsigned)((m + 31) / 32), ky, (unsigned)(j + 1)), rblk, 0, st>>>(W.V, W.w, n, m, W.hc);
            mg_subtract<<<eb, 256, 0, st>>>(W.V, W.hc, n, m, j + 1, W.w);
            mg_accum_h<<<(unsigned)(((j + 1) * m + 255) / 256), 256, 0, st>>>(W.hc, j + 1, j, r, m, W.H);
        }
        cudaMemsetAsync(W.hn, 0, 8 * m, st);
        mg_colnorm2<<<rgrid, rblk, 0, st>>>(W.w, n, m, W.hn);
        cudaMemsetAsync(W.count, 0, 4, st);
        mg_givens<<<cb, 128, 0, st>>>(W.H, W.cs, W.sn, W.g, W.hn, W.bnorm, j, r, m, tol, W.active, W.jend, W.count);
        mg_next_basis<<<eb, 256, 0, st>>>(W.w, W.hn, W.active, n, m, W.V + 2 * (size_t)(j + 1) * nm, W.v32);
        return check_launch("gmres_multi step");
    };
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
    };
    while (true) {
        // residual of the current iterate through the same product
        mg_to_c64<<<eb, 256, 0, s>>>(x, 2 * nm, W.v32);
        if ((rc = prod(W.v32, W.y32, s))) return cleanup(), rc;
        cudaMemsetAsync(W.beta, 0, 8 * m, s);
        mg_residual<<<rgrid, rblk, 0, s>>>(b, W.y32, n, m, W.V, W.beta);
        cudaMemcpyAsync(hbeta.data(), W.beta, 8 * m, cudaMemcpyDeviceToHost, s);
        if ((rc = mg_sync(s, "gmres_multi residual"))) return cleanup(), rc;
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
        if (use_graph) {
            if (!exec) {
                if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess ||
                    cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                    return cleanup(), set_error(MB_ERR_CUDA, "gmres_multi: stream capture failed");
                int e = MB_OK;
                for (int q = 0; q < r && e == MB_OK; ++q) e = step(q, cap);
                cudaError_t ce = cudaStreamEndCapture(cap, &graph);
                if (e) return cleanup(), e;
                if (ce != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
                    return cleanup(), set_error(MB_ERR_CUDA, "gmres_multi: graph capture / instantiate failed");
            }
            if (cudaGraphLaunch(exec, s) != cudaSuccess)
                return cleanup(), set_error(MB_ERR_CUDA, "gmres_multi: graph launch failed");
            j = r;
            iters += r;
        } else {
            for (; j < r && iters < max_iters; ++j, ++iters) {
                if ((rc = step(j, s))) return cleanup(), rc;
                int alive = 0;
                cudaMemcpyAsync(&alive, W.count, 4, cudaMemcpyDeviceToHost, s);
                if ((rc = mg_sync(s, "gmres_multi arnoldi"))) return cleanup(), rc;
                if (alive == 0) {
                    ++j;
                    ++iters;
                    break;
                }
            }
        }
        mg_backsolve<<<cb, 128, 0, s>>>(W.H, W.g, W.jend, r, m, W.yv);
        mg_update<<<eb, 256, 0, s>>>(W.V, W.yv, n, m, j, x);
        if ((rc = mg_sync(s, "gmres_multi update"))) return cleanup(), rc;
    }
    cleanup();
    if (iters_out) *iters_out = iters;
    if (cycles_out) *cycles_out = cycles;
    if (max_relres_out) *max_relres_out = worst;
    if (status_out) *status_out = status;
    return MB_OK;
}

int gmres_multi(const float* z_hi, const float* z_lo, int64_t n, const double* b, double* x, int64_t m, int r,
                int max_iters, double tol, void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out,
                double* max_relres_out, int* status_out, cudaStream_t s) {
    const size_t gws = cgemm_workspace_bytes(n, m);
    MgWork W;
    if (ws_bytes < mg_layout(n, m, r, gws, nullptr, &W)) return set_error(MB_ERR_ARG, "workspace too small");
    mg_layout(n, m, r, gws, workspace, &W);
    void* gemm_ws = W.gemm_ws;
    auto prod = [&](const float* v32, float* y32, cudaStream_t st) {
        return cgemm_tf32x3(z_hi, z_lo, n, v32, m, y32, gemm_ws, gws, st);
    };
    return gmres_lockstep(prod, n, b, x, m, r, max_iters, tol, gws, workspace, ws_bytes, false, iters_out,
                          cycles_out, max_relres_out, status_out, s);
}

// Many meshes, each with its own Z_i and nc right-hand sides: the block-diagonal system on
// the padded [n_rows, m] layout (m = n_mesh * nc columns).
int gmres_blockdiag(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                    int rows_per_warp, int nc, int64_t n_rows, const double* b, double* x, int r, int max_iters,
                    double tol, bool use_graph, void* workspace, size_t ws_bytes, int64_t* iters_out,
                    int64_t* cycles_out, double* max_relres_out, int* status_out, cudaStream_t s) {
    const int64_t m = (int64_t)n_mesh * nc;
    auto prod = [&](const float* v32, float* y32, cudaStream_t st) {
        return blockdiag_matvec(z, desc, goff, n_mesh, total_warps, v32, m, nc, rows_per_warp, y32, st);
    };
    return gmres_lockstep(prod, n_rows, b, x, m, r, max_iters, tol, 0, workspace, ws_bytes, use_graph, iters_out,
                          cycles_out, max_relres_out, status_out, s);
}

}  // namespace mb
