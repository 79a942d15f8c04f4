// laplace_sym.cu -- 3D Laplace boundary operators with the symmetric 7-point rule and
// closed-form singular integrals: an accurate mode next to the reference's quadrature
// (laplace.cu), needed by the Neumann / mixed problems whose hypersingular operator the
// reference never implemented, and by the single-layer collocation system.
//
// Galerkin (P0 / P1), for every ordered face pair (fy, fx) -- fy the "y" face whose normal
// the double layer uses, as in the reference (integrations_3d.py:367, 412-415):
//     out[fy, fx, a, b] = int_{fy} int_{fx} phi_a(y) phi_b(x) k(x, y) dS_x dS_y
//     k = 1/(4 pi R)  (single layer)   or   n_y.(x - y)/(4 pi R^3)  (double layer).
// Separated pairs (no shared vertex): 7 x 7 points, FP32 or FP64 as the output type, the
// pair's coordinates moved to the first vertex of fy.  Pairs sharing a vertex (self, edge-
// and vertex-adjacent): 7 points on fx and the inner integral over fy in closed form, in
// FP64 (closed_form.cuh).  P1 inner integrals use that a hat function is affine:
//     phi_a(y) = phi_a~(x) + grad phi_a . (y - x),   grad phi_a = n x (P_{a+2} - P_{a+1}) / (2A),
// so int phi_a / R = phi_a~(x) I0 + grad phi_a . I1 and, with d = n.(x - P0),
//     int phi_a n.(x - y)/R^3 = -phi_a~(x) Omega + d grad phi_a . J.
//
// Collocation (P0 single layer): A[i, j] = int_{T_j} 1/(4 pi |c_i - y|) dS_y at the
// centroid c_i of face i, 7 points (FP32 / FP64) or closed form (FP64) when i and j share
// a vertex.  Each thread keeps one source triangle and sweeps 16 collocation rows.
#include <cuda_runtime.h>
#include <stdint.h>

#include "closed_form.cuh"
#include "common.cuh"
#include "packed.cuh"

namespace mb {

constexpr int kSymThreads = 128;

__device__ __forceinline__ float rcp_sqrt(float x) { return rsqrtf(x); }
// FP64 1/sqrt(x): the FP32 estimate refined by two Newton steps r <- r (3 - x r^2) / 2
// (quadratic convergence: ~2^-23 -> 2^-46 -> below double rounding).
__device__ __forceinline__ double rcp_sqrt(double x) {
    double r = (double)rsqrtf((float)x);
    r = r * (1.5 - 0.5 * x * r * r);
    r = r * (1.5 - 0.5 * x * r * r);
    return r;
}


__device__ __forceinline__ bool share_vertex(const int32_t* f, int64_t p, int64_t q) {
    const int32_t a0 = __ldg(f + 3 * p), a1 = __ldg(f + 3 * p + 1), a2 = __ldg(f + 3 * p + 2);
    const int32_t b0 = __ldg(f + 3 * q), b1 = __ldg(f + 3 * q + 1), b2 = __ldg(f + 3 * q + 2);
    return (a0 == b0) | (a0 == b1) | (a0 == b2) | (a1 == b0) | (a1 == b1) | (a1 == b2) | (a2 == b0) |
           (a2 == b1) | (a2 == b2);
}

template <typename T, int LAYER, int NPHI>
__global__ void __launch_bounds__(kSymThreads)
    lap_sym_far_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces, int64_t nf,
                       int64_t row_begin, int64_t col_blocks, T* __restrict__ out) {
    __shared__ T s_rule[7][4];   // barycentric coordinates and weight of the 7-point rule
    __shared__ T s_y[7][4];      // source points (shifted) and weights w_j A_y
    __shared__ T s_n[3];
    __shared__ __align__(16) T s_out[kSymThreads * 9];
    const int64_t row_local = (int64_t)blockIdx.x / col_blocks;
    const int64_t fy = row_begin + row_local;
    const int64_t col0 = ((int64_t)blockIdx.x % col_blocks) * kSymThreads;
    const int64_t fx = col0 + threadIdx.x;
    const V3<T> o = load3(verts, __ldg(faces + 3 * fy));
    const V3<T> Y1 = load3(verts, __ldg(faces + 3 * fy + 1)) - o;
    const V3<T> Y2 = load3(verts, __ldg(faces + 3 * fy + 2)) - o;
    if (threadIdx.x < 7) {
        const int j = threadIdx.x;
        s_rule[j][0] = (T)c_d7[j][0];
        s_rule[j][1] = (T)c_d7[j][1];
        s_rule[j][2] = (T)c_d7[j][2];
        s_rule[j][3] = (T)c_d7[j][3];
        const V3<T> nr = cross(Y1, Y2 - Y1);
        const T ay = T(0.5) * sqrt_t(dot(nr, nr));
        const V3<T> y = (T)c_d7[j][1] * Y1 + (T)c_d7[j][2] * Y2;
        s_y[j][0] = y.x;
        s_y[j][1] = y.y;
        s_y[j][2] = y.z;
        s_y[j][3] = (T)c_d7[j][3] * ay;
        if (j == 0) {
            const T inv = rsqrt_t(dot(nr, nr));
            s_n[0] = nr.x * inv;
            s_n[1] = nr.y * inv;
            s_n[2] = nr.z * inv;
        }
    }
    __syncthreads();
    constexpr int nn = NPHI * NPHI;
    T acc[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) acc[c] = 0;
    if (fx < nf && !share_vertex(faces, fy, fx)) {
        const V3<T> X0 = load3(verts, __ldg(faces + 3 * fx)) - o;
        const V3<T> X1 = load3(verts, __ldg(faces + 3 * fx + 1)) - o;
        const V3<T> X2 = load3(verts, __ldg(faces + 3 * fx + 2)) - o;
        const V3<T> nx = cross(X1 - X0, X2 - X1);
        const T ax = T(0.5) * sqrt_t(dot(nx, nx));
        const V3<T> ny = v3<T>(s_n[0], s_n[1], s_n[2]);
#pragma unroll 1
        for (int i = 0; i < 7; ++i) {
            const V3<T> x = s_rule[i][0] * X0 + s_rule[i][1] * X1 + s_rule[i][2] * X2;
            T s0 = 0, s1 = 0, s2 = 0;
#pragma unroll
            for (int j = 0; j < 7; ++j) {
                const V3<T> d = x - v3<T>(s_y[j][0], s_y[j][1], s_y[j][2]);
                const T ri = rcp_sqrt(dot(d, d));
                T g = ri * s_y[j][3];
                if constexpr (LAYER == 2) g *= ri * ri;
                if constexpr (NPHI == 3) {
                    s0 += g * s_rule[j][0];
                    s1 += g * s_rule[j][1];
                    s2 += g * s_rule[j][2];
                } else {
                    s0 += g;
                }
            }
            if constexpr (LAYER == 2) {
                const T dn = dot(x, ny);  // n_y.(x - y_j): the shifted y_j lie in the plane through 0
                s0 *= dn;
                s1 *= dn;
                s2 *= dn;
            }
            const T wx = s_rule[i][3] * ax;
            if constexpr (NPHI == 3) {
                const T sa[3] = {s0, s1, s2};
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b) acc[3 * a + b] += sa[a] * (wx * s_rule[i][b]);
            } else {
                acc[0] += s0 * wx;
            }
        }
#pragma unroll
        for (int c = 0; c < 9; ++c) acc[c] *= T(kInv4Pi);
    }
#pragma unroll
    for (int c = 0; c < nn; ++c) s_out[threadIdx.x * nn + c] = acc[c];
    __syncthreads();
    const int64_t valid = (nf - col0) < kSymThreads ? (nf - col0) : kSymThreads;
    const int64_t base = (row_local * nf + col0) * nn;
    const int64_t n_out = valid * nn;
    for (int64_t c = threadIdx.x; c < n_out; c += kSymThreads) out[base + c] = s_out[c];
}

__device__ __forceinline__ V3<double> load3d(const float* p, int64_t i) {
    return v3<double>(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
__device__ __forceinline__ V3<double> load3d(const double* p, int64_t i) {
    return v3<double>(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

// Pairs sharing a vertex, FP64, one thread per listed pair (fy, fx); overwrites the entry.
template <typename T>
__global__ void lap_sym_near_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces, int64_t nf,
                                    const int32_t* __restrict__ pairs, int64_t n_pairs, int layer, int nphi,
                                    int64_t row_begin, int64_t row_end, T* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_pairs) return;
    const int64_t fy = pairs[2 * t], fx = pairs[2 * t + 1];
    if (fy < row_begin || fy >= row_end) return;
    V3<double> P[3], Q[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        P[v] = load3d(verts, faces[3 * fy + v]);
        Q[v] = load3d(verts, faces[3 * fx + v]);
    }
    const V3<double> ny2 = cross(P[1] - P[0], P[2] - P[1]);
    const double two_ay = sqrt(dot(ny2, ny2));
    const V3<double> ny = (1.0 / two_ay) * ny2;
    const V3<double> nx2 = cross(Q[1] - Q[0], Q[2] - Q[1]);
    const double ax = 0.5 * sqrt(dot(nx2, nx2));
    V3<double> grad[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) grad[a] = (1.0 / two_ay) * cross(ny, P[(a + 2) % 3] - P[(a + 1) % 3]);
    const V3<double> cy = (1.0 / 3.0) * (P[0] + P[1] + P[2]);
    double hmax = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const V3<double> e = P[(a + 1) % 3] - P[a];
        hmax = fmax(hmax, sqrt(dot(e, e)));
    }
    const double dtol = 1e-10 * hmax;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 7; ++i) {
        const V3<double> x = c_d7[i][0] * Q[0] + c_d7[i][1] * Q[1] + c_d7[i][2] * Q[2];
        const double wx = c_d7[i][3] * ax;
        double sa[3];
        if (layer == 1) {
            double I0;
            V3<double> I1;
            potential_integrals(x, P, &I0, &I1);
            if (nphi == 3) {
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    sa[a] = (1.0 / 3.0 + dot(grad[a], x - cy)) * I0 + dot(grad[a], I1);
            } else {
                sa[0] = I0;
            }
        } else {
            double om, d;
            V3<double> J;
            dl_integrals(x, P, dtol, &om, &J, &d);
            if (nphi == 3) {
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    sa[a] = -(1.0 / 3.0 + dot(grad[a], x - cy)) * om + d * dot(grad[a], J);
            } else {
                sa[0] = -om;
            }
        }
        if (nphi == 3) {
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) acc[3 * a + b] += sa[a] * wx * c_d7[i][b];
        } else {
            acc[0] += sa[0] * wx;
        }
    }
    const int nn = nphi * nphi;
    T* o = out + ((fy - row_begin) * nf + fx) * nn;
    for (int c = 0; c < nn; ++c) o[c] = (T)(acc[c] * kInv4Pi);
}

// P0 single-layer collocation at face centroids with the 7-point rule.  A block covers
// kSymThreads source faces j (one per thread) and kColRows consecutive collocation rows i:
// each thread builds its source triangle's 7 points once and evaluates them against the
// kColRows centroids held in shared memory, writing out[(i - row_begin) * nf + j]
// (coalesced per row).  Pairs sharing a vertex are then rewritten by lap_colloc_near_kernel.
constexpr int kColRows = 64;

template <typename T>
__global__ void __launch_bounds__(kSymThreads)
    lap_colloc_sl_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces, int64_t nf,
                         int64_t row_begin, int64_t row_end, T* __restrict__ out) {
    __shared__ T s_c[kColRows][3];
    const int64_t i0 = row_begin + (int64_t)blockIdx.y * kColRows;
    const int64_t j = (int64_t)blockIdx.x * kSymThreads + threadIdx.x;
    for (int t = threadIdx.x; t < kColRows; t += blockDim.x) {
        const int64_t i = i0 + t;
        if (i < row_end) {
            const int32_t a0 = faces[3 * i], a1 = faces[3 * i + 1], a2 = faces[3 * i + 2];
            const V3<T> c = T(1.0 / 3.0) * (load3(verts, a0) + load3(verts, a1) + load3(verts, a2));
            s_c[t][0] = c.x;
            s_c[t][1] = c.y;
            s_c[t][2] = c.z;
        }
    }
    __syncthreads();
    if (j >= nf) return;
    const V3<T> B0 = load3(verts, __ldg(faces + 3 * j));
    const V3<T> E1 = load3(verts, __ldg(faces + 3 * j + 1)) - B0, E2 = load3(verts, __ldg(faces + 3 * j + 2)) - B0;
    const V3<T> nr = cross(E1, E2);
    const T scale = T(0.5) * sqrt_t(dot(nr, nr)) * T(kInv4Pi);
    V3<T> y[7];
    T w[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        y[k] = B0 + ((T)c_d7[k][1] * E1 + (T)c_d7[k][2] * E2);
        w[k] = (T)c_d7[k][3] * scale;
    }
    // Pairs sharing a vertex are evaluated here too (the value is discarded: the near-pair
    // kernel, launched next on the same stream, overwrites them); the only coincident point,
    // the centroid of a face against its own rule, gives +inf, never a fault.
    const int64_t rows = row_end - i0;
    if constexpr (sizeof(T) == 4) {
        if (rows >= kColRows) {
            // two collocation rows per packed f32x2 instruction (the source points broadcast)
            float2 yx[7], yy[7], yz[7], wk[7];
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                yx[k] = bc(y[k].x);
                yy[k] = bc(y[k].y);
                yz[k] = bc(y[k].z);
                wk[k] = bc(w[k]);
            }
#pragma unroll 2
            for (int r = 0; r < kColRows; r += 2) {
                const float2 cx = make_float2(s_c[r][0], s_c[r + 1][0]);
                const float2 cy = make_float2(s_c[r][1], s_c[r + 1][1]);
                const float2 cz = make_float2(s_c[r][2], s_c[r + 1][2]);
                float2 acc = bc(0.f);
#pragma unroll
                for (int k = 0; k < 7; ++k) {
                    const float2 dx = sub2(yx[k], cx), dy = sub2(yy[k], cy), dz = sub2(yz[k], cz);
                    const float2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
                    float2 ri;
                    ri.x = rsqrtf(r2.x);
                    ri.y = rsqrtf(r2.y);
                    acc = fma2(wk[k], ri, acc);
                }
                out[(i0 - row_begin + r) * nf + j] = acc.x;
                out[(i0 - row_begin + r + 1) * nf + j] = acc.y;
            }
            return;
        }
    }
    if (rows >= kColRows) {
#pragma unroll 4
        for (int r = 0; r < kColRows; ++r) {
            const V3<T> c = v3<T>(s_c[r][0], s_c[r][1], s_c[r][2]);
            T acc = 0;
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const V3<T> d = y[k] - c;
                acc += w[k] * rcp_sqrt(dot(d, d));
            }
            out[(i0 - row_begin + r) * nf + j] = acc;
        }
    } else {
        for (int r = 0; r < (int)rows; ++r) {
            const V3<T> c = v3<T>(s_c[r][0], s_c[r][1], s_c[r][2]);
            T acc = 0;
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const V3<T> d = y[k] - c;
                acc += w[k] * rcp_sqrt(dot(d, d));
            }
            out[(i0 - row_begin + r) * nf + j] = acc;
        }
    }
}

// Collocation pairs sharing a vertex (listed as (i, j)): closed form in FP64.
template <typename T>
__global__ void lap_colloc_near_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces, int64_t nf,
                                       const int32_t* __restrict__ pairs, int64_t n_pairs, int64_t row_begin,
                                       int64_t row_end, T* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_pairs) return;
    const int64_t i = pairs[2 * t], j = pairs[2 * t + 1];
    if (i < row_begin || i >= row_end) return;
    V3<double> P[3];
    V3<double> c = v3<double>(0, 0, 0);
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        P[v] = load3d(verts, faces[3 * j + v]);
        c = c + (1.0 / 3.0) * load3d(verts, faces[3 * i + v]);
    }
    double I0;
    V3<double> I1;
    potential_integrals(c, P, &I0, &I1);
    out[(i - row_begin) * nf + j] = (T)(I0 * kInv4Pi);
}

template <typename T>
int launch_laplace_sym(const T* verts, const int32_t* faces, int64_t nf, int layer, int order,
                       const int32_t* pairs, int64_t n_pairs, int64_t row_begin, int64_t row_end, T* out,
                       cudaStream_t s) {
    if (nf <= 0 || row_end <= row_begin) return MB_OK;
    if (layer != 1 && layer != 2) return set_error(MB_ERR_ARG, "layer must be 1 (single) or 2 (double)");
    if (order != 0 && order != 1) return set_error(MB_ERR_ARG, "order must be 0 or 1");
    const int nphi = order == 1 ? 3 : 1;
    const int64_t col_blocks = (nf + kSymThreads - 1) / kSymThreads;
    const int64_t blocks = (row_end - row_begin) * col_blocks;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
#define MB_FAR(LY, NP)                                                                                   \
    lap_sym_far_kernel<T, LY, NP><<<(unsigned)blocks, kSymThreads, 0, s>>>(verts, faces, nf, row_begin, \
                                                                            col_blocks, out)
    if (layer == 1 && nphi == 1) MB_FAR(1, 1);
    else if (layer == 1) MB_FAR(1, 3);
    else if (nphi == 1) MB_FAR(2, 1);
    else MB_FAR(2, 3);
#undef MB_FAR
    if (n_pairs > 0) {
        lap_sym_near_kernel<T><<<(unsigned)((n_pairs + 127) / 128), 128, 0, s>>>(
            verts, faces, nf, pairs, n_pairs, layer, nphi, row_begin, row_end, out);
    }
    return check_launch("laplace_sym");
}
template int launch_laplace_sym<float>(const float*, const int32_t*, int64_t, int, int, const int32_t*, int64_t,
                                       int64_t, int64_t, float*, cudaStream_t);
template int launch_laplace_sym<double>(const double*, const int32_t*, int64_t, int, int, const int32_t*,
                                        int64_t, int64_t, int64_t, double*, cudaStream_t);

template <typename T>
int launch_laplace_colloc_sl(const T* verts, const int32_t* faces, int64_t nf, const int32_t* pairs,
                             int64_t n_pairs, int64_t row_begin, int64_t row_end, T* out, cudaStream_t s) {
    if (nf <= 0 || row_end <= row_begin) return MB_OK;
    const int64_t gx = (nf + kSymThreads - 1) / kSymThreads;
    const int64_t gy = (row_end - row_begin + kColRows - 1) / kColRows;
    if (gx > 0x7fffffffLL || gy > 65535) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
    lap_colloc_sl_kernel<T><<<dim3((unsigned)gx, (unsigned)gy), kSymThreads, 0, s>>>(verts, faces, nf, row_begin,
                                                                                      row_end, out);
    if (n_pairs > 0)
        lap_colloc_near_kernel<T><<<(unsigned)((n_pairs + 127) / 128), 128, 0, s>>>(verts, faces, nf, pairs, n_pairs,
                                                                                   row_begin, row_end, out);
    return check_launch("laplace_colloc_sl");
}
template int launch_laplace_colloc_sl<float>(const float*, const int32_t*, int64_t, const int32_t*, int64_t,
                                             int64_t, int64_t, float*, cudaStream_t);
template int launch_laplace_colloc_sl<double>(const double*, const int32_t*, int64_t, const int32_t*, int64_t,
                                              int64_t, int64_t, double*, cudaStream_t);

}  // namespace mb
