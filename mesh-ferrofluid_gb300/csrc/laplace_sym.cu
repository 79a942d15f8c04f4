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

// The 7 x 7-point integral of a separated pair: fy's rule points (shifted to fy's first
// vertex) and weights w_j A_y in s_y, the barycentric rule in s_rule, fx's corners X0..X2 in
// the same shifted frame; acc[3 a + b] (P1) or acc[0] (P0), without the 1 / (4 pi).
template <typename T, int LAYER, int NPHI>
__device__ __forceinline__ void sym_far_pair(const T (*s_rule)[4], const T (*s_y)[4], const V3<T>& ny,
                                             const V3<T>& X0, const V3<T>& X1, const V3<T>& X2, T acc[9]) {
    const V3<T> nx = cross(X1 - X0, X2 - X1);
    const T ax = T(0.5) * sqrt_t(dot(nx, nx));
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
}

// Two separated pairs (fy, fxa) and (fy, fxb) at once in packed f32x2 arithmetic (lane .x
// the first source face, .y the second): the same sums as sym_far_pair with half the FP32
// instructions.  X0..X2 hold both faces' shifted corners per coordinate; acc as in
// sym_far_pair, packed.
template <int LAYER, int NPHI>
__device__ __forceinline__ void sym_far_pair2(const float4 (*s_r4)[2], const float4 (*s_y4)[2], const float3& ny,
                                              const float2 X0[3], const float2 X1[3], const float2 X2[3],
                                              float2 acc[9]) {
    // s_r4[j] = {(r0, r0, r1, r1), (r2, r2, w, w)}, s_y4[j] = {(y.x, y.x, y.y, y.y),
    // (y.z, y.z, wA, wA)}: every value already duplicated, so one 16-byte shared load yields two
    // packed operands and no register moves are needed to broadcast them
    float2 e1[3], e2[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        e1[c] = sub2(X1[c], X0[c]);
        e2[c] = sub2(X2[c], X1[c]);
    }
    const float2 nx0 = fma2(e1[1], e2[2], mul2(bc(-1.f), mul2(e1[2], e2[1])));
    const float2 nx1 = fma2(e1[2], e2[0], mul2(bc(-1.f), mul2(e1[0], e2[2])));
    const float2 nx2 = fma2(e1[0], e2[1], mul2(bc(-1.f), mul2(e1[1], e2[0])));
    const float2 n2 = fma2(nx0, nx0, fma2(nx1, nx1, mul2(nx2, nx2)));
    const float2 ax = make_float2(0.5f * sqrtf(n2.x), 0.5f * sqrtf(n2.y));
#pragma unroll 1
    for (int i = 0; i < 7; ++i) {
        // re-read the tables every outer point instead of holding all 28 of them in registers
        asm volatile("" ::: "memory");
        const float4 ra = s_r4[i][0], rb = s_r4[i][1];
        const float2 r0 = make_float2(ra.x, ra.y), r1 = make_float2(ra.z, ra.w), r2 = make_float2(rb.x, rb.y);
        float2 x[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) x[c] = fma2(r0, X0[c], fma2(r1, X1[c], mul2(r2, X2[c])));
        float2 s0 = bc(0.f), s1 = bc(0.f), s2 = bc(0.f);
#pragma unroll
        for (int j = 0; j < 7; ++j) {
            const float4 ya = s_y4[j][0], yb = s_y4[j][1];
            const float2 dx = sub2(x[0], make_float2(ya.x, ya.y));
            const float2 dy = sub2(x[1], make_float2(ya.z, ya.w));
            const float2 dz = sub2(x[2], make_float2(yb.x, yb.y));
            const float2 d2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
            const float2 ri = make_float2(rsqrtf(d2.x), rsqrtf(d2.y));
            float2 g = mul2(ri, make_float2(yb.z, yb.w));
            if constexpr (LAYER == 2) g = mul2(g, mul2(ri, ri));
            if constexpr (NPHI == 3) {
                const float4 qa = s_r4[j][0], qb = s_r4[j][1];
                s0 = fma2(g, make_float2(qa.x, qa.y), s0);
                s1 = fma2(g, make_float2(qa.z, qa.w), s1);
                s2 = fma2(g, make_float2(qb.x, qb.y), s2);
            } else {
                s0 = add2(s0, g);
            }
        }
        if constexpr (LAYER == 2) {
            const float2 dn = fma2(x[0], bc(ny.x), fma2(x[1], bc(ny.y), mul2(x[2], bc(ny.z))));
            s0 = mul2(s0, dn);
            s1 = mul2(s1, dn);
            s2 = mul2(s2, dn);
        }
        const float2 wx = mul2(make_float2(rb.z, rb.w), ax);
        if constexpr (NPHI == 3) {
            const float2 sa[3] = {s0, s1, s2};
            const float2 rr[3] = {r0, r1, r2};
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const float2 wb = mul2(wx, rr[b]);
#pragma unroll
                for (int a = 0; a < 3; ++a) acc[3 * a + b] = fma2(sa[a], wb, acc[3 * a + b]);
            }
        } else {
            acc[0] = fma2(s0, wx, acc[0]);
        }
    }
}

// Block set-up shared by the panel and packed kernels: the 7-point rule, fy's shifted rule
// points with weights, and fy's unit normal.
template <typename T>
__device__ __forceinline__ void sym_source_setup(const V3<T>& Y1, const V3<T>& Y2, T (*s_rule)[4], T (*s_y)[4],
                                                 T* s_n) {
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
    sym_source_setup(Y1, Y2, s_rule, s_y, s_n);
    __syncthreads();
    constexpr int nn = NPHI * NPHI;
    T acc[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) acc[c] = 0;
    if (fx < nf && !share_vertex(faces, fy, fx)) {
        const V3<T> X0 = load3(verts, __ldg(faces + 3 * fx)) - o;
        const V3<T> X1 = load3(verts, __ldg(faces + 3 * fx + 1)) - o;
        const V3<T> X2 = load3(verts, __ldg(faces + 3 * fx + 2)) - o;
        sym_far_pair<T, LAYER, NPHI>(s_rule, s_y, v3<T>(s_n[0], s_n[1], s_n[2]), X0, X1, X2, acc);
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

// Surface curls (p_{a+1} - p_{a+2}) / (2 A) of the P1 hat functions of a triangle
// (translation invariant, so any common shift of the corners gives the same curls).
template <typename T>
__device__ __forceinline__ void tri_curls(const V3<T>& p0, const V3<T>& p1, const V3<T>& p2, V3<T> c[3]) {
    const V3<T> nr = cross(p1 - p0, p2 - p1);
    const T inv2a = T(1) / sqrt_t(dot(nr, nr));
    c[0] = inv2a * (p1 - p2);
    c[1] = inv2a * (p2 - p0);
    c[2] = inv2a * (p0 - p1);
}

// Packed operators [V, V] without the [F, F, 3, 3] panels: OP 1 single layer, 2 double layer
// (P1 x P1), 3 hypersingular (Maue: curl phi_a(fy) . curl phi_b(fx) times the P0 single
// layer).  One block per test face fy sweeps every source face fx, accumulates the three
// packed rows faces[fy, a] in shared memory (3 V values) and adds them to `packed` at the
// end.  Pairs sharing a vertex are skipped here and added by lap_sym_near_kernel.
template <typename T, int OP>
__global__ void __launch_bounds__(kSymThreads, sizeof(T) == 4 ? (OP == 3 ? 6 : 4) : 1)
    lap_sym_tight_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces, int64_t nf, int64_t nv,
                         int64_t row_begin, T* __restrict__ packed) {
    constexpr int LAYER = OP == 2 ? 2 : 1;
    constexpr int NPHI = OP == 3 ? 1 : 3;
    __shared__ T s_rule[7][4];
    __shared__ T s_y[7][4];
    __shared__ T s_n[3];
    __shared__ float4 s_r4[7][2];  // the same tables with every value duplicated (float path)
    __shared__ float4 s_y4[7][2];
    extern __shared__ __align__(16) unsigned char tight_smem[];
    T* rows = reinterpret_cast<T*>(tight_smem);
    const int64_t fy = row_begin + blockIdx.x;
    const V3<T> o = load3(verts, __ldg(faces + 3 * fy));
    const V3<T> Y1 = load3(verts, __ldg(faces + 3 * fy + 1)) - o;
    const V3<T> Y2 = load3(verts, __ldg(faces + 3 * fy + 2)) - o;
    sym_source_setup(Y1, Y2, s_rule, s_y, s_n);
    for (int64_t j = threadIdx.x; j < 3 * nv; j += blockDim.x) rows[j] = T(0);
    V3<T> cy[3];
    if constexpr (OP == 3) tri_curls(v3<T>(0, 0, 0), Y1, Y2, cy);
    __syncthreads();
    if (threadIdx.x < 7) {
        const int j = threadIdx.x;
        const float r0 = (float)s_rule[j][0], r1 = (float)s_rule[j][1], r2 = (float)s_rule[j][2];
        const float rw = (float)s_rule[j][3];
        s_r4[j][0] = make_float4(r0, r0, r1, r1);
        s_r4[j][1] = make_float4(r2, r2, rw, rw);
        const float y0 = (float)s_y[j][0], y1 = (float)s_y[j][1], y2 = (float)s_y[j][2], yw = (float)s_y[j][3];
        s_y4[j][0] = make_float4(y0, y0, y1, y1);
        s_y4[j][1] = make_float4(y2, y2, yw, yw);
    }
    __syncthreads();
    const V3<T> ny = v3<T>(s_n[0], s_n[1], s_n[2]);
    // each thread sweeps its own strip of consecutive source faces: neighbouring faces share
    // vertices, and lanes of a warp working on neighbours would collide in the shared-memory
    // accumulators (same-address atomics serialise)
    const int64_t strip = (nf + blockDim.x - 1) / blockDim.x;
    const int64_t strip0 = (int64_t)threadIdx.x * strip;
    const int64_t strip1 = strip0 + strip < nf ? strip0 + strip : nf;
    if constexpr (sizeof(T) == 4 && OP != 3) {
        // two source faces per thread and iteration (fxa, fxa + 1), packed arithmetic
        // (the P0 sums of OP 3 are light enough that occupancy matters more)
        const float3 nyf = make_float3(ny.x, ny.y, ny.z);
#pragma unroll 1
        for (int64_t k = 0; k < strip; k += 2) {
            const int64_t fxa = strip0 + k;
            if (fxa >= strip1) break;
            const int64_t fxb_raw = fxa + 1;
            const bool has_b = fxb_raw < strip1;
            const int64_t fxb = has_b ? fxb_raw : fxa;
            const bool use_a = !share_vertex(faces, fy, fxa);
            const bool use_b = has_b && !share_vertex(faces, fy, fxb);
            if (!use_a && !use_b) continue;
            const int32_t va[3] = {__ldg(faces + 3 * fxa), __ldg(faces + 3 * fxa + 1), __ldg(faces + 3 * fxa + 2)};
            const int32_t vb[3] = {__ldg(faces + 3 * fxb), __ldg(faces + 3 * fxb + 1), __ldg(faces + 3 * fxb + 2)};
            float2 X[3][3];  // corner, coordinate
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                const V3<T> pa = load3(verts, va[v]) - o;
                const V3<T> pb = load3(verts, vb[v]) - o;
                X[v][0] = make_float2(pa.x, pb.x);
                X[v][1] = make_float2(pa.y, pb.y);
                X[v][2] = make_float2(pa.z, pb.z);
            }
            float2 acc[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) acc[c] = bc(0.f);
            sym_far_pair2<LAYER, NPHI>(s_r4, s_y4, nyf, X[0], X[1], X[2], acc);
            {
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b) {
                        if (use_a) atomicAdd(rows + a * nv + va[b], acc[3 * a + b].x * T(kInv4Pi));
                        if (use_b) atomicAdd(rows + a * nv + vb[b], acc[3 * a + b].y * T(kInv4Pi));
                    }
            }
        }
    } else {
#pragma unroll 1
    for (int64_t fx = strip0; fx < strip1; ++fx) {
        if (share_vertex(faces, fy, fx)) continue;
        const int32_t vx[3] = {__ldg(faces + 3 * fx), __ldg(faces + 3 * fx + 1), __ldg(faces + 3 * fx + 2)};
        const V3<T> X0 = load3(verts, vx[0]) - o;
        const V3<T> X1 = load3(verts, vx[1]) - o;
        const V3<T> X2 = load3(verts, vx[2]) - o;
        T acc[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) acc[c] = 0;
        sym_far_pair<T, LAYER, NPHI>(s_rule, s_y, ny, X0, X1, X2, acc);
        if constexpr (OP == 3) {
            V3<T> cx[3];
            tri_curls(X0, X1, X2, cx);
            const T w = acc[0] * T(kInv4Pi);
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) atomicAdd(rows + a * nv + vx[b], dot(cy[a], cx[b]) * w);
        } else {
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) atomicAdd(rows + a * nv + vx[b], acc[3 * a + b] * T(kInv4Pi));
        }
    }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        T* dst = packed + (int64_t)__ldg(faces + 3 * fy + a) * nv;
        for (int64_t j = threadIdx.x; j < nv; j += blockDim.x) atomicAdd(dst + j, rows[a * nv + j]);
    }
}

__device__ __forceinline__ V3<double> load3d(const float* p, int64_t i) {
    return v3<double>(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
__device__ __forceinline__ V3<double> load3d(const double* p, int64_t i) {
    return v3<double>(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

// Pairs sharing a vertex; overwrites the entry.  The closed forms run in the output's
// arithmetic T (float outputs: float logs and arctangents, ~1e-7 of each integral, below
// the rounding of the stored value; GB300's FP64 rate is 1/64 of its FP32 rate), on
// coordinates moved to fy's first vertex in FP64 first.  Eight lanes per listed pair
// (fy, fx): lane i < 7 integrates over fy at the i-th point of fx, lane 7 idles, and the
// eight partial blocks are summed by shuffles within the group.  With `packed` set the
// pair's block is added to the packed matrix [nv, nv] instead (op 1 / 2: single / double
// layer P1; op 3: hypersingular from the P0 single layer and the faces' curls).
constexpr int kNearLanes = 8;

template <typename T>
__global__ void __launch_bounds__(128)
    lap_sym_near_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces, int64_t nf,
                        const int32_t* __restrict__ pairs, int64_t n_pairs, int layer, int nphi,
                        int64_t row_begin, int64_t row_end, T* __restrict__ out, int op, int64_t nv,
                        T* __restrict__ packed) {
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t t = gt / kNearLanes;
    const int i = (int)(gt % kNearLanes);
    // every lane of a group sees the same t, so a group leaves (or stays) as a whole
    if (t >= n_pairs) return;
    const int64_t fy = pairs[2 * t], fx = pairs[2 * t + 1];
    if (fy < row_begin || fy >= row_end) return;
    const unsigned gmask = 0xFFu << (threadIdx.x & 24);
    const V3<double> o = load3d(verts, faces[3 * fy]);
    V3<T> P[3], Q[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const V3<double> p = load3d(verts, faces[3 * fy + v]) - o;
        const V3<double> q = load3d(verts, faces[3 * fx + v]) - o;
        P[v] = v3<T>((T)p.x, (T)p.y, (T)p.z);
        Q[v] = v3<T>((T)q.x, (T)q.y, (T)q.z);
    }
    T acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (i < 7) {
        const V3<T> ny2 = cross(P[1] - P[0], P[2] - P[1]);
        const T two_ay = sqrt_t(dot(ny2, ny2));
        const V3<T> ny = (T(1) / two_ay) * ny2;
        const V3<T> nx2 = cross(Q[1] - Q[0], Q[2] - Q[1]);
        const T ax = T(0.5) * sqrt_t(dot(nx2, nx2));
        const V3<T> x = (T)c_d7[i][0] * Q[0] + (T)c_d7[i][1] * Q[1] + (T)c_d7[i][2] * Q[2];
        const T wx = (T)c_d7[i][3] * ax;
        T sa[3] = {0, 0, 0};
        V3<T> grad[3];
        V3<T> cy = v3<T>(0, 0, 0);
        if (nphi == 3) {
#pragma unroll
            for (int a = 0; a < 3; ++a) grad[a] = (T(1) / two_ay) * cross(ny, P[(a + 2) % 3] - P[(a + 1) % 3]);
            cy = T(1.0 / 3.0) * (P[0] + P[1] + P[2]);
        }
        if (layer == 1) {
            T I0;
            V3<T> I1;
            potential_integrals(x, P, &I0, &I1);
            if (nphi == 3) {
#pragma unroll
                for (int a = 0; a < 3; ++a) sa[a] = (T(1.0 / 3.0) + dot(grad[a], x - cy)) * I0 + dot(grad[a], I1);
            } else {
                sa[0] = I0;
            }
        } else {
            T hmax = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const V3<T> e = P[(a + 1) % 3] - P[a];
                hmax = fmax(hmax, sqrt_t(dot(e, e)));
            }
            // in-plane test: 1e-10 of the edge in FP64, 1e-5 in FP32 (its coordinate noise is ~1e-7)
            const T dtol = (sizeof(T) == 4 ? T(1e-5) : T(1e-10)) * hmax;
            T om, d;
            V3<T> J;
            dl_integrals(x, P, dtol, &om, &J, &d);
            if (nphi == 3) {
#pragma unroll
                for (int a = 0; a < 3; ++a) sa[a] = -(T(1.0 / 3.0) + dot(grad[a], x - cy)) * om + d * dot(grad[a], J);
            } else {
                sa[0] = -om;
            }
        }
        if (nphi == 3) {
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) acc[3 * a + b] = sa[a] * wx * (T)c_d7[i][b];
        } else {
            acc[0] = sa[0] * wx;
        }
    }
    const int nn = nphi * nphi;
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        if (c < nn) {
            acc[c] += __shfl_xor_sync(gmask, acc[c], 1);
            acc[c] += __shfl_xor_sync(gmask, acc[c], 2);
            acc[c] += __shfl_xor_sync(gmask, acc[c], 4);
        }
    }
    T mine = acc[0];
#pragma unroll
    for (int c = 1; c < 8; ++c)
        if (i == c) mine = acc[c];
    if (packed == nullptr) {
        T* dst = out + ((fy - row_begin) * nf + fx) * nn;
        if (i < nn) dst[i] = mine * T(kInv4Pi);
        if (i == 0 && nn == 9) dst[8] = acc[8] * T(kInv4Pi);
        return;
    }
    // packed: lane i adds entry (a, b) = (i / 3, i % 3); lane 0 also (2, 2)
    V3<T> cy[3], cx[3];
    if (op == 3) {
        tri_curls(P[0], P[1], P[2], cy);
        tri_curls(Q[0], Q[1], Q[2], cx);
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int c = k == 0 ? i : 8;
        if (k == 1 && i != 0) break;
        const int a = c / 3, b = c % 3;
        const T v = op == 3 ? dot(cy[a], cx[b]) * acc[0] * T(kInv4Pi) : (k == 0 ? mine : acc[8]) * T(kInv4Pi);
        atomicAdd(packed + (int64_t)faces[3 * fy + a] * nv + faces[3 * fx + b], v);
    }
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
        const int64_t near_blocks = (n_pairs * kNearLanes + 127) / 128;
        if (near_blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "near-pair list too long for one launch");
        lap_sym_near_kernel<T><<<(unsigned)near_blocks, 128, 0, s>>>(verts, faces, nf, pairs, n_pairs, layer, nphi,
                                                                     row_begin, row_end, out, 0, 0, nullptr);
    }
    return check_launch("laplace_sym");
}
// Packed operators (op 1 single layer, 2 double layer, 3 hypersingular) for test rows
// [row_begin, row_end), added to packed [nv, nv].
constexpr int64_t kTightSmemMax = 160 * 1024;

template <typename T>
int launch_laplace_sym_tight(const T* verts, const int32_t* faces, int64_t nf, int64_t nv, int op,
                             const int32_t* pairs, int64_t n_pairs, int64_t row_begin, int64_t row_end, T* packed,
                             cudaStream_t s) {
    if (nf <= 0 || row_end <= row_begin) return MB_OK;
    if (op < 1 || op > 3) return set_error(MB_ERR_ARG, "op must be 1 (single), 2 (double) or 3 (hypersingular)");
    const int64_t smem = 3 * nv * (int64_t)sizeof(T);
    if (smem > kTightSmemMax) return set_error(MB_ERR_SIZE, "too many vertices for the packed assembly");
    if (row_end - row_begin > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
    const unsigned blocks = (unsigned)(row_end - row_begin);
#define MB_TIGHT(OP)                                                                                          \
    do {                                                                                                      \
        if (smem > 48 * 1024) {                                                                               \
            const cudaError_t e = cudaFuncSetAttribute(lap_sym_tight_kernel<T, OP>,                          \
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
            if (e != cudaSuccess) return set_error(MB_ERR_CUDA, cudaGetErrorString(e));                     \
        }                                                                                                     \
        lap_sym_tight_kernel<T, OP><<<blocks, kSymThreads, (size_t)smem, s>>>(verts, faces, nf, nv, row_begin, \
                                                                              packed);                        \
    } while (0)
    if (op == 1) MB_TIGHT(1);
    else if (op == 2) MB_TIGHT(2);
    else MB_TIGHT(3);
#undef MB_TIGHT
    if (n_pairs > 0) {
        const int64_t near_blocks = (n_pairs * kNearLanes + 127) / 128;
        if (near_blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "near-pair list too long for one launch");
        lap_sym_near_kernel<T><<<(unsigned)near_blocks, 128, 0, s>>>(
            verts, faces, nf, pairs, n_pairs, op == 2 ? 2 : 1, op == 3 ? 1 : 3, row_begin, row_end, nullptr, op, nv,
            packed);
    }
    return check_launch("laplace_sym_tight");
}
template int launch_laplace_sym_tight<float>(const float*, const int32_t*, int64_t, int64_t, int, const int32_t*,
                                             int64_t, int64_t, int64_t, float*, cudaStream_t);
template int launch_laplace_sym_tight<double>(const double*, const int32_t*, int64_t, int64_t, int,
                                              const int32_t*, int64_t, int64_t, int64_t, double*, cudaStream_t);

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
