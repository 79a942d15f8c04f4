// mom_sym.cu -- EFIE with a symmetric triangle rule and analytic singularity extraction.
//
// A capability the reference does not have (its rule, mom_ref.cu, rotates with each local
// edge and has no singular treatment).  Both triangles use the 7-point degree-5 rule
// (Radon 1948; Dunavant 1985), whose points do not depend on the local edge, so one set
// of 49 kernel evaluations serves all nine RWG entries of a triangle pair:
//   Z_mn += c_m c_n [ jk (Txy - B_n.Tx - A_m.Ty + (A_m.B_n) T0) - (4j/k) T0 ]
// with the pair moments T0 = sum_i W_i S0_i, Tx = sum_i W_i x_i S0_i, Ty = sum_i W_i S1_i,
// Txy = sum_i W_i x_i.S1_i and S0_i = sum_j w_j G(x_i, y_j), S1_i = sum_j w_j G y_j.  The
// integrand terms are the reference's EFIE terms jk G f_m.f_n - (j/k) G div f_m div f_n
// (mesh_MOM_3d.cu:474-480) with its RWG convention (:154-242).
//
// Pairs that share a vertex (self, edge- and vertex-adjacent; ~13 per face) are skipped by
// the FP32 kernel and computed by an FP64 kernel that splits G = 1/(4 pi R) +
// (e^{-jkR} - 1)/(4 pi R): the smooth part with the source rule, the singular part with the
// closed-form potential integrals of D. R. Wilton, S. M. Rao, A. W. Glisson,
// D. H. Schaubert, O. M. Al-Bundak, C. M. Butler, IEEE Trans. AP-32(3):276-281, 1984:
//   int_T 1/R   = sum_i P0_i ln((R+_i + l+_i)/(R-_i + l-_i)) - |d| sum_i (beta+_i - beta-_i)
//   int_T (y-x)/R = 1/2 sum_i u_i [ R0_i^2 ln(...) + l+_i R+_i - l-_i R-_i ] - d n int_T 1/R.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "closed_form.cuh"
#include "common.cuh"
#include "packed.cuh"

namespace mb {

template <typename T>
__device__ __forceinline__ void add_c(T* p, T re, T im);
template <>
__device__ __forceinline__ void add_c<float>(float* p, float re, float im) {
    atomicAdd(reinterpret_cast<float2*>(p), make_float2(re, im));
}
template <>
__device__ __forceinline__ void add_c<double>(double* p, double re, double im) {
    atomicAdd(p, re);
    atomicAdd(p + 1, im);
}

__device__ __forceinline__ int shared_vertices(const int32_t* f, int64_t p, int64_t q) {
    const int32_t a0 = __ldg(f + 3 * p), a1 = __ldg(f + 3 * p + 1), a2 = __ldg(f + 3 * p + 2);
    const int32_t b0 = __ldg(f + 3 * q), b1 = __ldg(f + 3 * q + 1), b2 = __ldg(f + 3 * q + 2);
    return (a0 == b0) + (a0 == b1) + (a0 == b2) + (a1 == b0) + (a1 == b1) + (a1 == b2) + (a2 == b0) +
           (a2 == b1) + (a2 == b2);
}

template <typename T>
__device__ __forceinline__ void rwg_consts(const int32_t* f, int64_t p, const V3<T> P[3], T c[3], T* area) {
    const V3<T> e0 = P[1] - P[0], e1 = P[2] - P[1];
    const V3<T> cr = cross(e0, e1);
    *area = T(0.5) * sqrt_t(dot(cr, cr));
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int32_t i1 = __ldg(f + 3 * p + (e + 1) % 3), i2 = __ldg(f + 3 * p + (e + 2) % 3);
        const V3<T> d = P[(e + 2) % 3] - P[(e + 1) % 3];
        c[e] = (i1 < i2 ? T(1) : T(-1)) * sqrt_t(dot(d, d)) / (T(2) * *area);
    }
}

// ---------------------------------------------------------------------------------------
// separated pairs (no shared vertex): one thread per (test p, source q), 128 q per block
// ---------------------------------------------------------------------------------------
// One separated face pair (p test, q source): the nine RWG entries, accumulated into z
// ([n_edges, n_edges] interleaved complex) at the rows / columns fei gives.
template <typename T>
__device__ __forceinline__ void sym_regular_pair(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                                 const int32_t* __restrict__ fei, int64_t n_edges, T k, int64_t p,
                                                 int64_t q, const T (*s_b)[4], T* __restrict__ z) {
    if (shared_vertices(faces, p, q) != 0) return;  // done by the FP64 near-pair kernel
    const V3<T> o = load3(verts, __ldg(faces + 3 * q));
    V3<T> A[3], B[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        A[v] = load3(verts, __ldg(faces + 3 * p + v)) - o;
        B[v] = load3(verts, __ldg(faces + 3 * q + v)) - o;
    }
    T cm[3], cn[3], ap, aq;
    rwg_consts<T>(faces, p, A, cm, &ap);
    rwg_consts<T>(faces, q, B, cn, &aq);
    V3<T> y[7];
    T wy[7];
#pragma unroll
    for (int j = 0; j < 7; ++j) {
        y[j] = s_b[j][0] * B[0] + s_b[j][1] * B[1] + s_b[j][2] * B[2];
        wy[j] = s_b[j][3] * aq * T(kInv4Pi);
    }
    const T k_turn = k * T(kInv2Pi);
    T t0r = 0, t0i = 0, txr[3] = {0, 0, 0}, txi[3] = {0, 0, 0}, tyr[3] = {0, 0, 0}, tyi[3] = {0, 0, 0};
    T txyr = 0, txyi = 0;
#pragma unroll 1
    for (int i = 0; i < 7; ++i) {
        const V3<T> x = s_b[i][0] * A[0] + s_b[i][1] * A[1] + s_b[i][2] * A[2];
        const T wi = s_b[i][3] * ap;
        T s0r = 0, s0i = 0, s1r[3] = {0, 0, 0}, s1i[3] = {0, 0, 0};
#pragma unroll
        for (int j = 0; j < 7; ++j) {
            const V3<T> d = x - y[j];
            const T r2 = dot(d, d);
            const T rinv = rsqrt_t(r2);
            T sn, cs;
            sincos_turns(k_turn * (r2 * rinv), &sn, &cs);
            const T g = wy[j] * rinv;
            const T gr = g * cs, gi = -g * sn;
            s0r += gr;
            s0i += gi;
            s1r[0] += gr * y[j].x; s1i[0] += gi * y[j].x;
            s1r[1] += gr * y[j].y; s1i[1] += gi * y[j].y;
            s1r[2] += gr * y[j].z; s1i[2] += gi * y[j].z;
        }
        t0r += wi * s0r;
        t0i += wi * s0i;
        const T xs[3] = {x.x, x.y, x.z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            txr[a] += wi * xs[a] * s0r;
            txi[a] += wi * xs[a] * s0i;
            tyr[a] += wi * s1r[a];
            tyi[a] += wi * s1i[a];
        }
        txyr += wi * (xs[0] * s1r[0] + xs[1] * s1r[1] + xs[2] * s1r[2]);
        txyi += wi * (xs[0] * s1i[0] + xs[1] * s1i[1] + xs[2] * s1i[2]);
    }
    const V3<T> Txr = v3<T>(txr[0], txr[1], txr[2]), Txi = v3<T>(txi[0], txi[1], txi[2]);
    const V3<T> Tyr = v3<T>(tyr[0], tyr[1], tyr[2]), Tyi = v3<T>(tyi[0], tyi[1], tyi[2]);
    const T inv_k4 = T(4) / k;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const T amr = dot(A[m], Tyr), ami = dot(A[m], Tyi);
        const int64_t row = __ldg(fei + 3 * p + m);
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const T ab = dot(A[m], B[n]);
            const T fr = txyr - dot(B[n], Txr) - amr + ab * t0r;  // int int (x-A_m).(y-B_n) G
            const T fi = txyi - dot(B[n], Txi) - ami + ab * t0i;
            const T cc = cm[m] * cn[n];
            // jk cc f - (4j/k) cc T0
            const T re = cc * (-k * fi + inv_k4 * t0i);
            const T im = cc * (k * fr - inv_k4 * t0r);
            add_c<T>(z + 2 * (row * n_edges + __ldg(fei + 3 * q + n)), re, im);
        }
    }
}

// float separated pairs, the same entries with packed arithmetic: source points in f32x2
// pairs (3 pairs + the seventh point scalar), coordinates scaled by k so kR = |k x - k y|
// feeds the SFU sine / cosine directly, the weight k w so g = w / R = (k w) / (kR); the
// source moments are accumulated as k sum G y and the 1/k and the sign of Im G (G = gr - j gs)
// are applied once per test point / at the end.  The source side (origin o = its vertex 0)
// is set up once per source face and reused for every test face a thread meets.
struct SymSource {
    V3<float> o;                                // source vertex 0 (absolute)
    V3<float> B[3];                             // source vertices relative to o
    float cn[3];                                // RWG constants of the source edges
    int32_t v[3];                               // vertex ids (shared-vertex test)
    int32_t col[3];                             // RWG edge ids of the source edges
    float2 yx[3], yy[3], yz[3], yw[3];          // 6 source points, k-scaled, packed
    float tx, ty, tz, tw;                       // the seventh point
};

__device__ __forceinline__ void sym_source(const float* __restrict__ verts, const int32_t* __restrict__ faces,
                                           const int32_t* __restrict__ fei, float k, int64_t q,
                                           const float (*s_b)[4], SymSource& S) {
#pragma unroll
    for (int v = 0; v < 3; ++v) S.v[v] = __ldg(faces + 3 * q + v);
    S.o = load3(verts, S.v[0]);
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        S.B[v] = load3(verts, S.v[v]) - S.o;
        S.col[v] = __ldg(fei + 3 * q + v);
    }
    float aq;
    rwg_consts<float>(faces, q, S.B, S.cn, &aq);
#pragma unroll
    for (int j = 0; j < 7; ++j) {
        const V3<float> y = s_b[j][0] * S.B[0] + s_b[j][1] * S.B[1] + s_b[j][2] * S.B[2];
        const float w = s_b[j][3] * aq * float(kInv4Pi) * k;
        if (j < 6) {
            (reinterpret_cast<float*>(&S.yx[j / 2]) + (j & 1))[0] = k * y.x;
            (reinterpret_cast<float*>(&S.yy[j / 2]) + (j & 1))[0] = k * y.y;
            (reinterpret_cast<float*>(&S.yz[j / 2]) + (j & 1))[0] = k * y.z;
            (reinterpret_cast<float*>(&S.yw[j / 2]) + (j & 1))[0] = w;
        } else {
            S.tx = k * y.x;
            S.ty = k * y.y;
            S.tz = k * y.z;
            S.tw = w;
        }
    }
}

// The nine entries of one separated pair: test vertices A (relative to the source origin),
// their RWG constants cm, area ap and RWG edge ids rows.
__device__ __forceinline__ void sym_pair_eval(const SymSource& S, const V3<float> A[3], const float cm[3], float ap,
                                              const int32_t rows[3], float k, int64_t n_edges,
                                              const float (*s_b)[4], float* __restrict__ z) {
    // per pair: t0 = sum_i w_i S0_i, tx = sum_i w_i x_i S0_i, ty' = sum_i w_i S1'_i,
    // txy' = sum_i w_i x_i . S1'_i with S1' = k S1 (S0 = sum_j G, S1 = sum_j G y)
    float t0r = 0.f, t0i = 0.f, txr[3] = {0.f, 0.f, 0.f}, txi[3] = {0.f, 0.f, 0.f};
    float tyr[3] = {0.f, 0.f, 0.f}, tyi[3] = {0.f, 0.f, 0.f}, txyr = 0.f, txyi = 0.f;
#pragma unroll 1
    for (int i = 0; i < 7; ++i) {
        const V3<float> x = s_b[i][0] * A[0] + s_b[i][1] * A[1] + s_b[i][2] * A[2];
        const float wi = s_b[i][3] * ap;
        const float2 X = bc(k * x.x), Y = bc(k * x.y), Zc = bc(k * x.z);
        float2 s0r = bc(0.f), s0s = bc(0.f), sxr = bc(0.f), sxs = bc(0.f), syr = bc(0.f), sys = bc(0.f),
               szr = bc(0.f), szs = bc(0.f);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float2 dx = sub2(X, S.yx[j]);
            const float2 dy = sub2(Y, S.yy[j]);
            const float2 dz = sub2(Zc, S.yz[j]);
            const float2 r2d = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));  // (kR)^2
            float2 rinv;
            rinv.x = rsqrtf(r2d.x);
            rinv.y = rsqrtf(r2d.y);
            const float2 kR = mul2(r2d, rinv);
            float2 sn, cs;
            __sincosf(kR.x, &sn.x, &cs.x);
            __sincosf(kR.y, &sn.y, &cs.y);
            const float2 g = mul2(S.yw[j], rinv);
            const float2 gr = mul2(g, cs), gs = mul2(g, sn);  // G = gr - j gs
            s0r = add2(s0r, gr);
            s0s = add2(s0s, gs);
            sxr = fma2(gr, S.yx[j], sxr);
            sxs = fma2(gs, S.yx[j], sxs);
            syr = fma2(gr, S.yy[j], syr);
            sys = fma2(gs, S.yy[j], sys);
            szr = fma2(gr, S.yz[j], szr);
            szs = fma2(gs, S.yz[j], szs);
        }
        float a0r = s0r.x + s0r.y, a0s = s0s.x + s0s.y;
        float a1r[3] = {sxr.x + sxr.y, syr.x + syr.y, szr.x + szr.y};
        float a1s[3] = {sxs.x + sxs.y, sys.x + sys.y, szs.x + szs.y};
        {
            // the seventh source point, scalar
            const float dx = k * x.x - S.tx, dy = k * x.y - S.ty, dz = k * x.z - S.tz;
            const float r2d = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const float rinv = rsqrtf(r2d);
            const float kR = r2d * rinv;
            float sn, cs;
            __sincosf(kR, &sn, &cs);
            const float g = S.tw * rinv;
            const float gr = g * cs, gs = g * sn;
            a0r += gr;
            a0s += gs;
            a1r[0] = fmaf(gr, S.tx, a1r[0]);
            a1s[0] = fmaf(gs, S.tx, a1s[0]);
            a1r[1] = fmaf(gr, S.ty, a1r[1]);
            a1s[1] = fmaf(gs, S.ty, a1s[1]);
            a1r[2] = fmaf(gr, S.tz, a1r[2]);
            a1s[2] = fmaf(gs, S.tz, a1s[2]);
        }
        // Im G = -gs: the imaginary sums enter with a minus sign
        t0r = fmaf(wi, a0r, t0r);
        t0i = fmaf(-wi, a0s, t0i);
        const float xs[3] = {x.x, x.y, x.z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            txr[a] = fmaf(wi * xs[a], a0r, txr[a]);
            txi[a] = fmaf(-wi * xs[a], a0s, txi[a]);
            tyr[a] = fmaf(wi, a1r[a], tyr[a]);
            tyi[a] = fmaf(-wi, a1s[a], tyi[a]);
        }
        txyr = fmaf(wi, xs[0] * a1r[0] + xs[1] * a1r[1] + xs[2] * a1r[2], txyr);
        txyi = fmaf(-wi, xs[0] * a1s[0] + xs[1] * a1s[1] + xs[2] * a1s[2], txyi);
    }
    const float ik = 1.f / k;
    const V3<float> Txr = v3<float>(txr[0], txr[1], txr[2]), Txi = v3<float>(txi[0], txi[1], txi[2]);
    const V3<float> Tyr = v3<float>(tyr[0] * ik, tyr[1] * ik, tyr[2] * ik);
    const V3<float> Tyi = v3<float>(tyi[0] * ik, tyi[1] * ik, tyi[2] * ik);
    txyr *= ik;
    txyi *= ik;
    const float inv_k4 = 4.f / k;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const float amr = dot(A[m], Tyr), ami = dot(A[m], Tyi);
        const int64_t row = rows[m];
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const float ab = dot(A[m], S.B[n]);
            const float fr = txyr - dot(S.B[n], Txr) - amr + ab * t0r;  // int int (x-A_m).(y-B_n) G
            const float fi = txyi - dot(S.B[n], Txi) - ami + ab * t0i;
            const float cc = cm[m] * S.cn[n];
            const float re = cc * (-k * fi + inv_k4 * t0i);
            const float im = cc * (k * fr - inv_k4 * t0r);
            add_c<float>(z + 2 * (row * n_edges + S.col[n]), re, im);
        }
    }
}

template <>
__device__ __forceinline__ void sym_regular_pair<float>(const float* __restrict__ verts,
                                                        const int32_t* __restrict__ faces,
                                                        const int32_t* __restrict__ fei, int64_t n_edges, float k,
                                                        int64_t p, int64_t q, const float (*s_b)[4],
                                                        float* __restrict__ z) {
    if (shared_vertices(faces, p, q) != 0) return;  // done by the FP64 near-pair kernel
    SymSource S;
    sym_source(verts, faces, fei, k, q, s_b, S);
    V3<float> A[3];
    int32_t rows[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        A[v] = load3(verts, __ldg(faces + 3 * p + v)) - S.o;
        rows[v] = __ldg(fei + 3 * p + v);
    }
    float cm[3], ap;
    rwg_consts<float>(faces, p, A, cm, &ap);
    sym_pair_eval(S, A, cm, ap, rows, k, n_edges, s_b, z);
}

// Single-mesh float separated pairs: a block owns kSymRows test faces (their vertices, RWG
// constants and edge ids staged in shared memory) and 128 source faces; each thread sets up
// its source face once and evaluates it against every test face of the block.
constexpr int kSymRows = 32;
__global__ void __launch_bounds__(128) mom_sym_regular_rows_kernel(const float* __restrict__ verts,
                                                                   const int32_t* __restrict__ faces,
                                                                   const int32_t* __restrict__ fei,
                                                                   int64_t n_edges, float k, int64_t nf,
                                                                   int64_t p_begin, int64_t p_end,
                                                                   float* __restrict__ z) {
    __shared__ float s_b[7][4];
    __shared__ float s_A[kSymRows][9], s_cm[kSymRows][3], s_ap[kSymRows];
    __shared__ int32_t s_v[kSymRows][3], s_row[kSymRows][3];
    if (threadIdx.x < 28) s_b[threadIdx.x / 4][threadIdx.x % 4] = (float)c_d7[threadIdx.x / 4][threadIdx.x % 4];
    const int64_t p0 = p_begin + (int64_t)blockIdx.y * kSymRows;
    if (threadIdx.x < kSymRows && p0 + threadIdx.x < p_end) {
        const int64_t p = p0 + threadIdx.x;
        V3<float> A[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) {
            s_v[threadIdx.x][v] = __ldg(faces + 3 * p + v);
            s_row[threadIdx.x][v] = __ldg(fei + 3 * p + v);
            A[v] = load3(verts, s_v[threadIdx.x][v]);
            s_A[threadIdx.x][3 * v] = A[v].x;
            s_A[threadIdx.x][3 * v + 1] = A[v].y;
            s_A[threadIdx.x][3 * v + 2] = A[v].z;
        }
        float cm[3], ap;
        rwg_consts<float>(faces, p, A, cm, &ap);
        s_cm[threadIdx.x][0] = cm[0];
        s_cm[threadIdx.x][1] = cm[1];
        s_cm[threadIdx.x][2] = cm[2];
        s_ap[threadIdx.x] = ap;
    }
    __syncthreads();
    const int64_t q = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (q >= nf) return;
    SymSource S;
    sym_source(verts, faces, fei, k, q, s_b, S);
    const int nr = (int)min((int64_t)kSymRows, p_end - p0);
#pragma unroll 1
    for (int r = 0; r < nr; ++r) {
        int shared = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) shared += s_v[r][a] == S.v[b];
        if (shared) continue;  // done by the FP64 near-pair kernel
        V3<float> A[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) A[v] = v3<float>(s_A[r][3 * v], s_A[r][3 * v + 1], s_A[r][3 * v + 2]) - S.o;
        const float cm[3] = {s_cm[r][0], s_cm[r][1], s_cm[r][2]};
        const int32_t rows[3] = {s_row[r][0], s_row[r][1], s_row[r][2]};
        sym_pair_eval(S, A, cm, s_ap[r], rows, k, n_edges, s_b, z);
    }
}

template <typename T>
__global__ void __launch_bounds__(128) mom_sym_regular_kernel(const T* __restrict__ verts,
                                                              const int32_t* __restrict__ faces,
                                                              const int32_t* __restrict__ fei, int64_t n_edges,
                                                              T k, int64_t nf, int64_t p_begin, int64_t q_blocks,
                                                              T* __restrict__ z) {
    __shared__ T s_b[7][4];
    if (threadIdx.x < 28) s_b[threadIdx.x / 4][threadIdx.x % 4] = (T)c_d7[threadIdx.x / 4][threadIdx.x % 4];
    __syncthreads();
    const int64_t p = p_begin + (int64_t)blockIdx.x / q_blocks;
    const int64_t q = ((int64_t)blockIdx.x % q_blocks) * 128 + threadIdx.x;
    if (q >= nf) return;
    sym_regular_pair<T>(verts, faces, fei, n_edges, k, p, q, s_b, z);
}

// ---------------------------------------------------------------------------------------
// pairs sharing a vertex: FP64 with the singular part in closed form; one thread per pair
// ---------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void sym_near_pair(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                              const int32_t* __restrict__ fei, int64_t n_edges, double k, int64_t p,
                                              int64_t q, T* __restrict__ z) {
    V3<double> A[3], B[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const int64_t ia = faces[3 * p + v], ib = faces[3 * q + v];
        A[v] = v3<double>(verts[3 * ia], verts[3 * ia + 1], verts[3 * ia + 2]);
        B[v] = v3<double>(verts[3 * ib], verts[3 * ib + 1], verts[3 * ib + 2]);
    }
    double cm[3], cn[3], ap, aq;
    rwg_consts<double>(faces, p, A, cm, &ap);
    rwg_consts<double>(faces, q, B, cn, &aq);
    const double inv4pi = kInv4Pi;
    // moments over the test points (FP64): t0 = sum_i w_i g0_i, tx = sum_i w_i x_i g0_i,
    // ty = sum_i w_i gy_i, txy = sum_i w_i x_i . gy_i, with g0 = int G, gy = int G y over q
    double t0r = 0, t0i = 0, txyr = 0, txyi = 0;
    V3<double> txr = v3<double>(0, 0, 0), txi = v3<double>(0, 0, 0), tyr = v3<double>(0, 0, 0),
               tyi = v3<double>(0, 0, 0);
    for (int i = 0; i < 7; ++i) {
        const V3<double> x = c_d7[i][0] * A[0] + c_d7[i][1] * A[1] + c_d7[i][2] * A[2];
        double g0r = 0, g0i = 0;
        V3<double> gyr = v3<double>(0, 0, 0), gyi = v3<double>(0, 0, 0);
        if constexpr (sizeof(T) == 4) {
            // complex64 output: the smooth part (e^{-jkR} - 1) / (4 pi R) in FP32 (point
            // differences taken in FP64, moments relative to B0), the singular 1/R part below
            // in FP64 and closed form
            const float kf = (float)k;
            float s0r = 0.f, s0i = 0.f, syr[3] = {0.f, 0.f, 0.f}, syi[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int j = 0; j < 7; ++j) {
                const V3<double> y = c_d7[j][0] * B[0] + c_d7[j][1] * B[1] + c_d7[j][2] * B[2];
                const V3<double> dd = x - y;
                const float dx = (float)dd.x, dy = (float)dd.y, dz = (float)dd.z;
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                const float wj = (float)(c_d7[j][3] * aq * inv4pi);
                float gr, gi;
                if (r2 <= 0.f) {  // coincident points of the self pair: limit of the smooth part
                    gr = 0.f;
                    gi = -kf * wj;
                } else {
                    const float rinv = rsqrtf(r2);
                    const float kR = kf * (r2 * rinv);
                    float sn, cs, sh, ch;
                    __sincosf(kR, &sn, &cs);
                    __sincosf(0.5f * kR, &sh, &ch);
                    gr = -2.f * sh * sh * rinv * wj;  // (cos kR - 1) / R without cancellation
                    gi = -sn * rinv * wj;
                }
                const float yl[3] = {(float)(y.x - B[0].x), (float)(y.y - B[0].y), (float)(y.z - B[0].z)};
                s0r += gr;
                s0i += gi;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    syr[a] = fmaf(gr, yl[a], syr[a]);
                    syi[a] = fmaf(gi, yl[a], syi[a]);
                }
            }
            g0r = s0r;
            g0i = s0i;
            gyr = v3<double>(syr[0], syr[1], syr[2]) + g0r * B[0];
            gyi = v3<double>(syi[0], syi[1], syi[2]) + g0i * B[0];
        } else {
            for (int j = 0; j < 7; ++j) {
                const V3<double> y = c_d7[j][0] * B[0] + c_d7[j][1] * B[1] + c_d7[j][2] * B[2];
                const V3<double> dd = x - y;
                const double R = sqrt(dot(dd, dd));
                double gr, gi;
                if (R < 1e-300) {  // coincident points of the self pair: limit of the smooth part
                    gr = 0.0;
                    gi = -k * inv4pi;
                } else {
                    double sn, cs;
                    sincos(k * R, &sn, &cs);
                    const double sh = sin(0.5 * k * R);
                    gr = -2.0 * sh * sh / R * inv4pi;  // (cos kR - 1) / (4 pi R)
                    gi = -sn / R * inv4pi;
                }
                const double wj = c_d7[j][3] * aq;
                g0r += wj * gr;
                g0i += wj * gi;
                gyr = gyr + (wj * gr) * y;
                gyi = gyi + (wj * gi) * y;
            }
        }
        double I1;
        V3<double> Iv;
        potential_integrals(x, B, &I1, &Iv);
        g0r += inv4pi * I1;
        gyr = gyr + inv4pi * (Iv + I1 * x);
        const double wi = c_d7[i][3] * ap;
        t0r += wi * g0r;
        t0i += wi * g0i;
        txr = txr + (wi * g0r) * x;
        txi = txi + (wi * g0i) * x;
        tyr = tyr + wi * gyr;
        tyi = tyi + wi * gyi;
        txyr += wi * dot(x, gyr);
        txyi += wi * dot(x, gyi);
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const int64_t row = fei[3 * p + m];
        const double amr = dot(A[m], tyr), ami = dot(A[m], tyi);
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const double ab = dot(A[m], B[n]);
            const double fr = txyr - dot(B[n], txr) - amr + ab * t0r;  // sum_i w_i (x - A_m).(gy - g0 B_n)
            const double fi = txyi - dot(B[n], txi) - ami + ab * t0i;
            const double cc = cm[m] * cn[n];
            add_c<T>(z + 2 * (row * n_edges + fei[3 * q + n]), (T)(cc * (-k * fi + 4.0 / k * t0i)),
                     (T)(cc * (k * fr - 4.0 / k * t0r)));
        }
    }
}

template <typename T>
__global__ void mom_sym_near_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                    const int32_t* __restrict__ fei, int64_t n_edges,
                                    const int32_t* __restrict__ pairs, int64_t n_pairs, double k,
                                    T* __restrict__ z) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_pairs) return;
    sym_near_pair<T>(verts, faces, fei, n_edges, k, pairs[2 * t], pairs[2 * t + 1], z);
}

// ---------------------------------------------------------------------------------------
// EFIE excitation with the same rule: rhs[fei, r] += int f_m . E0 e^{-j k khat.x}
// waves: [n_rhs, 9] float64 (k khat, E0, H0); one thread per (face, wave)
// ---------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void sym_rhs_face(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                             const int32_t* __restrict__ fei, const double* __restrict__ w,
                                             int64_t p, int64_t ld, int64_t col, T* __restrict__ rhs) {
    V3<T> A[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) A[v] = load3(verts, faces[3 * p + v]);
    T c[3], area;
    rwg_consts<T>(faces, p, A, c, &area);
    const V3<T> kv = v3<T>((T)w[0], (T)w[1], (T)w[2]), E0 = v3<T>((T)w[3], (T)w[4], (T)w[5]);
    T sr[3] = {0, 0, 0}, si[3] = {0, 0, 0};
    for (int i = 0; i < 7; ++i) {
        const V3<T> x = (T)c_d7[i][0] * A[0] + (T)c_d7[i][1] * A[1] + (T)c_d7[i][2] * A[2];
        T sn, cs;
        sincos_turns(dot(kv, x) * T(kInv2Pi), &sn, &cs);
        const T wi = (T)c_d7[i][3] * area;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const T proj = wi * c[m] * dot(x - A[m], E0);
            sr[m] += proj * cs;
            si[m] -= proj * sn;
        }
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) add_c<T>(rhs + 2 * ((int64_t)fei[3 * p + m] * ld + col), sr[m], si[m]);
}

template <typename T>
__global__ void mom_sym_rhs_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                   const int32_t* __restrict__ fei, const double* __restrict__ waves, int nrhs,
                                   int64_t nf, T* __restrict__ rhs) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nf * nrhs) return;
    const int r = (int)(t / nf);
    sym_rhs_face<T>(verts, faces, fei, waves + 9 * r, t % nf, nrhs, r, rhs);
}

// ---------------------------------------------------------------------------------------
// many meshes in one launch each.  The meshes are packed into one vertex / face array
// (vertex ids global, edge ids local to each mesh); desc[i] = (face offset, faces, edges,
// offset of the mesh's Z in the flat block-diagonal array (complex entries), first block of
// the mesh in the regular launch, first right-hand-side column); ks[i] its wavenumber.
// ---------------------------------------------------------------------------------------
constexpr int kDesc = 6;

__device__ __forceinline__ int mesh_of(const int64_t* __restrict__ desc, int n_mesh, int field, int64_t v) {
    int lo = 0, hi = n_mesh - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(desc + kDesc * mid + field) <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <typename T>
__global__ void __launch_bounds__(128) mom_sym_regular_batched_kernel(
    const T* __restrict__ verts, const int32_t* __restrict__ faces, const int32_t* __restrict__ fei,
    const int64_t* __restrict__ desc, const double* __restrict__ ks, int n_mesh, T* __restrict__ z) {
    __shared__ T s_b[7][4];
    if (threadIdx.x < 28) s_b[threadIdx.x / 4][threadIdx.x % 4] = (T)c_d7[threadIdx.x / 4][threadIdx.x % 4];
    __syncthreads();
    const int64_t b = blockIdx.x;
    const int i = mesh_of(desc, n_mesh, 4, b);
    const int64_t fo = __ldg(desc + kDesc * i), nf = __ldg(desc + kDesc * i + 1);
    const int64_t qb = (nf + 127) / 128, local = b - __ldg(desc + kDesc * i + 4);
    const int64_t p = fo + local / qb, q = fo + (local % qb) * 128 + threadIdx.x;
    if (q >= fo + nf) return;
    const int64_t ne = __ldg(desc + kDesc * i + 2);
    sym_regular_pair<T>(verts, faces, fei, ne + (ne & 1), (T)__ldg(ks + i), p, q, s_b,
                        z + 2 * __ldg(desc + kDesc * i + 3));
}

template <typename T>
__global__ void mom_sym_near_batched_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                            const int32_t* __restrict__ fei, const int64_t* __restrict__ desc,
                                            const double* __restrict__ ks, int n_mesh,
                                            const int32_t* __restrict__ pairs, int64_t n_pairs,
                                            T* __restrict__ z) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_pairs) return;
    const int64_t p = pairs[2 * t];
    const int i = mesh_of(desc, n_mesh, 0, p);
    const int64_t ne = desc[kDesc * i + 2];
    sym_near_pair<T>(verts, faces, fei, ne + (ne & 1), ks[i], p, pairs[2 * t + 1], z + 2 * desc[kDesc * i + 3]);
}

// waves: [n_mesh * nrhs, 9]; rhs: [rows, ld] interleaved complex, column desc[i][5] + r.
template <typename T>
__global__ void mom_sym_rhs_batched_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                           const int32_t* __restrict__ fei, const int64_t* __restrict__ desc,
                                           int n_mesh, int64_t total_faces, const double* __restrict__ waves,
                                           int nrhs, int64_t ld, T* __restrict__ rhs) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total_faces * nrhs) return;
    const int r = (int)(t / total_faces);
    const int64_t p = t % total_faces;
    const int i = mesh_of(desc, n_mesh, 0, p);
    sym_rhs_face<T>(verts, faces, fei, waves + 9 * ((int64_t)i * nrhs + r), p, ld, desc[kDesc * i + 5] + r, rhs);
}

// Batched float separated pairs in the rows layout of mom_sym_regular_rows_kernel: a block
// owns R test faces of one mesh (staged in shared memory) and 128 of its source faces.  The
// blocks of the meshes are laid out in a schedule: sched[j] is the j-th mesh of the launch and
// boff[j] its first block (boff[n_mesh] = the launch size), so the autotuner can put the
// largest meshes first or keep the packing order, and pick R.
template <int R>
__global__ void __launch_bounds__(128) mom_sym_rows_batched_kernel(
    const float* __restrict__ verts, const int32_t* __restrict__ faces, const int32_t* __restrict__ fei,
    const int64_t* __restrict__ desc, const double* __restrict__ ks, const int32_t* __restrict__ sched,
    const int64_t* __restrict__ boff, int n_mesh, float* __restrict__ z) {
    __shared__ float s_b[7][4];
    __shared__ float s_A[R][9], s_cm[R][3], s_ap[R];
    __shared__ int32_t s_v[R][3], s_row[R][3];
    if (threadIdx.x < 28) s_b[threadIdx.x / 4][threadIdx.x % 4] = (float)c_d7[threadIdx.x / 4][threadIdx.x % 4];
    const int64_t b = blockIdx.x;
    int lo = 0, hi = n_mesh - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(boff + mid) <= b) lo = mid; else hi = mid - 1;
    }
    const int i = __ldg(sched + lo);
    const int64_t fo = __ldg(desc + kDesc * i), nf = __ldg(desc + kDesc * i + 1), ne = __ldg(desc + kDesc * i + 2);
    const int64_t qb = (nf + 127) / 128, local = b - __ldg(boff + lo);
    const int64_t p0 = fo + (local / qb) * R, p_end = fo + nf;
    if (threadIdx.x < R && p0 + threadIdx.x < p_end) {
        const int64_t p = p0 + threadIdx.x;
        V3<float> A[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) {
            s_v[threadIdx.x][v] = __ldg(faces + 3 * p + v);
            s_row[threadIdx.x][v] = __ldg(fei + 3 * p + v);
            A[v] = load3(verts, s_v[threadIdx.x][v]);
            s_A[threadIdx.x][3 * v] = A[v].x;
            s_A[threadIdx.x][3 * v + 1] = A[v].y;
            s_A[threadIdx.x][3 * v + 2] = A[v].z;
        }
        float cm[3], ap;
        rwg_consts<float>(faces, p, A, cm, &ap);
        s_cm[threadIdx.x][0] = cm[0];
        s_cm[threadIdx.x][1] = cm[1];
        s_cm[threadIdx.x][2] = cm[2];
        s_ap[threadIdx.x] = ap;
    }
    __syncthreads();
    const int64_t q = fo + (local % qb) * 128 + threadIdx.x;
    if (q >= p_end) return;
    const float k = (float)__ldg(ks + i);
    SymSource S;
    sym_source(verts, faces, fei, k, q, s_b, S);
    const int nr = (int)min((int64_t)R, p_end - p0);
    float* zi = z + 2 * __ldg(desc + kDesc * i + 3);
    const int64_t pitch = ne + (ne & 1);
#pragma unroll 1
    for (int r = 0; r < nr; ++r) {
        int shared = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) shared += s_v[r][a] == S.v[c];
        if (shared) continue;  // done by the FP64 near-pair kernel
        V3<float> A[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) A[v] = v3<float>(s_A[r][3 * v], s_A[r][3 * v + 1], s_A[r][3 * v + 2]) - S.o;
        const float cm[3] = {s_cm[r][0], s_cm[r][1], s_cm[r][2]};
        const int32_t rows[3] = {s_row[r][0], s_row[r][1], s_row[r][2]};
        sym_pair_eval(S, A, cm, s_ap[r], rows, k, pitch, s_b, zi);
    }
}

int launch_mom_sym_rows_batched(const float* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc,
                                const double* ks, int n_mesh, const int32_t* sched, const int64_t* boff,
                                int64_t total_blocks, int rows_per_block, const int32_t* pairs, int64_t n_pairs,
                                float* z, cudaStream_t s) {
    if (n_mesh <= 0) return MB_OK;
    if (total_blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "batch too large for one launch");
    if (total_blocks > 0) {
        const unsigned nb = (unsigned)total_blocks;
        if (rows_per_block == 8)
            mom_sym_rows_batched_kernel<8><<<nb, 128, 0, s>>>(verts, faces, fei, desc, ks, sched, boff, n_mesh, z);
        else if (rows_per_block == 16)
            mom_sym_rows_batched_kernel<16><<<nb, 128, 0, s>>>(verts, faces, fei, desc, ks, sched, boff, n_mesh, z);
        else if (rows_per_block == 32)
            mom_sym_rows_batched_kernel<32><<<nb, 128, 0, s>>>(verts, faces, fei, desc, ks, sched, boff, n_mesh, z);
        else
            return set_error(MB_ERR_UNSUPPORTED, "rows per block must be 8, 16 or 32");
    }
    if (n_pairs > 0)
        mom_sym_near_batched_kernel<float><<<(unsigned)((n_pairs + 127) / 128), 128, 0, s>>>(
            verts, faces, fei, desc, ks, n_mesh, pairs, n_pairs, z);
    return check_launch("mom_sym_rows_batched");
}

template <typename T>
int launch_mom_sym_batched(const T* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc,
                           const double* ks, int n_mesh, int64_t total_blocks, const int32_t* pairs,
                           int64_t n_pairs, T* z, cudaStream_t s) {
    if (n_mesh <= 0) return MB_OK;
    if (total_blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "batch too large for one launch");
    if (total_blocks > 0)
        mom_sym_regular_batched_kernel<T><<<(unsigned)total_blocks, 128, 0, s>>>(verts, faces, fei, desc, ks, n_mesh,
                                                                                  z);
    if (n_pairs > 0)
        mom_sym_near_batched_kernel<T><<<(unsigned)((n_pairs + 127) / 128), 128, 0, s>>>(verts, faces, fei, desc, ks,
                                                                                         n_mesh, pairs, n_pairs, z);
    return check_launch("mom_sym_batched");
}

template <typename T>
int launch_mom_sym_rhs_batched(const T* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc,
                               int n_mesh, int64_t total_faces, const double* waves, int nrhs, int64_t ld, T* rhs,
                               cudaStream_t s) {
    if (n_mesh <= 0 || total_faces <= 0 || nrhs <= 0) return MB_OK;
    const int64_t total = total_faces * nrhs;
    mom_sym_rhs_batched_kernel<T><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(verts, faces, fei, desc, n_mesh,
                                                                                   total_faces, waves, nrhs, ld, rhs);
    return check_launch("mom_sym_rhs_batched");
}

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------
// Z rows -> host memory: rows[] of src copied to the same rows of dst (device-accessible host
// memory); a few blocks loop over the rows so the copy leaves the SMs to the assembly.
__global__ void drain_rows_kernel(const float2* __restrict__ src, float2* dst, const int32_t* __restrict__ rows,
                                  int64_t n_rows, int64_t n_edges) {
    for (int64_t r = blockIdx.x; r < n_rows; r += gridDim.x) {
        const int64_t m = rows[r];
        const float2* sp = src + m * n_edges;
        float2* dp = dst + m * n_edges;
        for (int64_t j = threadIdx.x; j < n_edges; j += blockDim.x) dp[j] = sp[j];
    }
}

template <typename T>
int launch_mom_sym_regular(const T* verts, const int32_t* faces, const int32_t* fei, int64_t n_edges, double k,
                           int64_t nf, int64_t p_begin, int64_t p_end, T* z, cudaStream_t s);
template <typename T>
int launch_mom_sym_near(const T* verts, const int32_t* faces, const int32_t* fei, int64_t n_edges,
                        const int32_t* pairs, int64_t n_pairs, double k, T* z, cudaStream_t s);

// The symmetric-rule Z (separated pairs + near pairs, complex64) into pinned host memory with
// the copy overlapped: test faces in `chunks` ranges; after each range the Z rows whose faces
// have all been processed are written to z_host by a small drain kernel on a second stream
// while the next range is assembled.  pairs must be sorted by test face (near_pairs order).
int sym_zmat_to_host(const float* verts, const int32_t* faces, const int32_t* fei, int64_t nf, int64_t n_edges,
                     double k, const int32_t* pairs, int64_t n_pairs, float* z_dev, float* z_host, int chunks,
                     cudaStream_t s) {
    chunks = std::max(1, std::min<int>(chunks, (int)std::max<int64_t>(1, nf)));
    float2* hdst = nullptr;
    if (cudaHostGetDevicePointer(reinterpret_cast<void**>(&hdst), z_host, 0) != cudaSuccess || !hdst) {
        cudaGetLastError();
        return set_error(MB_ERR_ARG, "z_host must be page-locked host memory (pinned)");
    }
    // host copies of the face-edge map and the near-pair list
    std::vector<int32_t> hfei((size_t)3 * nf), hp((size_t)2 * n_pairs);
    cudaMemcpyAsync(hfei.data(), fei, 12 * (size_t)nf, cudaMemcpyDeviceToHost, s);
    if (n_pairs) cudaMemcpyAsync(hp.data(), pairs, 8 * (size_t)n_pairs, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return check_launch("sym zmat to host: maps");
    for (int64_t t = 1; t < n_pairs; ++t)
        if (hp[2 * t] < hp[2 * (t - 1)]) return set_error(MB_ERR_ARG, "near pairs must be sorted by test face");
    std::vector<int64_t> fb((size_t)chunks + 1);
    for (int c = 0; c <= chunks; ++c) fb[c] = nf * c / chunks;
    // chunk after which each Z row is complete: the range of its last face
    std::vector<int32_t> last((size_t)n_edges, -1);
    for (int64_t r = 0; r < 3 * nf; ++r) {
        const int32_t m = hfei[r];
        if (m < 0 || m >= n_edges) return set_error(MB_ERR_ARG, "face_edge_indices out of range");
        last[m] = std::max<int32_t>(last[m], (int32_t)(r / 3));
    }
    std::vector<int64_t> off((size_t)chunks + 1, 0);
    std::vector<int32_t> chunk_of((size_t)n_edges);
    for (int64_t m = 0; m < n_edges; ++m) {
        const int64_t f = std::max<int32_t>(last[m], 0);
        int c = (int)std::min<int64_t>(chunks - 1, f * chunks / std::max<int64_t>(nf, 1));
        while (c > 0 && fb[c] > f) --c;
        while (c + 1 < chunks && fb[c + 1] <= f) ++c;
        chunk_of[m] = c;
        ++off[c + 1];
    }
    for (int c = 0; c < chunks; ++c) off[c + 1] += off[c];
    std::vector<int32_t> rows((size_t)n_edges);
    {
        std::vector<int64_t> pos(off.begin(), off.end() - 1);
        for (int64_t m = 0; m < n_edges; ++m) rows[pos[chunk_of[m]]++] = (int32_t)m;
    }
    std::vector<int64_t> pb((size_t)chunks + 1);
    for (int c = 0; c <= chunks; ++c) {
        int64_t lo = 0, hi = n_pairs;  // first pair with test face >= fb[c]
        while (lo < hi) {
            const int64_t mid = (lo + hi) / 2;
            if (hp[2 * mid] < fb[c]) lo = mid + 1;
            else hi = mid;
        }
        pb[c] = lo;
    }
    int32_t* drows = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void**>(&drows), 4 * (size_t)n_edges, s) != cudaSuccess)
        return set_error(MB_ERR_CUDA, "sym zmat to host: row list");
    cudaMemcpyAsync(drows, rows.data(), 4 * (size_t)n_edges, cudaMemcpyHostToDevice, s);
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
        cudaFreeAsync(drows, s);
        return set_error(MB_ERR_CUDA, "sym zmat to host: copy stream");
    }
    std::vector<cudaEvent_t> ev((size_t)chunks + 1, nullptr);
    int rc = MB_OK;
    for (auto& e : ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = MB_ERR_CUDA;
    if (rc) rc = set_error(MB_ERR_CUDA, "sym zmat to host: events");
    cudaMemsetAsync(z_dev, 0, (size_t)n_edges * n_edges * 8, s);
    for (int c = 0; c < chunks && rc == MB_OK; ++c) {
        if ((rc = launch_mom_sym_regular<float>(verts, faces, fei, n_edges, k, nf, fb[c], fb[c + 1], z_dev, s)))
            break;
        if (pb[c + 1] > pb[c] &&
            (rc = launch_mom_sym_near<float>(verts, faces, fei, n_edges, pairs + 2 * pb[c], pb[c + 1] - pb[c], k,
                                             z_dev, s)))
            break;
        cudaEventRecord(ev[c], s);
        cudaStreamWaitEvent(cs, ev[c], 0);
        if (off[c + 1] > off[c])
            drain_rows_kernel<<<32, 512, 0, cs>>>(reinterpret_cast<const float2*>(z_dev), hdst, drows + off[c],
                                                   off[c + 1] - off[c], n_edges);
    }
    cudaEventRecord(ev[chunks], cs);
    cudaStreamWaitEvent(s, ev[chunks], 0);
    cudaFreeAsync(drows, s);
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    cudaStreamDestroy(cs);
    if (rc) return rc;
    return check_launch("sym zmat to host");
}

template <typename T>
int launch_mom_sym_regular(const T* verts, const int32_t* faces, const int32_t* fei, int64_t n_edges, double k,
                           int64_t nf, int64_t p_begin, int64_t p_end, T* z, cudaStream_t s) {
    if (nf <= 0 || p_end <= p_begin) return MB_OK;
    if (!(k > 0)) return set_error(MB_ERR_ARG, "wavenumber must be > 0");
    const int64_t q_blocks = (nf + 127) / 128;
    if constexpr (sizeof(T) == 4) {
        const int64_t py = (p_end - p_begin + kSymRows - 1) / kSymRows;
        if (q_blocks > 0x7fffffffLL || py > 65535) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
        mom_sym_regular_rows_kernel<<<dim3((unsigned)q_blocks, (unsigned)py), 128, 0, s>>>(
            verts, faces, fei, n_edges, (float)k, nf, p_begin, p_end, z);
        return check_launch("mom_sym_regular");
    }
    const int64_t blocks = (p_end - p_begin) * q_blocks;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
    mom_sym_regular_kernel<T><<<(unsigned)blocks, 128, 0, s>>>(verts, faces, fei, n_edges, (T)k, nf, p_begin,
                                                                q_blocks, z);
    return check_launch("mom_sym_regular");
}

template <typename T>
int launch_mom_sym_near(const T* verts, const int32_t* faces, const int32_t* fei, int64_t n_edges,
                        const int32_t* pairs, int64_t n_pairs, double k, T* z, cudaStream_t s) {
    if (n_pairs <= 0) return MB_OK;
    if (!(k > 0)) return set_error(MB_ERR_ARG, "wavenumber must be > 0");
    const int64_t blocks = (n_pairs + 127) / 128;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "too many near pairs for one launch");
    mom_sym_near_kernel<T><<<(unsigned)blocks, 128, 0, s>>>(verts, faces, fei, n_edges, pairs, n_pairs, k, z);
    return check_launch("mom_sym_near");
}

template <typename T>
int launch_mom_sym_rhs(const T* verts, const int32_t* faces, const int32_t* fei, const double* waves, int nrhs,
                       int64_t nf, T* rhs, cudaStream_t s) {
    if (nf <= 0 || nrhs <= 0) return MB_OK;
    const int64_t total = nf * nrhs;
    mom_sym_rhs_kernel<T><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(verts, faces, fei, waves, nrhs, nf, rhs);
    return check_launch("mom_sym_rhs");
}

#define MB_INST(T)                                                                                       \
    template int launch_mom_sym_batched<T>(const T*, const int32_t*, const int32_t*, const int64_t*, const double*, \
                                           int, int64_t, const int32_t*, int64_t, T*, cudaStream_t);     \
    template int launch_mom_sym_rhs_batched<T>(const T*, const int32_t*, const int32_t*, const int64_t*, int,   \
                                               int64_t, const double*, int, int64_t, T*, cudaStream_t);   \
    template int launch_mom_sym_regular<T>(const T*, const int32_t*, const int32_t*, int64_t, double, int64_t, \
                                           int64_t, int64_t, T*, cudaStream_t);                         \
    template int launch_mom_sym_near<T>(const T*, const int32_t*, const int32_t*, int64_t, const int32_t*,   \
                                        int64_t, double, T*, cudaStream_t);                             \
    template int launch_mom_sym_rhs<T>(const T*, const int32_t*, const int32_t*, const double*, int, int64_t, \
                                       T*, cudaStream_t);
MB_INST(float)
MB_INST(double)
#undef MB_INST

}  // namespace mb
