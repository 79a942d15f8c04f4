// mom_ref.cu -- RWG MoM kernels with the reference's quadrature rule.
//
// The reference (GeCao/Mesh-Ferrofluid, src/mesh_BEM/cuda/mesh_MOM_3d.cu) integrates each
// face-edge pair (test face f1 / local edge e1, source face f2 / local edge e2) with a
// collapsed Gauss-Legendre rule whose points are laid out from the vertex opposite the
// local edge (x = (1-r1) v_e + (r1-r2) v_{e+1} + r2 v_{e+2}, r2 = p_j r1, weight w_i w_j 2A,
// Jacobian r1; :410-421).  The rule is not invariant under vertex rotation, so the nine
// entries of a triangle pair use nine different point sets: the work per entry is
// irreducible at Nt x Ns kernel evaluations, exactly as in the reference.  What this file
// removes is everything around it:
//   * one sincos per point pair shared by G and grad G (the reference evaluates both
//     separately, :461-465), a MUFU rsqrt instead of sqrt + divide;
//   * the per-test-point moment form: with the origin moved to the source vertex B0,
//       L1 = jk c2 S1,   L2 = -(j/k) div2 S0,   K = -c2 (H1 x x)
//     where S0 = sum w G, S1 = sum w G y, H1 = sum w h y and grad_x G = -h (x - y), so the
//     inner loop only accumulates four complex moments (see `mom_entry`);
//   * RWG constants computed once per thread instead of per point (:167-242);
//   * float arithmetic stays float (the reference's M_PI / 0.5 / 1.0 literals promote the
//     float build to FP64, :93-94, :123-124, :434, :479-480);
//   * 64-bit indexing (the reference's `int idx` overflows at F > 15447, :364-374);
//   * coordinates are shifted to a per-pair origin so FP32 keeps the precision of the
//     short near-field distances.
// Entry algebra: with c = s l/(2A) (RWG scale) and div = 2c, every term of the entry is
// proportional to c1 c2, so the entry is
//   c1 c2 sum_i w_i [ -H1_i . (x_i x ((x_i - A0) x n1)) + jk (x_i - A0) . S1_i - (4j/k) S0_i ]
//   + (same face only) c1 c2 sum_i w_i 0.5 (x_i - A0) . (x_i - B0)
// which reproduces :408-493 term by term.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "packed.cuh"

namespace mb {

// Rule tables are passed per launch as device pointers (at most 16 nodes per direction);
// each block copies them to shared memory.

// ---------------------------------------------------------------------------------------
// One face-edge entry (row = f1*3+e1, col = f2*3+e2), reference rule.
// NS > 0: source points held in registers (NS = ny*ny); NS == 0: recomputed per use.
// ---------------------------------------------------------------------------------------
template <typename T, int NS>
__device__ __forceinline__ void mom_entry(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                          const T* __restrict__ areas, const T* __restrict__ normals,
                                          const T* s_px, const T* s_wx, int nx, const T* s_py,
                                          const T* s_wy, int ny, T k, int64_t f1, int e1, int64_t f2,
                                          int e2, T* out_re, T* out_im) {
    const int32_t a0 = __ldg(faces + 3 * f1 + e1);
    const int32_t a1 = __ldg(faces + 3 * f1 + (e1 + 1) % 3);
    const int32_t a2 = __ldg(faces + 3 * f1 + (e1 + 2) % 3);
    const int32_t b0 = __ldg(faces + 3 * f2 + e2);
    const int32_t b1 = __ldg(faces + 3 * f2 + (e2 + 1) % 3);
    const int32_t b2 = __ldg(faces + 3 * f2 + (e2 + 2) % 3);
    const V3<T> o = load3(verts, b0);
    const V3<T> A0 = load3(verts, a0) - o;
    const V3<T> A1 = load3(verts, a1) - o;
    const V3<T> A2 = load3(verts, a2) - o;
    const V3<T> B1 = load3(verts, b1) - o;
    const V3<T> B2 = load3(verts, b2) - o;
    const V3<T> n1 = load3(normals, f1);
    const T area1 = __ldg(areas + f1), area2 = __ldg(areas + f2);
    const V3<T> d1 = A2 - A1, d2 = B2 - B1;
    const T c1 = (a1 < a2 ? T(1) : T(-1)) * sqrt_t(dot(d1, d1)) / (T(2) * area1);
    const T c2 = (b1 < b2 ? T(1) : T(-1)) * sqrt_t(dot(d2, d2)) / (T(2) * area2);
    const T k_turn = k * T(kInv2Pi);  // kR / (2 pi) per unit R
    const T inv_k = T(1) / k;
    const T src_scale = T(2) * area2 * T(kInv4Pi);

    T ysx[NS > 0 ? NS : 1], ysy[NS > 0 ? NS : 1], ysz[NS > 0 ? NS : 1], ysw[NS > 0 ? NS : 1];
    if constexpr (NS > 0) {
#pragma unroll
        for (int j = 0; j < NS; ++j) {
            constexpr int NY = NS == 1 ? 1 : (NS == 4 ? 2 : (NS == 9 ? 3 : 4));
            const int ji = j / NY, jj = j % NY;
            const T r3 = s_py[ji];
            const T r4 = s_py[jj] * r3;
            // y - B0 = (r3 - r4)(B1 - B0) + r4 (B2 - B0), B0 = 0 after the shift
            ysx[j] = (r3 - r4) * B1.x + r4 * B2.x;
            ysy[j] = (r3 - r4) * B1.y + r4 * B2.y;
            ysz[j] = (r3 - r4) * B1.z + r4 * B2.z;
            ysw[j] = s_wy[ji] * s_wy[jj] * src_scale * r3;
        }
    }

    T acc_re = 0, acc_im = 0, self_acc = 0;
    const bool same = (f1 == f2);
    const int nt = nx * nx;
    for (int i = 0; i < nt; ++i) {
        const T r1 = s_px[i / nx];
        const T r2 = s_px[i % nx] * r1;
        const T w1 = s_wx[i / nx] * s_wx[i % nx] * (T(2) * area1) * r1;
        const V3<T> x = (T(1) - r1) * A0 + (r1 - r2) * A1 + r2 * A2;
        T s0r = 0, s0i = 0, s1xr = 0, s1xi = 0, s1yr = 0, s1yi = 0, s1zr = 0, s1zi = 0;
        T h1xr = 0, h1xi = 0, h1yr = 0, h1yi = 0, h1zr = 0, h1zi = 0;
        const int ns = (NS > 0) ? NS : ny * ny;
#pragma unroll
        for (int j = 0; j < (NS > 0 ? NS : 1); ++j) {
            // NS > 0 branch (registers); NS == 0 handled in the loop below
            if constexpr (NS > 0) {
                const T dx = x.x - ysx[j], dy = x.y - ysy[j], dz = x.z - ysz[j];
                const T r2d = dx * dx + dy * dy + dz * dz;
                const T rinv = rsqrt_t(r2d);
                const T R = r2d * rinv;
                T sn, cs;
                sincos_turns(k_turn * R, &sn, &cs);
                const T g = ysw[j] * rinv;
                const T gr = g * cs, gi = -g * sn;  // e^{-jkR}/(4 pi R) * weight
                const T kR = k * R;
                const T rinv2 = rinv * rinv;
                const T hr = (gr - gi * kR) * rinv2;  // G (1 + jkR) / R^2
                const T hi = (gi + gr * kR) * rinv2;
                s0r += gr; s0i += gi;
                s1xr += gr * ysx[j]; s1xi += gi * ysx[j];
                s1yr += gr * ysy[j]; s1yi += gi * ysy[j];
                s1zr += gr * ysz[j]; s1zi += gi * ysz[j];
                h1xr += hr * ysx[j]; h1xi += hi * ysx[j];
                h1yr += hr * ysy[j]; h1yi += hi * ysy[j];
                h1zr += hr * ysz[j]; h1zi += hi * ysz[j];
            }
        }
        if constexpr (NS == 0) {
            for (int j = 0; j < ns; ++j) {
                const T r3 = s_py[j / ny];
                const T r4 = s_py[j % ny] * r3;
                const T yx = (r3 - r4) * B1.x + r4 * B2.x;
                const T yy = (r3 - r4) * B1.y + r4 * B2.y;
                const T yz = (r3 - r4) * B1.z + r4 * B2.z;
                const T yw = s_wy[j / ny] * s_wy[j % ny] * src_scale * r3;
                const T dx = x.x - yx, dy = x.y - yy, dz = x.z - yz;
                const T r2d = dx * dx + dy * dy + dz * dz;
                const T rinv = rsqrt_t(r2d);
                const T R = r2d * rinv;
                T sn, cs;
                sincos_turns(k_turn * R, &sn, &cs);
                const T g = yw * rinv;
                const T gr = g * cs, gi = -g * sn;
                const T kR = k * R;
                const T rinv2 = rinv * rinv;
                const T hr = (gr - gi * kR) * rinv2;
                const T hi = (gi + gr * kR) * rinv2;
                s0r += gr; s0i += gi;
                s1xr += gr * yx; s1xi += gi * yx;
                s1yr += gr * yy; s1yi += gi * yy;
                s1zr += gr * yz; s1zi += gi * yz;
                h1xr += hr * yx; h1xi += hi * yx;
                h1yr += hr * yy; h1yi += hi * yy;
                h1zr += hr * yz; h1zi += hi * yz;
            }
        }
        const V3<T> a = x - A0;
        const V3<T> u = cross(x, cross(a, n1));
        const T hu_r = h1xr * u.x + h1yr * u.y + h1zr * u.z;
        const T hu_i = h1xi * u.x + h1yi * u.y + h1zi * u.z;
        const T p_r = s1xr * a.x + s1yr * a.y + s1zr * a.z;
        const T p_i = s1xi * a.x + s1yi * a.y + s1zi * a.z;
        // -H1.u + jk (a.S1) - (4j/k) S0
        const T t_re = -hu_r - k * p_i + T(4) * inv_k * s0i;
        const T t_im = -hu_i + k * p_r - T(4) * inv_k * s0r;
        acc_re += w1 * t_re;
        acc_im += w1 * t_im;
        if (same) self_acc += w1 * dot(a, x);  // (x - A0) . (x - B0), B0 = 0
    }
    const T cc = c1 * c2;
    *out_re = cc * (acc_re + T(0.5) * self_acc);
    *out_im = cc * acc_im;
}

// Face-edge layout [batch, 3F, 3F], split real/imag (drop-in for the reference op).
// grid.x = rows * col_blocks, block = kThreads columns.
template <typename T, int NS>
__global__ void __launch_bounds__(128) mom_ref_zmat_fe_kernel(
    const T* __restrict__ verts, const int32_t* __restrict__ faces, const T* __restrict__ areas,
    const T* __restrict__ normals, const T* __restrict__ gpx, const T* __restrict__ gwx, int nx,
    const T* __restrict__ gpy, const T* __restrict__ gwy, int ny, T k, int64_t nf, int64_t batch,
    int64_t col_blocks, T* __restrict__ zr, T* __restrict__ zi) {
    __shared__ T s_px[16], s_wx[16], s_py[16], s_wy[16];
    if (threadIdx.x < nx) { s_px[threadIdx.x] = gpx[threadIdx.x]; s_wx[threadIdx.x] = gwx[threadIdx.x]; }
    if (threadIdx.x < ny) { s_py[threadIdx.x] = gpy[threadIdx.x]; s_wy[threadIdx.x] = gwy[threadIdx.x]; }
    __syncthreads();
    const int64_t ncol = 3 * nf;
    const int64_t row = (int64_t)blockIdx.x / col_blocks;
    const int64_t col = ((int64_t)blockIdx.x % col_blocks) * blockDim.x + threadIdx.x;
    if (col >= ncol) return;
    T re, im;
    mom_entry<T, NS>(verts, faces, areas, normals, s_px, s_wx, nx, s_py, s_wy, ny, k, row / 3,
                     (int)(row % 3), col / 3, (int)(col % 3), &re, &im);
    for (int64_t b = 0; b < batch; ++b) {
        const int64_t o = (b * ncol + row) * ncol + col;
        zr[o] = re;
        zi[o] = im;
    }
}

// RWG layout: Z[fei[row], fei[col]] += entry, interleaved complex [E, E] (caller zeroes).
// Every Z_mn receives its four face-pair contributions through vector atomics.
template <typename T>
__device__ __forceinline__ void atomic_add_c(T* p, T re, T im);
template <>
__device__ __forceinline__ void atomic_add_c<float>(float* p, float re, float im) {
    atomicAdd(reinterpret_cast<float2*>(p), make_float2(re, im));
}
template <>
__device__ __forceinline__ void atomic_add_c<double>(double* p, double re, double im) {
    atomicAdd(p, re);
    atomicAdd(p + 1, im);
}

template <typename T, int NS>
__global__ void __launch_bounds__(128) mom_ref_zmat_rwg_kernel(
    const T* __restrict__ verts, const int32_t* __restrict__ faces, const T* __restrict__ areas,
    const T* __restrict__ normals, const int32_t* __restrict__ fei, int64_t n_edges,
    const T* __restrict__ gpx, const T* __restrict__ gwx, int nx, const T* __restrict__ gpy,
    const T* __restrict__ gwy, int ny, T k, int64_t nf, int64_t row_begin, int64_t col_blocks,
    T* __restrict__ z) {
    __shared__ T s_px[16], s_wx[16], s_py[16], s_wy[16];
    if (threadIdx.x < nx) { s_px[threadIdx.x] = gpx[threadIdx.x]; s_wx[threadIdx.x] = gwx[threadIdx.x]; }
    if (threadIdx.x < ny) { s_py[threadIdx.x] = gpy[threadIdx.x]; s_wy[threadIdx.x] = gwy[threadIdx.x]; }
    __syncthreads();
    const int64_t ncol = 3 * nf;
    const int64_t row = row_begin + (int64_t)blockIdx.x / col_blocks;
    const int64_t col = ((int64_t)blockIdx.x % col_blocks) * blockDim.x + threadIdx.x;
    if (col >= ncol) return;
    T re, im;
    mom_entry<T, NS>(verts, faces, areas, normals, s_px, s_wx, nx, s_py, s_wy, ny, k, row / 3,
                     (int)(row % 3), col / 3, (int)(col % 3), &re, &im);
    const int64_t m = __ldg(fei + row), n = __ldg(fei + col);
    atomic_add_c<T>(z + 2 * (m * n_edges + n), re, im);
}

// ---------------------------------------------------------------------------------------
// float fast path: compile-time rule sizes, projected moments, packed f32x2 arithmetic.
//
// Per test point x_i the entry needs only three complex sums over the source points:
//   S0 = sum G,   P = sum G (y.a),   Q = sum G (1 + jkR) R^-2 (y.u)
// with a = x - A0 and u = x x (a x n1) = a (x.n1) - n1 (x.a), because the old vector
// moments were only ever used as a.S1 and u.H1.  y.a = r1 (y.e1) + r2 (y.e2) with the test
// edge vectors e1 = A1 - A0, e2 = A2 - A1, so per source point the kernel keeps (y, w,
// y.e1, y.e2, y.n1) in registers and an evaluation costs ~26 FP32 ops.  Two source points
// ride in one packed f32x2 instruction (Blackwell `fma/mul/add/sub.rn.f32x2`); the SFU does
// rsqrt, sin and cos.  The entry is then
//   c1 c2 sum_i w_i [ -Q + jk P - (4j/k) S0 ]  (+ self term), identical to mom_entry.
// ---------------------------------------------------------------------------------------


// Rule tables staged in shared memory: test (r1, r2, w_a w_b r1), source
// (r3, r4, w_a w_b r3 / (4 pi)); index b*n + a as in the reference loops (:410-415).
template <int NX, int NY>
__device__ __forceinline__ void stage_rules(const float* gpx, const float* gwx, const float* gpy,
                                            const float* gwy, float4* s_t, float4* s_s) {
    const int t = threadIdx.x;
    if (t < NX * NX) {
        const float r1 = gpx[t / NX];
        s_t[t] = make_float4(r1, gpx[t % NX] * r1, gwx[t / NX] * gwx[t % NX] * r1, 0.f);
    } else if (t < NX * NX + NY * NY) {
        const int j = t - NX * NX;
        const float r3 = gpy[j / NY];
        s_s[j] = make_float4(r3, gpy[j % NY] * r3, gwy[j / NY] * gwy[j % NY] * r3 * float(kInv4Pi), 0.f);
    }
}

template <int NX, int NY>
__device__ __forceinline__ void mom_entry_fast(const float* __restrict__ verts,
                                               const int32_t* __restrict__ faces,
                                               const float* __restrict__ areas,
                                               const float* __restrict__ normals, const float4* s_t,
                                               const float4* s_s, float k, int64_t f1, int e1, int64_t f2,
                                               int e2, float* out_re, float* out_im) {
    // NP full pairs of source points in packed f32x2 registers; an odd count leaves one
    // source point (TAIL) that is evaluated with scalar instructions.
    constexpr int NT = NX * NX, NS = NY * NY, NP = NS / 2, TAIL = NS & 1;
    const int32_t a0 = __ldg(faces + 3 * f1 + e1);
    const int32_t a1 = __ldg(faces + 3 * f1 + (e1 + 1) % 3);
    const int32_t a2 = __ldg(faces + 3 * f1 + (e1 + 2) % 3);
    const int32_t b0 = __ldg(faces + 3 * f2 + e2);
    const int32_t b1 = __ldg(faces + 3 * f2 + (e2 + 1) % 3);
    const int32_t b2 = __ldg(faces + 3 * f2 + (e2 + 2) % 3);
    const V3<float> o = load3(verts, b0);
    const V3<float> A0 = load3(verts, a0) - o;
    const V3<float> A1 = load3(verts, a1) - o;
    const V3<float> A2 = load3(verts, a2) - o;
    const V3<float> B1 = load3(verts, b1) - o;
    const V3<float> B2 = load3(verts, b2) - o;
    const V3<float> n1 = load3(normals, f1);
    const float area1 = __ldg(areas + f1), area2 = __ldg(areas + f2);
    const V3<float> ev1 = A1 - A0, ev2 = A2 - A1;
    const V3<float> d2 = B2 - B1;
    const float c1 = (a1 < a2 ? 1.f : -1.f) * sqrtf(dot(ev2, ev2)) / (2.f * area1);
    const float c2 = (b1 < b2 ? 1.f : -1.f) * sqrtf(dot(d2, d2)) / (2.f * area2);

    // Source points (origin B0) packed two per register pair: coordinates scaled by k (only
    // distances use them: |k x - k y| = kR), the weight k w (so g = w / R = (k w) / (kR)), and
    // the projections k (y.e1), k (y.e2) on the test edge vectors and y.n1 on the normal.
    float2 yx[NP > 0 ? NP : 1], yy[NP > 0 ? NP : 1], yz[NP > 0 ? NP : 1], yw[NP > 0 ? NP : 1],
        ye1[NP > 0 ? NP : 1], ye2[NP > 0 ? NP : 1], yn[NP > 0 ? NP : 1];
    float tx = 0.f, ty = 0.f, tz = 0.f, tw = 0.f, te1 = 0.f, te2 = 0.f, tn = 0.f;  // the tail point
#pragma unroll
    for (int j = 0; j < NS; ++j) {
        const float4 r = s_s[j];
        const V3<float> y = (r.x - r.y) * B1 + r.y * B2;
        const float w = r.z * (2.f * area2) * k;
        if (j < 2 * NP) {
            (reinterpret_cast<float*>(&yx[j / 2]) + (j & 1))[0] = k * y.x;
            (reinterpret_cast<float*>(&yy[j / 2]) + (j & 1))[0] = k * y.y;
            (reinterpret_cast<float*>(&yz[j / 2]) + (j & 1))[0] = k * y.z;
            (reinterpret_cast<float*>(&yw[j / 2]) + (j & 1))[0] = w;
            (reinterpret_cast<float*>(&ye1[j / 2]) + (j & 1))[0] = k * dot(y, ev1);
            (reinterpret_cast<float*>(&ye2[j / 2]) + (j & 1))[0] = k * dot(y, ev2);
            (reinterpret_cast<float*>(&yn[j / 2]) + (j & 1))[0] = dot(y, n1);
        } else {
            tx = k * y.x;
            ty = k * y.y;
            tz = k * y.z;
            tw = w;
            te1 = k * dot(y, ev1);
            te2 = k * dot(y, ev2);
            tn = dot(y, n1);
        }
    }
    // Per evaluation, with c = k (y.a) - 4/k, yu = (y.a)(x.n1) - (y.n1)(x.a), m = -R^-2 yu and
    // G = gr - j gs:  t_re += gs c + m Re[G(1 + jkR)],  t_im += gr c + m Im[G(1 + jkR)]
    // (Re = gr + gs kR, Im = gr kR - gs), i.e. the per-test-point combination
    // -Q + jk P - (4j/k) S0 of the three sums, summed directly.  yu = c (x.n1)/k + (4 (x.n1)/k^2 - (y.n1)(x.a)) and R^-2 = k^2 (kR)^-2, so
    // -R^-2 yu = (kR)^-2 [c (-k (x.n1)) + (y.n1) k^2 (x.a) - 4 (x.n1)].
    const float2 M4K = bc(-4.f / k);
    float2 acc_re = bc(0.f), acc_im = bc(0.f);
    float self_acc = 0.f;
    const bool same = (f1 == f2);
    // The test-point loop stays rolled: its body (the unrolled source loop) is ~2 KB of
    // code, and unrolling it 16 times overflows the instruction cache.
#pragma unroll 1
    for (int i = 0; i < NT; ++i) {
        const float4 t = s_t[i];
        const float w1 = t.z * (2.f * area1);
        const V3<float> a = t.x * ev1 + t.y * ev2;
        const V3<float> x = A0 + a;
        const float xn = dot(x, n1), xa = dot(x, a);
        const float2 X = bc(k * x.x), Y = bc(k * x.y), Z = bc(k * x.z), R1 = bc(t.x), R2 = bc(t.y),
                     CN = bc(-k * xn), CA = bc(k * k * xa), C4 = bc(-4.f * xn);
        float2 tr = bc(0.f), ti = bc(0.f);
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const float2 dx = sub2(X, yx[p]);
            const float2 dy = sub2(Y, yy[p]);
            const float2 dz = sub2(Z, yz[p]);
            const float2 r2d = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));  // (kR)^2
            float2 rinv;                                                 // (kR)^-1
            rinv.x = rsqrtf(r2d.x);
            rinv.y = rsqrtf(r2d.y);
            const float2 kR = mul2(r2d, rinv);
            float2 sn, cs;
            __sincosf(kR.x, &sn.x, &cs.x);
            __sincosf(kR.y, &sn.y, &cs.y);
            const float2 g = mul2(yw[p], rinv);
            const float2 gr = mul2(g, cs), gs = mul2(g, sn);  // G = gr - j gs
            const float2 c = fma2(R1, ye1[p], fma2(R2, ye2[p], M4K));
            const float2 nyu = fma2(c, CN, fma2(yn[p], CA, C4));  // -k^2 yu
            const float2 m = mul2(mul2(rinv, rinv), nyu);         // -R^-2 yu
            // m G(1 + jkR) + c G in the conjugate form (gr + j gs)(u + j m), u = m kR + c
            const float2 u = fma2(m, kR, c);
            tr = fma2(gs, u, fma2(m, gr, tr));
            ti = sub2(fma2(gr, u, ti), mul2(m, gs));
        }
        if constexpr (TAIL) {
            // the odd source point, scalar: same algebra as one lane of the packed loop
            const float dx = k * x.x - tx, dy = k * x.y - ty, dz = k * x.z - tz;
            const float r2d = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const float rinv = rsqrtf(r2d);
            const float kR = r2d * rinv;
            float sn, cs;
            __sincosf(kR, &sn, &cs);
            const float g = tw * rinv;
            const float gr = g * cs, gs = g * sn;
            const float c = fmaf(t.x, te1, fmaf(t.y, te2, -4.f / k));
            const float nyu = fmaf(c, -k * xn, fmaf(tn, k * k * xa, -4.f * xn));
            const float m = rinv * rinv * nyu;
            const float u = fmaf(m, kR, c);
            tr.x = fmaf(gs, u, fmaf(m, gr, tr.x));
            ti.x = fmaf(gr, u, fmaf(-m, gs, ti.x));
        }
        const float2 W1 = bc(w1);
        acc_re = fma2(W1, tr, acc_re);
        acc_im = fma2(W1, ti, acc_im);
        if (same) self_acc += w1 * xa;  // (x - A0) . (x - B0), B0 = 0
    }
    const float cc = c1 * c2;
    *out_re = cc * (acc_re.x + acc_re.y + 0.5f * self_acc);
    *out_im = cc * (acc_im.x + acc_im.y);
}

#ifndef MB_FAST_MIN_BLOCKS
#define MB_FAST_MIN_BLOCKS 4
#endif
template <int NX, int NY, bool RWG>
__global__ void __launch_bounds__(128, NX <= 4 ? MB_FAST_MIN_BLOCKS : 2) mom_ref_zmat_fast_kernel(
    const float* __restrict__ verts, const int32_t* __restrict__ faces, const float* __restrict__ areas,
    const float* __restrict__ normals, const int32_t* __restrict__ fei, int64_t n_edges,
    const float* __restrict__ gpx, const float* __restrict__ gwx, const float* __restrict__ gpy,
    const float* __restrict__ gwy, float k, int64_t nf, int64_t batch, int64_t row_begin,
    int64_t col_blocks, float* __restrict__ zr, float* __restrict__ zi) {
    __shared__ float4 s_t[NX * NX], s_s[NY * NY];
    stage_rules<NX, NY>(gpx, gwx, gpy, gwy, s_t, s_s);
    __syncthreads();
    const int64_t ncol = 3 * nf;
    const int64_t row = row_begin + (int64_t)blockIdx.x / col_blocks;
    const int64_t col = ((int64_t)blockIdx.x % col_blocks) * blockDim.x + threadIdx.x;
    if (col >= ncol) return;
    float re, im;
    mom_entry_fast<NX, NY>(verts, faces, areas, normals, s_t, s_s, k, row / 3, (int)(row % 3), col / 3,
                           (int)(col % 3), &re, &im);
    if constexpr (RWG) {
        const int64_t m = __ldg(fei + row), n = __ldg(fei + col);
        atomicAdd(reinterpret_cast<float2*>(zr + 2 * (m * n_edges + n)), make_float2(re, im));
    } else {
        for (int64_t b = 0; b < batch; ++b) {
            const int64_t o = (b * ncol + row) * ncol + col;
            zr[o] = re;
            zi[o] = im;
        }
    }
}

// Edge-row order (RWG layout): block row m is Z row m, i.e. edge m; its (at most two)
// face-edge test rows edge_rows[2m], edge_rows[2m + 1] (3 f + e, or -1) are evaluated by the
// same thread and summed before one atomic per entry, and Z row m is complete when its
// blocks end -- so row ranges can be assembled and copied out in chunks.
template <int NX, int NY>
__global__ void __launch_bounds__(128, NX <= 4 ? MB_FAST_MIN_BLOCKS : 2) mom_ref_zmat_edge_kernel(
    const float* __restrict__ verts, const int32_t* __restrict__ faces, const float* __restrict__ areas,
    const float* __restrict__ normals, const int32_t* __restrict__ fei, const int32_t* __restrict__ edge_rows,
    int64_t n_edges, const float* __restrict__ gpx, const float* __restrict__ gwx, const float* __restrict__ gpy,
    const float* __restrict__ gwy, float k, int64_t nf, int64_t m_begin, int64_t col_blocks,
    float* __restrict__ z) {
    __shared__ float4 s_t[NX * NX], s_s[NY * NY];
    stage_rules<NX, NY>(gpx, gwx, gpy, gwy, s_t, s_s);
    __syncthreads();
    const int64_t ncol = 3 * nf;
    const int64_t m = m_begin + (int64_t)blockIdx.x / col_blocks;
    const int64_t col = ((int64_t)blockIdx.x % col_blocks) * blockDim.x + threadIdx.x;
    if (col >= ncol) return;
    float re = 0.f, im = 0.f;
#pragma unroll 1
    for (int j = 0; j < 2; ++j) {
        const int32_t row = __ldg(edge_rows + 2 * m + j);
        if (row < 0) continue;
        float a, b;
        mom_entry_fast<NX, NY>(verts, faces, areas, normals, s_t, s_s, k, row / 3, row % 3, col / 3,
                               (int)(col % 3), &a, &b);
        re += a;
        im += b;
    }
    atomicAdd(reinterpret_cast<float2*>(z + 2 * (m * n_edges + __ldg(fei + col))), make_float2(re, im));
}

// Gather form (RWG layout): thread (m, n) owns Z[m, n] and sums the (at most 2 x 2) face-edge
// entries of test edge m and source edge n -- every face-edge pair still evaluated exactly
// once -- then writes the entry with one coalesced store: no atomics, and no zeroing pass
// (rows [m_begin, m_end) are overwritten).
template <int NX, int NY>
__global__ void __launch_bounds__(128, NX <= 4 ? MB_FAST_MIN_BLOCKS : 2) mom_ref_zmat_gather_kernel(
    const float* __restrict__ verts, const int32_t* __restrict__ faces, const float* __restrict__ areas,
    const float* __restrict__ normals, const int32_t* __restrict__ edge_rows, int64_t n_edges,
    const float* __restrict__ gpx, const float* __restrict__ gwx, const float* __restrict__ gpy,
    const float* __restrict__ gwy, float k, int64_t m_begin, int64_t col_blocks, float* __restrict__ z) {
    __shared__ float4 s_t[NX * NX], s_s[NY * NY];
    stage_rules<NX, NY>(gpx, gwx, gpy, gwy, s_t, s_s);
    __syncthreads();
    const int64_t m = m_begin + (int64_t)blockIdx.x / col_blocks;
    const int64_t n = ((int64_t)blockIdx.x % col_blocks) * blockDim.x + threadIdx.x;
    if (n >= n_edges) return;
    float re = 0.f, im = 0.f;
#pragma unroll 1
    for (int j = 0; j < 2; ++j) {
        const int32_t row = __ldg(edge_rows + 2 * m + j);
        if (row < 0) continue;
#pragma unroll 1
        for (int q = 0; q < 2; ++q) {
            const int32_t col = __ldg(edge_rows + 2 * n + q);
            if (col < 0) continue;
            float a, b;
            mom_entry_fast<NX, NY>(verts, faces, areas, normals, s_t, s_s, k, row / 3, row % 3, col / 3, col % 3,
                                   &a, &b);
            re += a;
            im += b;
        }
    }
    reinterpret_cast<float2*>(z)[m * n_edges + n] = make_float2(re, im);
}

// Edge -> face-edge rows: slot 0 the smaller row, slot 1 the larger (or -1 for a boundary
// edge); edge_rows[2E] is set to 1 when some edge has more than two faces.
__global__ void edge_rows_init(int32_t* __restrict__ er, int64_t n_edges) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m < n_edges) {
        er[2 * m] = 0x7fffffff;
        er[2 * m + 1] = -1;
    }
    if (m == 0) er[2 * n_edges] = 0;
}
__global__ void edge_rows_minmax(const int32_t* __restrict__ fei, int64_t nfe, int32_t* __restrict__ er) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nfe) return;
    const int32_t m = fei[r];
    atomicMin(er + 2 * m, (int32_t)r);
    atomicMax(er + 2 * m + 1, (int32_t)r);
}
__global__ void edge_rows_check(const int32_t* __restrict__ fei, int64_t nfe, int64_t n_edges, int32_t* er) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nfe) return;
    const int32_t m = fei[r];
    if (r != er[2 * m] && r != er[2 * m + 1]) er[2 * n_edges] = 1;
}
__global__ void edge_rows_finish(int32_t* __restrict__ er, int64_t n_edges) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_edges) return;
    if (er[2 * m] == 0x7fffffff) er[2 * m] = -1;
    if (er[2 * m + 1] == er[2 * m]) er[2 * m + 1] = -1;
}

int launch_edge_rows(const int32_t* fei, int64_t nf, int64_t n_edges, int32_t* er, cudaStream_t s) {
    const int64_t nfe = 3 * nf;
    const unsigned be = (unsigned)((n_edges + 255) / 256 + 1), bf = (unsigned)((nfe + 255) / 256 + 1);
    edge_rows_init<<<be, 256, 0, s>>>(er, n_edges);
    edge_rows_minmax<<<bf, 256, 0, s>>>(fei, nfe, er);
    edge_rows_check<<<bf, 256, 0, s>>>(fei, nfe, n_edges, er);
    edge_rows_finish<<<be, 256, 0, s>>>(er, n_edges);
    return check_launch("edge_rows");
}

// Edge-row launch over Z rows [m_begin, m_end) for the float fast path; false when the rule
// sizes have no fast instance.
bool launch_fast_zmat_edges(const float* verts, const int32_t* faces, const float* areas, const float* normals,
                            const int32_t* fei, const int32_t* edge_rows, int64_t n_edges, const float* gpx,
                            const float* gwx, int nx, const float* gpy, const float* gwy, int ny, double k,
                            int64_t nf, int64_t m_begin, int64_t m_end, float* z, cudaStream_t stream) {
    const int64_t col_blocks = (3 * nf + 127) / 128;
    const int64_t blocks = (m_end - m_begin) * col_blocks;
    if (blocks <= 0) return true;
#define MB_FAST_E(NXV, NYV)                                                                           \
    if (nx == NXV && ny == NYV) {                                                                     \
        mom_ref_zmat_edge_kernel<NXV, NYV><<<(unsigned)blocks, 128, 0, stream>>>(                      \
            verts, faces, areas, normals, fei, edge_rows, n_edges, gpx, gwx, gpy, gwy, (float)k, nf,   \
            m_begin, col_blocks, z);                                                                  \
        return true;                                                                                  \
    }
    MB_FAST_E(4, 3)
    MB_FAST_E(3, 2)
    MB_FAST_E(2, 1)
    MB_FAST_E(5, 4)
#undef MB_FAST_E
    return false;
}

// Z to host memory with the copy overlapped: Z rows are assembled in `chunks` edge-row
// ranges on stream s, each range copied to z_host on a second stream as soon as its kernel
// ends (z_dev: device scratch [E, E]; edge_rows: from launch_edge_rows, every edge at most
// two faces).  The calling stream waits for the last copy.
// Gather-form launch over Z rows [m_begin, m_end) (overwritten); false when the rule sizes
// have no fast instance.
bool launch_fast_zmat_gather(const float* verts, const int32_t* faces, const float* areas, const float* normals,
                             const int32_t* edge_rows, int64_t n_edges, const float* gpx, const float* gwx, int nx,
                             const float* gpy, const float* gwy, int ny, double k, int64_t m_begin, int64_t m_end,
                             float* z, cudaStream_t stream) {
    const int64_t col_blocks = (n_edges + 127) / 128;
    const int64_t blocks = (m_end - m_begin) * col_blocks;
    if (blocks <= 0) return true;
#define MB_FAST_G(NXV, NYV)                                                                           \
    if (nx == NXV && ny == NYV) {                                                                     \
        mom_ref_zmat_gather_kernel<NXV, NYV><<<(unsigned)blocks, 128, 0, stream>>>(                    \
            verts, faces, areas, normals, edge_rows, n_edges, gpx, gwx, gpy, gwy, (float)k, m_begin,    \
            col_blocks, z);                                                                           \
        return true;                                                                                  \
    }
    MB_FAST_G(4, 3)
    MB_FAST_G(3, 2)
    MB_FAST_G(2, 1)
    MB_FAST_G(5, 4)
#undef MB_FAST_G
    return false;
}

int zmat_edges_to_host(const float* verts, const int32_t* faces, const float* areas, const float* normals,
                       const int32_t* fei, const int32_t* edge_rows, int64_t n_edges, const float* gpx,
                       const float* gwx, int nx, const float* gpy, const float* gwy, int ny, double k, int64_t nf,
                       float* z_dev, float* z_host, int chunks, cudaStream_t s) {
    chunks = std::max(1, std::min(chunks, 256));
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
        return set_error(MB_ERR_CUDA, "zmat to host: copy stream");
    std::vector<cudaEvent_t> ev((size_t)chunks + 1, nullptr);
    int rc = MB_OK;
    for (auto& e : ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = MB_ERR_CUDA;
    if (rc == MB_OK) {
        for (int c = 0; c < chunks; ++c) {
            const int64_t m0 = n_edges * c / chunks, m1 = n_edges * (c + 1) / chunks;
            if (m1 <= m0) continue;
            const size_t off = (size_t)m0 * n_edges * 2, bytes = (size_t)(m1 - m0) * n_edges * 8;
            cudaMemsetAsync(z_dev + off, 0, bytes, s);
            if (!launch_fast_zmat_edges(verts, faces, areas, normals, fei, edge_rows, n_edges, gpx, gwx, nx, gpy,
                                        gwy, ny, k, nf, m0, m1, z_dev, s)) {
                rc = set_error(MB_ERR_UNSUPPORTED, "zmat to host: no fast rule (%d, %d)", nx, ny);
                break;
            }
            cudaEventRecord(ev[c], s);
            cudaStreamWaitEvent(cs, ev[c], 0);
            cudaMemcpyAsync(z_host + off, z_dev + off, bytes, cudaMemcpyDeviceToHost, cs);
        }
        cudaEventRecord(ev[chunks], cs);
        cudaStreamWaitEvent(s, ev[chunks], 0);
    } else {
        rc = set_error(MB_ERR_CUDA, "zmat to host: events");
    }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    cudaStreamDestroy(cs);
    if (rc) return rc;
    return check_launch("zmat to host");
}

// Launches the fast path for float and supported rule sizes; returns false otherwise.
template <typename T>
bool launch_fast_zmat(const T*, const int32_t*, const T*, const T*, const int32_t*, int64_t, const T*,
                      const T*, int, const T*, const T*, int, double, int64_t, int64_t, int64_t, int64_t,
                      unsigned, T*, T*, cudaStream_t) {
    return false;
}
template <>
bool launch_fast_zmat<float>(const float* verts, const int32_t* faces, const float* areas,
                             const float* normals, const int32_t* fei, int64_t n_edges, const float* gpx,
                             const float* gwx, int nx, const float* gpy, const float* gwy, int ny, double k,
                             int64_t nf, int64_t batch, int64_t row_begin, int64_t col_blocks,
                             unsigned blocks, float* zr, float* zi, cudaStream_t stream) {
#define MB_FAST(NXV, NYV)                                                                          \
    if (nx == NXV && ny == NYV) {                                                                  \
        if (fei)                                                                                   \
            mom_ref_zmat_fast_kernel<NXV, NYV, true><<<blocks, 128, 0, stream>>>(                   \
                verts, faces, areas, normals, fei, n_edges, gpx, gwx, gpy, gwy, (float)k, nf, batch,  \
                row_begin, col_blocks, zr, zi);                                                    \
        else                                                                                       \
            mom_ref_zmat_fast_kernel<NXV, NYV, false><<<blocks, 128, 0, stream>>>(                  \
                verts, faces, areas, normals, fei, n_edges, gpx, gwx, gpy, gwy, (float)k, nf, batch,  \
                row_begin, col_blocks, zr, zi);                                                    \
        return true;                                                                               \
    }
    MB_FAST(4, 3)
    MB_FAST(3, 2)
    MB_FAST(2, 1)
    MB_FAST(5, 4)
#undef MB_FAST
    return false;
}

// ---------------------------------------------------------------------------------------
// Excitation (mesh_MOM_3d.cu:244-330).  One thread per face-edge and right-hand side.
// Plane wave E = e0 exp(-j k khat.x), H = (khat x e0)/eta exp(-j k khat.x); the
// reference's hard-coded wave is khat = (cos 30, sin 30, 0), e0 = z, eta = 1.
// out_mode 0: face-edge split [B, F, 3] (batch copies identical, as the reference).
// out_mode 1: RWG interleaved complex [E, nrhs] accumulated via atomics (caller zeroes).
// ---------------------------------------------------------------------------------------
struct PlaneWave {
    double kx, ky, kz;     // k * khat
    double ex, ey, ez;     // E polarisation
    double hx, hy, hz;     // H = khat x e0 / eta
};

// <f_fe, E + n x H> of one face-edge (face f, local edge e) for one plane wave.
template <typename T>
__device__ __forceinline__ void ref_rhs_entry(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                              const T* __restrict__ areas, const T* __restrict__ normals,
                                              const T* s_p, const T* s_w, int n, const PlaneWave& pw, int64_t f,
                                              int e, T* out_re, T* out_im) {
    const int32_t i0 = faces[3 * f + e], i1 = faces[3 * f + (e + 1) % 3], i2 = faces[3 * f + (e + 2) % 3];
    const V3<T> v0 = load3(verts, i0), v1 = load3(verts, i1), v2 = load3(verts, i2);
    const V3<T> nrm = load3(normals, f);
    const T area = areas[f];
    const V3<T> d = v2 - v1;
    const T c = (i1 < i2 ? T(1) : T(-1)) * sqrt_t(dot(d, d)) / (T(2) * area);
    const V3<T> kv = v3<T>((T)pw.kx, (T)pw.ky, (T)pw.kz);
    const V3<T> E0 = v3<T>((T)pw.ex, (T)pw.ey, (T)pw.ez);
    const V3<T> H0 = v3<T>((T)pw.hx, (T)pw.hy, (T)pw.hz);
    const V3<T> nxh = cross(nrm, H0);
    T acc_r = 0, acc_i = 0;
    for (int i = 0; i < n * n; ++i) {
        const T r1 = s_p[i / n];
        const T r2 = s_p[i % n] * r1;
        const T w = s_w[i / n] * s_w[i % n] * (T(2) * area) * r1;
        const V3<T> x = (T(1) - r1) * v0 + (r1 - r2) * v1 + r2 * v2;
        const V3<T> fv = c * (x - v0);
        T sn, cs;
        sincos_turns(dot(kv, x) * T(kInv2Pi), &sn, &cs);  // e^{-j k.x} = cs - j sn
        const T proj = dot(fv, E0) + dot(fv, nxh);
        acc_r += w * proj * cs;
        acc_i -= w * proj * sn;
    }
    *out_re = acc_r;
    *out_im = acc_i;
}

template <typename T>
__global__ void mom_ref_rhs_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                   const T* __restrict__ areas, const T* __restrict__ normals,
                                   const T* __restrict__ gp, const T* __restrict__ gw, int n,
                                   const PlaneWave* __restrict__ waves, PlaneWave w0, int nrhs, int64_t nf,
                                   int out_mode, int64_t batch, const int32_t* __restrict__ fei,
                                   T* __restrict__ out_r, T* __restrict__ out_i) {
    __shared__ T s_p[16], s_w[16];
    if (threadIdx.x < n) { s_p[threadIdx.x] = gp[threadIdx.x]; s_w[threadIdx.x] = gw[threadIdx.x]; }
    __syncthreads();
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * nf * nrhs) return;
    const int rhs = (int)(idx / (3 * nf));
    const int64_t fe = idx % (3 * nf);
    T acc_r, acc_i;
    ref_rhs_entry<T>(verts, faces, areas, normals, s_p, s_w, n, waves ? waves[rhs] : w0, fe / 3, (int)(fe % 3),
                     &acc_r, &acc_i);
    if (out_mode == 0) {
        for (int64_t b = 0; b < batch; ++b) {
            out_r[b * 3 * nf + fe] = acc_r;
            out_i[b * 3 * nf + fe] = acc_i;
        }
    } else {
        const int64_t m = fei[fe];
        atomic_add_c<T>(out_r + 2 * (m * nrhs + rhs), acc_r, acc_i);
    }
}

// ---------------------------------------------------------------------------------------
// Edge coefficients -> vertex currents (mesh_MOM_3d.cu:498-565).
// mode 0: per-face vertex slots [B, 3F, 3] split real/imag, accumulated (+=) exactly like
//         the reference (each thread owns its face's nine slots).
// mode 1: fused with the vertex scatter of solve_MOM (mesh_BEM_solver_3d.py:185-192):
//         interleaved complex [B, V, 3] accumulated with atomics.
// I is interleaved complex [B, E] in mode 1, split real/imag in mode 0.
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void mom_interp_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                  const int32_t* __restrict__ fei, const T* __restrict__ areas,
                                  const T* __restrict__ ir, const T* __restrict__ ii, int64_t n_edges,
                                  int64_t nf, int64_t nv, int64_t batch, int mode,
                                  T* __restrict__ jr, T* __restrict__ ji) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= batch * nf) return;
    const int64_t b = idx / nf, f = idx % nf;
    const int32_t vid[3] = {faces[3 * f], faces[3 * f + 1], faces[3 * f + 2]};
    const V3<T> p[3] = {load3(verts, vid[0]), load3(verts, vid[1]), load3(verts, vid[2])};
    const T area = areas[f];
    T accr[3][3] = {}, acci[3][3] = {};
    for (int e = 0; e < 3; ++e) {
        const int64_t edge = fei[3 * f + e];
        const int e1 = (e + 1) % 3, e2 = (e + 2) % 3;
        const V3<T> d = p[e2] - p[e1];
        const T c = (vid[e1] < vid[e2] ? T(1) : T(-1)) * sqrt_t(dot(d, d)) / (T(2) * area);
        T Ir, Ii;
        if (mode == 0) {
            Ir = ir[b * n_edges + edge];
            Ii = ii[b * n_edges + edge];
        } else {
            Ir = ir[2 * (b * n_edges + edge)];
            Ii = ir[2 * (b * n_edges + edge) + 1];
        }
        const V3<T> g1 = c * (p[e1] - p[e]);
        const V3<T> g2 = c * (p[e2] - p[e]);
        const T g1a[3] = {g1.x, g1.y, g1.z}, g2a[3] = {g2.x, g2.y, g2.z};
        for (int a = 0; a < 3; ++a) {
            accr[e1][a] += g1a[a] * Ir; acci[e1][a] += g1a[a] * Ii;
            accr[e2][a] += g2a[a] * Ir; acci[e2][a] += g2a[a] * Ii;
        }
    }
    if (mode == 0) {
        const int64_t base = b * nf * 9 + f * 9;
        for (int s = 0; s < 3; ++s)
            for (int a = 0; a < 3; ++a) {
                jr[base + s * 3 + a] += accr[s][a];
                ji[base + s * 3 + a] += acci[s][a];
            }
    } else {
        for (int s = 0; s < 3; ++s)
            for (int a = 0; a < 3; ++a)
                atomic_add_c<T>(jr + 2 * ((b * nv + vid[s]) * 3 + a), accr[s][a], acci[s][a]);
    }
}

// ---------------------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------------------
template <typename T>
int launch_mom_ref_zmat(const T* verts, int64_t nv, const int32_t* faces, int64_t nf, const T* areas,
                        const T* normals, const T* gpx, const T* gwx, int nx, const T* gpy,
                        const T* gwy, int ny, double k, const int32_t* fei, int64_t n_edges,
                        int64_t row_begin, int64_t row_end, int64_t batch, T* zr, T* zi,
                        cudaStream_t stream) {
    (void)nv;
    if (nf <= 0) return MB_OK;
    if (nx < 1 || nx > 16 || ny < 1 || ny > 16)
        return set_error(MB_ERR_UNSUPPORTED, "quadrature order must be in [1, 16] (got %d, %d)", nx, ny);
    if (!(k > 0)) return set_error(MB_ERR_ARG, "wavenumber must be > 0");
    constexpr int threads = 128;
    const int64_t ncol = 3 * nf;
    const int64_t col_blocks = (ncol + threads - 1) / threads;
    const int64_t rows = row_end - row_begin;
    const int64_t blocks = rows * col_blocks;
    if (blocks <= 0) return MB_OK;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
    if (launch_fast_zmat<T>(verts, faces, areas, normals, fei, n_edges, gpx, gwx, nx, gpy, gwy, ny, k, nf,
                            batch, row_begin, col_blocks, (unsigned)blocks, zr, zi, stream))
        return check_launch("mom_ref_zmat");
    const int ns = ny * ny;
#define MB_ZMAT_LAUNCH(NSV)                                                                              \
    do {                                                                                                \
        if (fei == nullptr)                                                                             \
            mom_ref_zmat_fe_kernel<T, NSV><<<(unsigned)blocks, threads, 0, stream>>>(                    \
                verts, faces, areas, normals, gpx, gwx, nx, gpy, gwy, ny, (T)k, nf, batch, col_blocks, zr, \
                zi);                                                                                    \
        else                                                                                            \
            mom_ref_zmat_rwg_kernel<T, NSV><<<(unsigned)blocks, threads, 0, stream>>>(                   \
                verts, faces, areas, normals, fei, n_edges, gpx, gwx, nx, gpy, gwy, ny, (T)k, nf,        \
                row_begin, col_blocks, zr);                                                             \
    } while (0)
    switch (ns) {
        case 1: MB_ZMAT_LAUNCH(1); break;
        case 4: MB_ZMAT_LAUNCH(4); break;
        case 9: MB_ZMAT_LAUNCH(9); break;
        case 16: MB_ZMAT_LAUNCH(16); break;
        default: MB_ZMAT_LAUNCH(0); break;
    }
#undef MB_ZMAT_LAUNCH
    return check_launch("mom_ref_zmat");
}

template int launch_mom_ref_zmat<float>(const float*, int64_t, const int32_t*, int64_t, const float*,
                                        const float*, const float*, const float*, int, const float*,
                                        const float*, int, double, const int32_t*, int64_t, int64_t,
                                        int64_t, int64_t, float*, float*, cudaStream_t);
template int launch_mom_ref_zmat<double>(const double*, int64_t, const int32_t*, int64_t, const double*,
                                         const double*, const double*, const double*, int,
                                         const double*, const double*, int, double, const int32_t*,
                                         int64_t, int64_t, int64_t, int64_t, double*, double*,
                                         cudaStream_t);

// ---------------------------------------------------------------------------------------
// many meshes, the reference's operator and rule: one launch for all impedance matrices and
// one for all excitations.  desc[i] = (first face, faces, edges, offset of Z_i in the flat
// array (complex entries), -, first right-hand-side column); boff [n_mesh + 1] = first
// block of each mesh (3 F_i rows of ceil(3 F_i / 128) blocks); fei holds local edge ids.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ int seg_find(const int64_t* __restrict__ off, int stride, int n, int64_t v) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + (int64_t)stride * mid) <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int NX, int NY>
__global__ void __launch_bounds__(128, NX <= 4 ? MB_FAST_MIN_BLOCKS : 2) mom_ref_zmat_batched_kernel(
    const float* __restrict__ verts, const int32_t* __restrict__ faces, const float* __restrict__ areas,
    const float* __restrict__ normals, const int32_t* __restrict__ fei, const int64_t* __restrict__ desc,
    const int64_t* __restrict__ boff, const double* __restrict__ ks, int n_mesh, const float* __restrict__ gpx,
    const float* __restrict__ gwx, const float* __restrict__ gpy, const float* __restrict__ gwy,
    float* __restrict__ z) {
    __shared__ float4 s_t[NX * NX], s_s[NY * NY];
    stage_rules<NX, NY>(gpx, gwx, gpy, gwy, s_t, s_s);
    __syncthreads();
    const int64_t b = blockIdx.x;
    const int i = seg_find(boff, 1, n_mesh, b);
    const int64_t fo = __ldg(desc + 6 * i), nf = __ldg(desc + 6 * i + 1), ne = __ldg(desc + 6 * i + 2);
    const int64_t ncol = 3 * nf, cb = (ncol + 127) / 128, local = b - __ldg(boff + i);
    const int64_t row = local / cb, col = (local % cb) * 128 + threadIdx.x;
    if (col >= ncol) return;
    float re, im;
    mom_entry_fast<NX, NY>(verts, faces, areas, normals, s_t, s_s, (float)__ldg(ks + i), fo + row / 3,
                           (int)(row % 3), fo + col / 3, (int)(col % 3), &re, &im);
    const int64_t m = __ldg(fei + 3 * fo + row), n = __ldg(fei + 3 * fo + col);
    atomicAdd(reinterpret_cast<float2*>(z + 2 * (__ldg(desc + 6 * i + 3) + m * (ne + (ne & 1)) + n)),
              make_float2(re, im));
}

// Persistent form: one resident grid (SMs x blocks per SM); each block takes work items --
// the same (mesh, row, 128-column tile) items as the grid form's blocks, in the same order --
// from a counter in device memory until they run out.  No wait on another block: a block
// only increments the counter.
template <int NX, int NY>
__global__ void __launch_bounds__(128, NX <= 4 ? MB_FAST_MIN_BLOCKS : 2) mom_ref_zmat_batched_persistent_kernel(
    const float* __restrict__ verts, const int32_t* __restrict__ faces, const float* __restrict__ areas,
    const float* __restrict__ normals, const int32_t* __restrict__ fei, const int64_t* __restrict__ desc,
    const int64_t* __restrict__ boff, int64_t total_items, unsigned long long* queue,
    const double* __restrict__ ks, int n_mesh, const float* __restrict__ gpx, const float* __restrict__ gwx,
    const float* __restrict__ gpy, const float* __restrict__ gwy, float* __restrict__ z) {
    __shared__ float4 s_t[NX * NX], s_s[NY * NY];
    __shared__ long long s_item;
    stage_rules<NX, NY>(gpx, gwx, gpy, gwy, s_t, s_s);
    for (;;) {
        __syncthreads();  // the rules are staged / every thread has read the previous item
        if (threadIdx.x == 0) s_item = (long long)atomicAdd(queue, 1ull);
        __syncthreads();
        const int64_t b = s_item;
        if (b >= total_items) return;
        const int i = seg_find(boff, 1, n_mesh, b);
        const int64_t fo = __ldg(desc + 6 * i), nf = __ldg(desc + 6 * i + 1), ne = __ldg(desc + 6 * i + 2);
        const int64_t ncol = 3 * nf, cb = (ncol + 127) / 128, local = b - __ldg(boff + i);
        const int64_t row = local / cb, col = (local % cb) * 128 + threadIdx.x;
        if (col < ncol) {
            float re, im;
            mom_entry_fast<NX, NY>(verts, faces, areas, normals, s_t, s_s, (float)__ldg(ks + i), fo + row / 3,
                                   (int)(row % 3), fo + col / 3, (int)(col % 3), &re, &im);
            const int64_t m = __ldg(fei + 3 * fo + row), n = __ldg(fei + 3 * fo + col);
            atomicAdd(reinterpret_cast<float2*>(z + 2 * (__ldg(desc + 6 * i + 3) + m * (ne + (ne & 1)) + n)),
                      make_float2(re, im));
        }
    }
}

int launch_mom_ref_zmat_batched(const float* verts, const int32_t* faces, const float* areas, const float* normals,
                                const int32_t* fei, const int64_t* desc, const int64_t* boff, int64_t total_blocks,
                                const double* ks, int n_mesh, const float* gpx, const float* gwx, int nx,
                                const float* gpy, const float* gwy, int ny, float* z, cudaStream_t s,
                                int persistent) {
    if (n_mesh <= 0 || total_blocks <= 0) return MB_OK;
    if (!persistent && total_blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "batch too large for one launch");
    unsigned long long* queue = nullptr;
    unsigned grid = 0;
    if (persistent) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaMallocAsync(reinterpret_cast<void**>(&queue), sizeof(unsigned long long), s) != cudaSuccess) {
            cudaGetLastError();
            return set_error(MB_ERR_CUDA, "mom_ref_zmat_batched: work counter allocation failed");
        }
        cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
        grid = (unsigned)sms;
    }
    int rc = MB_ERR_UNSUPPORTED;
#define MB_RB(NXV, NYV)                                                                                      \
    if (rc == MB_ERR_UNSUPPORTED && nx == NXV && ny == NYV) {                                                \
        if (persistent) {                                                                                    \
            int per_sm = 1;                                                                                  \
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mom_ref_zmat_batched_persistent_kernel<NXV, NYV>, \
                                                          128, 0);                                           \
            const int64_t g = std::min<int64_t>(total_blocks, (int64_t)grid * std::max(per_sm, 1));          \
            mom_ref_zmat_batched_persistent_kernel<NXV, NYV><<<(unsigned)g, 128, 0, s>>>(                    \
                verts, faces, areas, normals, fei, desc, boff, total_blocks, queue, ks, n_mesh, gpx, gwx, gpy, gwy, z); \
        } else {                                                                                             \
            mom_ref_zmat_batched_kernel<NXV, NYV><<<(unsigned)total_blocks, 128, 0, s>>>(                    \
                verts, faces, areas, normals, fei, desc, boff, ks, n_mesh, gpx, gwx, gpy, gwy, z);          \
        }                                                                                                    \
        rc = check_launch("mom_ref_zmat_batched");                                                          \
    }
    MB_RB(4, 3)
    MB_RB(3, 2)
    MB_RB(2, 1)
    MB_RB(5, 4)
#undef MB_RB
    if (queue) cudaFreeAsync(queue, s);
    if (rc == MB_ERR_UNSUPPORTED) return set_error(MB_ERR_UNSUPPORTED, "batched reference rule: gaussQR in {2, 3, 4, 5}");
    return rc;
}

// waves [n_mesh * nrhs] plane-wave records; rhs: [rows, ld] interleaved complex64,
// row = local edge, column desc[i][5] + r (accumulated).
template <typename T>
__global__ void mom_ref_rhs_batched_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                           const T* __restrict__ areas, const T* __restrict__ normals,
                                           const int32_t* __restrict__ fei, const int64_t* __restrict__ desc,
                                           int n_mesh, int64_t total_faces, const T* __restrict__ gp,
                                           const T* __restrict__ gw, int n, const PlaneWave* __restrict__ waves,
                                           int nrhs, int64_t ld, T* __restrict__ rhs) {
    __shared__ T s_p[16], s_w[16];
    if (threadIdx.x < n) { s_p[threadIdx.x] = gp[threadIdx.x]; s_w[threadIdx.x] = gw[threadIdx.x]; }
    __syncthreads();
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * total_faces * nrhs) return;
    const int r = (int)(idx / (3 * total_faces));
    const int64_t fe = idx % (3 * total_faces);
    const int i = seg_find(desc, 6, n_mesh, fe / 3);
    T acc_r, acc_i;
    ref_rhs_entry<T>(verts, faces, areas, normals, s_p, s_w, n, waves[(int64_t)i * nrhs + r], fe / 3, (int)(fe % 3),
                     &acc_r, &acc_i);
    atomic_add_c<T>(rhs + 2 * ((int64_t)fei[fe] * ld + desc[6 * i + 5] + r), acc_r, acc_i);
}

template <typename T>
int launch_mom_ref_rhs_batched(const T* verts, const int32_t* faces, const T* areas, const T* normals,
                               const int32_t* fei, const int64_t* desc, int n_mesh, int64_t total_faces, const T* gp,
                               const T* gw, int n, const PlaneWave* waves, int nrhs, int64_t ld, T* rhs,
                               cudaStream_t s) {
    if (n_mesh <= 0 || total_faces <= 0 || nrhs <= 0) return MB_OK;
    if (n < 1 || n > 16) return set_error(MB_ERR_UNSUPPORTED, "quadrature order must be in [1, 16]");
    const int64_t total = 3 * total_faces * nrhs;
    mom_ref_rhs_batched_kernel<T><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
        verts, faces, areas, normals, fei, desc, n_mesh, total_faces, gp, gw, n, waves, nrhs, ld, rhs);
    return check_launch("mom_ref_rhs_batched");
}
template int launch_mom_ref_rhs_batched<float>(const float*, const int32_t*, const float*, const float*,
                                               const int32_t*, const int64_t*, int, int64_t, const float*,
                                               const float*, int, const PlaneWave*, int, int64_t, float*,
                                               cudaStream_t);
template int launch_mom_ref_rhs_batched<double>(const double*, const int32_t*, const double*, const double*,
                                                const int32_t*, const int64_t*, int, int64_t, const double*,
                                                const double*, int, const PlaneWave*, int, int64_t, double*,
                                                cudaStream_t);

// The reference's hard-coded incidence (mesh_MOM_3d.cu:24-70): k along azimuth 30 deg in
// the xy plane, E along z, H along azimuth -60 deg, eta = 1.
PlaneWave reference_wave(double k) {
    const double az = 30.0 / 180.0 * kPi, hdir = az - 0.5 * kPi;
    return PlaneWave{k * cos(az), k * sin(az), 0.0, 0.0, 0.0, 1.0, cos(hdir), sin(hdir), 0.0};
}

template <typename T>
int launch_mom_ref_rhs(const T* verts, const int32_t* faces, int64_t nf, const T* areas,
                       const T* normals, const T* gp, const T* gw, int n, const PlaneWave* waves_dev,
                       double k_ref, int nrhs, int out_mode, int64_t batch, const int32_t* fei, T* out_r,
                       T* out_i, cudaStream_t stream) {
    if (nf <= 0) return MB_OK;
    if (n < 1 || n > 16) return set_error(MB_ERR_UNSUPPORTED, "quadrature order must be in [1, 16]");
    const int threads = 256;
    const int64_t total = 3 * nf * nrhs;
    const int64_t blocks = (total + threads - 1) / threads;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "too many right-hand sides for one launch");
    mom_ref_rhs_kernel<T><<<(unsigned)blocks, threads, 0, stream>>>(
        verts, faces, areas, normals, gp, gw, n, waves_dev, reference_wave(k_ref), nrhs, nf, out_mode,
        batch, fei, out_r, out_i);
    return check_launch("mom_ref_rhs");
}
template int launch_mom_ref_rhs<float>(const float*, const int32_t*, int64_t, const float*, const float*,
                                       const float*, const float*, int, const PlaneWave*, double, int,
                                       int, int64_t, const int32_t*, float*, float*, cudaStream_t);
template int launch_mom_ref_rhs<double>(const double*, const int32_t*, int64_t, const double*,
                                        const double*, const double*, const double*, int,
                                        const PlaneWave*, double, int, int, int64_t, const int32_t*,
                                        double*, double*, cudaStream_t);

template <typename T>
int launch_mom_interp(const T* verts, const int32_t* faces, const int32_t* fei, const T* areas,
                      const T* ir, const T* ii, int64_t n_edges, int64_t nf, int64_t nv, int64_t batch,
                      int mode, T* jr, T* ji, cudaStream_t stream) {
    if (nf <= 0 || batch <= 0) return MB_OK;
    const int threads = 256;
    const int64_t total = batch * nf;
    const int64_t blocks = (total + threads - 1) / threads;
    mom_interp_kernel<T><<<(unsigned)blocks, threads, 0, stream>>>(verts, faces, fei, areas, ir, ii,
                                                                    n_edges, nf, nv, batch, mode, jr, ji);
    return check_launch("mom_interp");
}
template int launch_mom_interp<float>(const float*, const int32_t*, const int32_t*, const float*,
                                      const float*, const float*, int64_t, int64_t, int64_t, int64_t, int,
                                      float*, float*, cudaStream_t);
template int launch_mom_interp<double>(const double*, const int32_t*, const int32_t*, const double*,
                                       const double*, const double*, int64_t, int64_t, int64_t, int64_t,
                                       int, double*, double*, cudaStream_t);

}  // namespace mb
