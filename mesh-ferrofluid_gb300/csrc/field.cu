// field.cu -- scattered magnetic field radiated by the solved vertex currents.
//
// Reference: the post-solve step of demo/demo_Helmholtz_MOM_3d.py:246-257,
//   H(p) = -sum_v A_v ( J_v x (-gradG_y(k, p, v)) )
// with gradG_y / G of src/utils/functions.py:807-868 (pos_k = False), which evaluate to
//   gradG_y = e^{+jkR} (1 + jkR) / (4 pi R^2) * (p - v)/R,   zero where R < 1e-6.
// (The +jkR phase is what those helpers compute -- G is called with the already negated
// wavenumber -- and is reproduced as is.)
//
// A dense P x V sum: each thread owns one observation point (two in the float path, one per
// lane of packed f32x2 instructions) and accumulates the six components of H; 256 vertices
// at a time (position and A_v J_v, 9 values) are staged in shared memory so each vertex is
// read once per block.  Per interaction: ~40 FP32 ops and 3 SFU ops (rsqrt, sin, cos).
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "packed.cuh"

namespace mb {

constexpr int kFieldThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kFieldThreads) radiate_h_kernel(const T* __restrict__ points, int64_t np,
                                                                  const T* __restrict__ verts,
                                                                  const T* __restrict__ vert_areas,
                                                                  const T* __restrict__ js, int64_t nv, T k,
                                                                  T* __restrict__ h) {
    __shared__ T s_v[kFieldThreads][9];
    const int64_t m = (int64_t)blockIdx.x * kFieldThreads + threadIdx.x;
    V3<T> p = v3<T>(0, 0, 0);
    if (m < np) p = load3(points, m);
    T hr[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    const T k_turn = k * T(kInv2Pi);
    const T eps2 = T(1e-12);  // R < 1e-6 contributes nothing (functions.py:832-834, :860-862)
    for (int64_t base = 0; base < nv; base += kFieldThreads) {
        const int64_t v = base + threadIdx.x;
        if (v < nv) {
            const T a = vert_areas[v];
            s_v[threadIdx.x][0] = verts[3 * v];
            s_v[threadIdx.x][1] = verts[3 * v + 1];
            s_v[threadIdx.x][2] = verts[3 * v + 2];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                s_v[threadIdx.x][3 + c] = a * js[2 * (3 * v + c)];
                s_v[threadIdx.x][6 + c] = a * js[2 * (3 * v + c) + 1];
            }
        }
        __syncthreads();
        const int cnt = (int)((nv - base) < kFieldThreads ? (nv - base) : kFieldThreads);
        if (m < np) {
            for (int t = 0; t < cnt; ++t) {
                const T* q = s_v[t];
                const T dx = p.x - q[0], dy = p.y - q[1], dz = p.z - q[2];
                const T r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < eps2) continue;
                const T rinv = rsqrt_t(r2);
                const T R = r2 * rinv;
                T sn, cs;
                sincos_turns(k_turn * R, &sn, &cs);  // e^{+jkR} = cs + j sn
                const T kR = k * R;
                const T s = rinv * rinv * rinv * T(kInv4Pi);
                const T fr = (cs - kR * sn) * s;  // (1 + jkR) e^{+jkR} / (4 pi R^3)
                const T fi = (sn + kR * cs) * s;
                // (A J) x d, real and imaginary parts
                const T crx = q[4] * dz - q[5] * dy, cry = q[5] * dx - q[3] * dz, crz = q[3] * dy - q[4] * dx;
                const T cix = q[7] * dz - q[8] * dy, ciy = q[8] * dx - q[6] * dz, ciz = q[6] * dy - q[7] * dx;
                hr[0] += fr * crx - fi * cix;
                hr[1] += fr * cry - fi * ciy;
                hr[2] += fr * crz - fi * ciz;
                hi[0] += fr * cix + fi * crx;
                hi[1] += fr * ciy + fi * cry;
                hi[2] += fr * ciz + fi * crz;
            }
        }
        __syncthreads();
    }
    if (m < np) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            h[2 * (3 * m + c)] = hr[c];
            h[2 * (3 * m + c) + 1] = hi[c];
        }
    }
}

// float path: each thread owns two observation points, both lanes of every packed f32x2
// instruction (the staged vertex broadcast to the pair); kR goes to the SFU sine / cosine
// directly (for the tens of radians of observation distances its phase error stays at a
// few 1e-6, inside the float32 parity tolerance); pairs closer than 1e-6 get a zero weight
// instead of a branch.
__global__ void __launch_bounds__(kFieldThreads) radiate_h_f32x2_kernel(const float* __restrict__ points, int64_t np,
                                                                        const float* __restrict__ verts,
                                                                        const float* __restrict__ vert_areas,
                                                                        const float* __restrict__ js, int64_t nv,
                                                                        float k, float* __restrict__ h) {
    __shared__ float s_v[kFieldThreads][9];
    const int64_t m0 = 2 * ((int64_t)blockIdx.x * kFieldThreads + threadIdx.x);
    float2 px = bc(0.f), py = bc(0.f), pz = bc(0.f);
    if (m0 < np) {
        px.x = points[3 * m0];
        py.x = points[3 * m0 + 1];
        pz.x = points[3 * m0 + 2];
    }
    if (m0 + 1 < np) {
        px.y = points[3 * m0 + 3];
        py.y = points[3 * m0 + 4];
        pz.y = points[3 * m0 + 5];
    }
    float2 hr0 = bc(0.f), hr1 = bc(0.f), hr2 = bc(0.f), hi0 = bc(0.f), hi1 = bc(0.f), hi2 = bc(0.f);
    const float2 K = bc(k), I4PI = bc(float(kInv4Pi));
    for (int64_t base = 0; base < nv; base += kFieldThreads) {
        const int64_t v = base + threadIdx.x;
        if (v < nv) {
            const float a = vert_areas[v];
            s_v[threadIdx.x][0] = verts[3 * v];
            s_v[threadIdx.x][1] = verts[3 * v + 1];
            s_v[threadIdx.x][2] = verts[3 * v + 2];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                s_v[threadIdx.x][3 + c] = a * js[2 * (3 * v + c)];
                s_v[threadIdx.x][6 + c] = a * js[2 * (3 * v + c) + 1];
            }
        }
        __syncthreads();
        const int cnt = (int)((nv - base) < kFieldThreads ? (nv - base) : kFieldThreads);
        if (m0 < np) {
#pragma unroll 2
            for (int t = 0; t < cnt; ++t) {
                const float* q = s_v[t];
                const float2 dx = sub2(px, bc(q[0])), dy = sub2(py, bc(q[1])), dz = sub2(pz, bc(q[2]));
                const float2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
                float2 rinv;  // R < 1e-6 contributes nothing (functions.py:832-834, :860-862)
                rinv.x = r2.x < 1e-12f ? 0.f : rsqrtf(r2.x);
                rinv.y = r2.y < 1e-12f ? 0.f : rsqrtf(r2.y);
                const float2 kR = mul2(K, mul2(r2, rinv));
                float2 sn, cs;
                __sincosf(kR.x, &sn.x, &cs.x);
                __sincosf(kR.y, &sn.y, &cs.y);
                const float2 sc = mul2(mul2(rinv, rinv), mul2(rinv, I4PI));
                const float2 fr = mul2(sub2(cs, mul2(kR, sn)), sc);  // (1 + jkR) e^{+jkR} / (4 pi R^3)
                const float2 fi = mul2(fma2(kR, cs, sn), sc);
                const float2 q3 = bc(q[3]), q4 = bc(q[4]), q5 = bc(q[5]), q6 = bc(q[6]), q7 = bc(q[7]), q8 = bc(q[8]);
                // (A J) x d, real and imaginary parts
                const float2 crx = sub2(mul2(q4, dz), mul2(q5, dy)), cry = sub2(mul2(q5, dx), mul2(q3, dz)),
                             crz = sub2(mul2(q3, dy), mul2(q4, dx));
                const float2 cix = sub2(mul2(q7, dz), mul2(q8, dy)), ciy = sub2(mul2(q8, dx), mul2(q6, dz)),
                             ciz = sub2(mul2(q6, dy), mul2(q7, dx));
                hr0 = sub2(fma2(fr, crx, hr0), mul2(fi, cix));
                hr1 = sub2(fma2(fr, cry, hr1), mul2(fi, ciy));
                hr2 = sub2(fma2(fr, crz, hr2), mul2(fi, ciz));
                hi0 = fma2(fi, crx, fma2(fr, cix, hi0));
                hi1 = fma2(fi, cry, fma2(fr, ciy, hi1));
                hi2 = fma2(fi, crz, fma2(fr, ciz, hi2));
            }
        }
        __syncthreads();
    }
    const float2 hr[3] = {hr0, hr1, hr2}, hi[3] = {hi0, hi1, hi2};
    if (m0 < np) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            h[2 * (3 * m0 + c)] = hr[c].x;
            h[2 * (3 * m0 + c) + 1] = hi[c].x;
        }
    }
    if (m0 + 1 < np) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            h[2 * (3 * (m0 + 1) + c)] = hr[c].y;
            h[2 * (3 * (m0 + 1) + c) + 1] = hi[c].y;
        }
    }
}

template <typename T>
int launch_radiate_h(const T* points, int64_t np, const T* verts, const T* vert_areas, const T* js, int64_t nv,
                     double k, T* h, cudaStream_t stream) {
    if (np <= 0) return MB_OK;
    if constexpr (sizeof(T) == 4) {
        const int64_t blocks2 = (np + 2 * kFieldThreads - 1) / (2 * kFieldThreads);
        if (blocks2 > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "too many observation points for one launch");
        radiate_h_f32x2_kernel<<<(unsigned)blocks2, kFieldThreads, 0, stream>>>(points, np, verts, vert_areas, js,
                                                                               nv, (float)k, h);
        return check_launch("radiate_h");
    }
    const int64_t blocks = (np + kFieldThreads - 1) / kFieldThreads;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "too many observation points for one launch");
    radiate_h_kernel<T><<<(unsigned)blocks, kFieldThreads, 0, stream>>>(points, np, verts, vert_areas, js, nv,
                                                                        (T)k, h);
    return check_launch("radiate_h");
}
template int launch_radiate_h<float>(const float*, int64_t, const float*, const float*, const float*, int64_t,
                                     double, float*, cudaStream_t);
template int launch_radiate_h<double>(const double*, int64_t, const double*, const double*, const double*,
                                      int64_t, double, double*, cudaStream_t);

}  // namespace mb
