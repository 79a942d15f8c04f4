// laplace.cu -- Galerkin single/double-layer panel integrals for the 3D Laplace (and
// Helmholtz-BEM) boundary integral operators, with the reference's quadrature.
//
// Reference: double_integration_on_panels_3d (src/mesh_BEM/utils/integrations_3d.py:252-452).
// For every ordered face pair (fy, fx) -- fy the "y" (first) panel, fx the "x" panel -- it
// sums, over the 4-D rule of the pair's relation (separate / shared vertex / shared edge /
// same face, sub-domain maps of get_rands_and_jacobian_3d :18-249),
//     f(x, y) * 4 A_fy A_fx * phi_a(y) * phi_b(x) * w * jac
// with f = 1/(4 pi R) (single layer, BEM_utils.py:72-104) or grad_y G . n_fy (double layer,
// BEM_utils.py:141-172), phi the P1 shape functions (1-r1, r1-r2, r2) or 1 (P0).
//
// The host flattens the sub-domain maps into one table of rows (r1x, r2x, r1y, r2y, w*jac)
// with per-relation segments, computed in the caller's dtype exactly like the reference; the
// kernel walks the segment of each pair's relation.  One thread per face pair, 128 pairs
// (one fy row segment) per block; the nine results of each thread go through shared memory
// so the [F, F, nphi, nphi] output is written with coalesced 16-byte stores.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "packed.cuh"

namespace mb {

constexpr int kLapThreads = 128;

template <typename T>
__device__ __forceinline__ int relation_of(const int32_t* faces, int64_t i, int64_t j) {
    const int32_t a0 = __ldg(faces + 3 * i), a1 = __ldg(faces + 3 * i + 1), a2 = __ldg(faces + 3 * i + 2);
    const int32_t b0 = __ldg(faces + 3 * j), b1 = __ldg(faces + 3 * j + 1), b2 = __ldg(faces + 3 * j + 2);
    const int cnt = (a0 == b0) + (a0 == b1) + (a0 == b2) + (a1 == b0) + (a1 == b1) + (a1 == b2) +
                    (a2 == b0) + (a2 == b1) + (a2 == b2);
    return cnt <= 3 ? cnt : 0;
}

// KIND 0: Laplace (real).  KIND 1: Helmholtz e^{+jkR} (BEM_utils.py:95-102, :161-170).
// LAYER 1: single, 2: double.
template <typename T, int NPHI, int KIND, int LAYER>
__global__ void __launch_bounds__(kLapThreads) laplace_panels_kernel(
    const T* __restrict__ verts, const int32_t* __restrict__ faces, const T* __restrict__ areas,
    const T* __restrict__ normals, const T* __restrict__ tab, int4 seg_lo, int seg_end,
    const uint8_t* __restrict__ rel, int64_t nf, int64_t row_begin, int64_t col_blocks, T k,
    T* __restrict__ out_r, T* __restrict__ out_i) {
    constexpr int NN = NPHI * NPHI;
    __shared__ __align__(16) T s_out[KIND == 1 ? 2 : 1][kLapThreads * NN];
    const int64_t row_local = (int64_t)blockIdx.x / col_blocks;
    const int64_t fy = row_begin + row_local;
    const int64_t col0 = ((int64_t)blockIdx.x % col_blocks) * kLapThreads;
    const int64_t fx = col0 + threadIdx.x;
    T accr[NN], acci[NN];
#pragma unroll
    for (int c = 0; c < NN; ++c) { accr[c] = 0; acci[c] = 0; }
    if (fx < nf) {
        const int r = rel ? (int)rel[fy * nf + fx] : relation_of<T>(faces, fy, fx);
        const int beg = r == 0 ? seg_lo.x : r == 1 ? seg_lo.y : r == 2 ? seg_lo.z : seg_lo.w;
        const int end = r == 0 ? seg_lo.y : r == 1 ? seg_lo.z : r == 2 ? seg_lo.w : seg_end;
        const V3<T> o = load3(verts, __ldg(faces + 3 * fy));
        const V3<T> Y1 = load3(verts, __ldg(faces + 3 * fy + 1)) - o;
        const V3<T> Y2 = load3(verts, __ldg(faces + 3 * fy + 2)) - o;
        const V3<T> X0 = load3(verts, __ldg(faces + 3 * fx)) - o;
        const V3<T> X1 = load3(verts, __ldg(faces + 3 * fx + 1)) - o;
        const V3<T> X2 = load3(verts, __ldg(faces + 3 * fx + 2)) - o;
        const V3<T> ny = load3(normals, fy);
        for (int t = beg; t < end; ++t) {
            const T r1x = __ldg(tab + 5 * t), r2x = __ldg(tab + 5 * t + 1);
            const T r1y = __ldg(tab + 5 * t + 2), r2y = __ldg(tab + 5 * t + 3);
            const T wj = __ldg(tab + 5 * t + 4);
            const V3<T> x = (T(1) - r1x) * X0 + (r1x - r2x) * X1 + r2x * X2;
            const V3<T> y = (r1y - r2y) * Y1 + r2y * Y2;  // Y0 = 0 after the shift
            const V3<T> d = x - y;
            const T r2d = dot(d, d);
            const T rinv = rsqrt_t(r2d);
            T fr, fi = 0;
            if constexpr (LAYER == 1) {
                fr = rinv;
            } else {
                fr = dot(d, ny) * rinv * rinv * rinv;
            }
            if constexpr (KIND == 1) {
                const T R = r2d * rinv;
                T sn, cs;
                sincos_turns(k * R * T(kInv2Pi), &sn, &cs);
                if constexpr (LAYER == 1) {
                    fi = fr * sn;
                    fr = fr * cs;
                } else {
                    const T kR = k * R;
                    fi = fr * (sn - kR * cs);
                    fr = fr * (cs + kR * sn);
                }
            }
            fr *= wj;
            fi *= wj;
            T py[3], px[3];
            if constexpr (NPHI == 3) {
                py[0] = T(1) - r1y; py[1] = r1y - r2y; py[2] = r2y;
                px[0] = T(1) - r1x; px[1] = r1x - r2x; px[2] = r2x;
            } else {
                py[0] = T(1); px[0] = T(1);
            }
#pragma unroll
            for (int a = 0; a < NPHI; ++a) {
                const T ta = fr * py[a];
                const T tb = fi * py[a];
#pragma unroll
                for (int b = 0; b < NPHI; ++b) {
                    accr[a * NPHI + b] += ta * px[b];
                    if constexpr (KIND == 1) acci[a * NPHI + b] += tb * px[b];
                }
            }
        }
        const T scale = T(4) * __ldg(areas + fy) * __ldg(areas + fx) * T(kInv4Pi);
#pragma unroll
        for (int c = 0; c < NN; ++c) {
            accr[c] *= scale;
            acci[c] *= scale;
        }
    }
#pragma unroll
    for (int c = 0; c < NN; ++c) {
        s_out[0][threadIdx.x * NN + c] = accr[c];
        if constexpr (KIND == 1) s_out[KIND == 1 ? 1 : 0][threadIdx.x * NN + c] = acci[c];
    }
    __syncthreads();
    const int64_t valid = (nf - col0) < kLapThreads ? (nf - col0) : kLapThreads;
    const int64_t base = (row_local * nf + col0) * NN;
    const int64_t n_out = valid * NN;
    for (int64_t c = threadIdx.x; c < n_out; c += kLapThreads) {
        out_r[base + c] = s_out[0][c];
        if constexpr (KIND == 1) out_i[base + c] = s_out[KIND == 1 ? 1 : 0][c];
    }
}

// ---------------------------------------------------------------------------------------
// Tiled form for the separated pairs.  The reference's separated-pair rule is a tensor
// product (get_rands_and_jacobian_3d, integrations_3d.py:18-60): the x point of rule row
// g = s Q + t depends on t only, the y point on s only.  A block takes kLapTileRows
// consecutive y faces x 128 x faces; the y points of its rows and the rule weights times the
// y shape functions, W[t][s][a] = w_g phi_a(y_s), sit in shared memory, each thread builds the
// Q x points of its x face once for all rows, and per row sums
//     out[a][b] = sum_t phi_b(x_t) sum_s f(x_t, y_s) W[t][s][a]
// (the same terms as the flattened table, summed in another order).  Every pair gets the
// separated rule here; laplace_near_rows_kernel then overwrites the pairs that share a vertex
// (no divergent per-pair loop inside a warp of separated pairs).  Coordinates are taken
// relative to the first vertex of the block's first y face.
// ---------------------------------------------------------------------------------------
constexpr int kLapTileRows = 16;

// Bulk (TMA) store of a staged output row: shared -> global, 16-byte aligned addresses and a
// size that is a multiple of 16 bytes.  The writers fence their shared-memory stores to the
// async proxy before the barrier after which one thread issues the copy.
__device__ __forceinline__ void lap_fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void lap_bulk_store(void* gdst, const void* ssrc, unsigned bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(ssrc);
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(s), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// the committed bulk stores have finished reading shared memory
__device__ __forceinline__ void lap_bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// the committed bulk stores are complete
__device__ __forceinline__ void lap_bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// The per-pair loop of laplace_panels_kernel over the rows beg, beg + step, ... < end of a
// relation segment, added into acc.
template <typename T, int NPHI, int KIND, int LAYER>
__device__ __forceinline__ void panel_pair_loop(const T* __restrict__ verts, const int32_t* __restrict__ faces,
                                                const T* __restrict__ normals, const T* __restrict__ tab, int beg,
                                                int end, int step, int64_t fy, int64_t fx, T k, T* accr,
                                                T* acci) {
    const V3<T> o = load3(verts, __ldg(faces + 3 * fy));
    const V3<T> Y1 = load3(verts, __ldg(faces + 3 * fy + 1)) - o;
    const V3<T> Y2 = load3(verts, __ldg(faces + 3 * fy + 2)) - o;
    const V3<T> X0 = load3(verts, __ldg(faces + 3 * fx)) - o;
    const V3<T> X1 = load3(verts, __ldg(faces + 3 * fx + 1)) - o;
    const V3<T> X2 = load3(verts, __ldg(faces + 3 * fx + 2)) - o;
    const V3<T> ny = load3(normals, fy);
    for (int t = beg; t < end; t += step) {
        const T r1x = __ldg(tab + 5 * t), r2x = __ldg(tab + 5 * t + 1);
        const T r1y = __ldg(tab + 5 * t + 2), r2y = __ldg(tab + 5 * t + 3);
        const T wj = __ldg(tab + 5 * t + 4);
        const V3<T> x = (T(1) - r1x) * X0 + (r1x - r2x) * X1 + r2x * X2;
        const V3<T> y = (r1y - r2y) * Y1 + r2y * Y2;
        const V3<T> d = x - y;
        const T r2d = dot(d, d);
        const T rinv = rsqrt_t(r2d);
        T fr, fi = 0;
        if constexpr (LAYER == 1) {
            fr = rinv;
        } else {
            fr = dot(d, ny) * rinv * rinv * rinv;
        }
        if constexpr (KIND == 1) {
            const T R = r2d * rinv;
            T sn, cs;
            sincos_turns(k * R * T(kInv2Pi), &sn, &cs);
            if constexpr (LAYER == 1) {
                fi = fr * sn;
                fr = fr * cs;
            } else {
                const T kR = k * R;
                fi = fr * (sn - kR * cs);
                fr = fr * (cs + kR * sn);
            }
        }
        fr *= wj;
        fi *= wj;
        T py[3], px[3];
        if constexpr (NPHI == 3) {
            py[0] = T(1) - r1y; py[1] = r1y - r2y; py[2] = r2y;
            px[0] = T(1) - r1x; px[1] = r1x - r2x; px[2] = r2x;
        } else {
            py[0] = T(1); px[0] = T(1);
        }
#pragma unroll
        for (int a = 0; a < NPHI; ++a) {
#pragma unroll
            for (int b = 0; b < NPHI; ++b) {
                accr[a * NPHI + b] += fr * py[a] * px[b];
                if constexpr (KIND == 1) acci[a * NPHI + b] += fi * py[a] * px[b];
            }
        }
    }
}

template <typename T, int Q, int NPHI, int KIND, int LAYER>
__global__ void __launch_bounds__(kLapThreads) laplace_panels_tiled_kernel(
    const T* __restrict__ verts, const int32_t* __restrict__ faces, const T* __restrict__ areas,
    const T* __restrict__ normals, const T* __restrict__ tab, int4 seg_lo, int64_t nf, int64_t row_begin,
    int64_t row_end, int64_t col_blocks, T k, T* __restrict__ out_r, T* __restrict__ out_i) {
    constexpr int NN = NPHI * NPHI;
    constexpr int NC = KIND == 1 ? 2 : 1;
    __shared__ T s_w[Q][Q][NPHI];          // W[t][s][a]
    __shared__ T s_rx[Q][2];               // (r1x, r2x) of x point t
    __shared__ T s_px[Q][NPHI];            // phi_b(x_t)
    __shared__ T s_y[kLapTileRows][Q][3];  // y points of the tile's rows
    __shared__ T s_ny[kLapTileRows][3];
    __shared__ T s_ay[kLapTileRows];
    __shared__ __align__(16) T s_out[2][NC][kLapThreads * NN];  // double-buffered row staging
    const int tid = threadIdx.x;
    const int64_t col_block = (int64_t)blockIdx.x % col_blocks;
    const int64_t fy0 = row_begin + ((int64_t)blockIdx.x / col_blocks) * kLapTileRows;
    const int rows = (int)((row_end - fy0) < kLapTileRows ? (row_end - fy0) : kLapTileRows);
    const int64_t col0 = col_block * kLapThreads;
    const int64_t fx = col0 + tid;
    const T* t0 = tab + 5 * seg_lo.x;  // relation-0 rows, g = s Q + t
    for (int i = tid; i < Q * Q; i += kLapThreads) {
        const int s = i / Q, t = i - s * Q;
        const T r1y = __ldg(t0 + 5 * i + 2), r2y = __ldg(t0 + 5 * i + 3), w = __ldg(t0 + 5 * i + 4);
        if constexpr (NPHI == 3) {
            s_w[t][s][0] = w * (T(1) - r1y);
            s_w[t][s][1] = w * (r1y - r2y);
            s_w[t][s][2] = w * r2y;
        } else {
            s_w[t][s][0] = w;
        }
        if (s == 0) {
            const T r1x = __ldg(t0 + 5 * i), r2x = __ldg(t0 + 5 * i + 1);
            s_rx[t][0] = r1x;
            s_rx[t][1] = r2x;
            if constexpr (NPHI == 3) {
                s_px[t][0] = T(1) - r1x;
                s_px[t][1] = r1x - r2x;
                s_px[t][2] = r2x;
            } else {
                s_px[t][0] = T(1);
            }
        }
    }
    const V3<T> o = load3(verts, __ldg(faces + 3 * fy0));
    for (int i = tid; i < rows * Q; i += kLapThreads) {
        const int r = i / Q, sq = i - r * Q;
        const int64_t fy = fy0 + r;
        const T r1y = __ldg(t0 + 5 * (sq * Q) + 2), r2y = __ldg(t0 + 5 * (sq * Q) + 3);
        const V3<T> Y0 = load3(verts, __ldg(faces + 3 * fy)) - o;
        const V3<T> Y1 = load3(verts, __ldg(faces + 3 * fy + 1)) - o;
        const V3<T> Y2 = load3(verts, __ldg(faces + 3 * fy + 2)) - o;
        const V3<T> y = (T(1) - r1y) * Y0 + (r1y - r2y) * Y1 + r2y * Y2;
        s_y[r][sq][0] = y.x;
        s_y[r][sq][1] = y.y;
        s_y[r][sq][2] = y.z;
    }
    for (int r = tid; r < rows; r += kLapThreads) {
        const V3<T> n = load3(normals, fy0 + r);
        s_ny[r][0] = n.x;
        s_ny[r][1] = n.y;
        s_ny[r][2] = n.z;
        s_ay[r] = __ldg(areas + fy0 + r);
    }
    __syncthreads();
    T xp[Q][3];
    T ax = 0;
    if (fx < nf) {
        const V3<T> X0 = load3(verts, __ldg(faces + 3 * fx)) - o;
        const V3<T> X1 = load3(verts, __ldg(faces + 3 * fx + 1)) - o;
        const V3<T> X2 = load3(verts, __ldg(faces + 3 * fx + 2)) - o;
#pragma unroll
        for (int t = 0; t < Q; ++t) {
            const T r1x = s_rx[t][0], r2x = s_rx[t][1];
            const V3<T> x = (T(1) - r1x) * X0 + (r1x - r2x) * X1 + r2x * X2;
            xp[t][0] = x.x;
            xp[t][1] = x.y;
            xp[t][2] = x.z;
        }
        ax = __ldg(areas + fx);
    }
    // small rules keep W and phi(x_t) in registers (no shared-memory load per evaluation)
    constexpr bool kRegW = Q <= 4;
    T wreg[kRegW ? Q : 1][kRegW ? Q : 1][NPHI], preg[kRegW ? Q : 1][NPHI];
    if constexpr (kRegW) {
#pragma unroll
        for (int t = 0; t < Q; ++t) {
#pragma unroll
            for (int a = 0; a < NPHI; ++a) {
                preg[t][a] = s_px[t][a];
#pragma unroll
                for (int sq = 0; sq < Q; ++sq) wreg[t][sq][a] = s_w[t][sq][a];
            }
        }
    }
    const int64_t valid = (nf - col0) < kLapThreads ? (nf - col0) : kLapThreads;
#pragma unroll 1
    for (int r = 0; r < rows; ++r) {
        const int64_t fy = fy0 + r;
        T accr[NN], acci[NN];
#pragma unroll
        for (int c = 0; c < NN; ++c) { accr[c] = 0; acci[c] = 0; }
        if (fx < nf) {
            {
                const T nyx = s_ny[r][0], nyy = s_ny[r][1], nyz = s_ny[r][2];
                T yr[Q][3];
#pragma unroll
                for (int sq = 0; sq < Q; ++sq) {
                    yr[sq][0] = s_y[r][sq][0];
                    yr[sq][1] = s_y[r][sq][1];
                    yr[sq][2] = s_y[r][sq][2];
                }
#pragma unroll
                for (int t = 0; t < Q; ++t) {
                    T ur[NPHI], ui[NPHI];
#pragma unroll
                    for (int a = 0; a < NPHI; ++a) { ur[a] = 0; ui[a] = 0; }
#pragma unroll
                    for (int sq = 0; sq < Q; ++sq) {
                        const T dx = xp[t][0] - yr[sq][0], dy = xp[t][1] - yr[sq][1], dz = xp[t][2] - yr[sq][2];
                        const T r2d = dx * dx + dy * dy + dz * dz;
                        const T rinv = rsqrt_t(r2d);
                        T fr, fi = 0;
                        if constexpr (LAYER == 1) {
                            fr = rinv;
                        } else {
                            fr = (dx * nyx + dy * nyy + dz * nyz) * rinv * rinv * rinv;
                        }
                        if constexpr (KIND == 1) {
                            const T R = r2d * rinv;
                            T sn, cs;
                            sincos_turns(k * R * T(kInv2Pi), &sn, &cs);
                            if constexpr (LAYER == 1) {
                                fi = fr * sn;
                                fr = fr * cs;
                            } else {
                                const T kR = k * R;
                                fi = fr * (sn - kR * cs);
                                fr = fr * (cs + kR * sn);
                            }
                        }
#pragma unroll
                        for (int a = 0; a < NPHI; ++a) {
                            const T wv = kRegW ? wreg[kRegW ? t : 0][kRegW ? sq : 0][a] : s_w[t][sq][a];
                            ur[a] += fr * wv;
                            if constexpr (KIND == 1) ui[a] += fi * wv;
                        }
                    }
#pragma unroll
                    for (int a = 0; a < NPHI; ++a) {
#pragma unroll
                        for (int b = 0; b < NPHI; ++b) {
                            const T pv = kRegW ? preg[kRegW ? t : 0][b] : s_px[t][b];
                            accr[a * NPHI + b] += ur[a] * pv;
                            if constexpr (KIND == 1) acci[a * NPHI + b] += ui[a] * pv;
                        }
                    }
                }
            }
            const T scale = T(4) * s_ay[r] * ax * T(kInv4Pi);
#pragma unroll
            for (int c = 0; c < NN; ++c) {
                accr[c] *= scale;
                acci[c] *= scale;
            }
        }
        // row r goes through buffer r & 1: the barrier below also orders the stores of row
        // r - 1 before buffer (r + 1) & 1 is written again
        T(&so)[NC][kLapThreads * NN] = s_out[r & 1];
#pragma unroll
        for (int c = 0; c < NN; ++c) {
            so[0][tid * NN + c] = accr[c];
            if constexpr (KIND == 1) so[NC - 1][tid * NN + c] = acci[c];
        }
        __syncthreads();
        const int64_t base = ((fy - row_begin) * nf + col0) * NN;
        for (int64_t c = tid; c < valid * NN; c += kLapThreads) {
            out_r[base + c] = so[0][c];
            if constexpr (KIND == 1) out_i[base + c] = so[NC - 1][c];
        }
    }
}

// Float Laplace form of the tiled kernel for the 4 x 4 separated rule (gaussQR = 2, the
// reference demo's setting): each thread takes two x faces, col0 + tid and col0 + 128 + tid,
// and evaluates both in packed f32x2 arithmetic (two independent chains per thread, half the
// FP32 instructions).  The per-row operands every thread shares -- the y points, the weights
// W[t][s][a] and phi_b(x_t) -- sit in shared memory as duplicated pairs {v, v}, padded to 16
// bytes per group, so one 16-byte load yields two packed operands.  A row's 256 x 9 results
// are staged in shared memory and written by one bulk store when the output rows are 16-byte
// aligned (per-warp bulk stores of the two 32-face runs measured slower).  Pairs sharing a
// vertex are overwritten afterwards by laplace_near_rows_kernel.
template <int NPHI, int LAYER>
__global__ void __launch_bounds__(kLapThreads) laplace_panels_pair2_kernel(
    const float* __restrict__ verts, const int32_t* __restrict__ faces, const float* __restrict__ areas,
    const float* __restrict__ normals, const float* __restrict__ tab, int4 seg_lo, int64_t nf,
    int64_t row_begin, int64_t row_end, int64_t col_blocks, int bulk, float* __restrict__ out_r) {
    constexpr int Q = 4;
    constexpr int NN = NPHI * NPHI;
    constexpr int W2 = 2 * kLapThreads;  // x faces per block
    constexpr int NP4 = NPHI == 3 ? 4 : 2;  // float2 slots per phi group (3 or 1 used)
    __shared__ __align__(16) float2 s_w2[Q][Q * NPHI];     // {W[t][s][a], same} at [t][s NPHI + a]
    __shared__ __align__(16) float2 s_px2[Q][NP4];         // {phi_b(x_t), same}
    __shared__ __align__(16) float2 s_y2[kLapTileRows][Q * 3];  // {y_s, same} at [r][3 s + coordinate]
    __shared__ __align__(16) float2 s_n2[kLapTileRows][4];     // {n_y, same} (3 used)
    __shared__ float s_rx[Q][2];
    __shared__ float s_ay[kLapTileRows];
    __shared__ __align__(16) float s_out[2][W2 * NN];
    const int tid = threadIdx.x;
    const int64_t col_block = (int64_t)blockIdx.x % col_blocks;
    const int64_t fy0 = row_begin + ((int64_t)blockIdx.x / col_blocks) * kLapTileRows;
    const int rows = (int)((row_end - fy0) < kLapTileRows ? (row_end - fy0) : kLapTileRows);
    const int64_t col0 = col_block * W2;
    const int64_t fxa = col0 + tid, fxb = col0 + kLapThreads + tid;
    const float* t0 = tab + 5 * seg_lo.x;
    for (int i = tid; i < Q * Q; i += kLapThreads) {
        const int sq = i / Q, t = i - sq * Q;
        const float r1y = __ldg(t0 + 5 * i + 2), r2y = __ldg(t0 + 5 * i + 3), w = __ldg(t0 + 5 * i + 4);
        if constexpr (NPHI == 3) {
            s_w2[t][3 * sq] = bc(w * (1.f - r1y));
            s_w2[t][3 * sq + 1] = bc(w * (r1y - r2y));
            s_w2[t][3 * sq + 2] = bc(w * r2y);
        } else {
            s_w2[t][sq] = bc(w);
        }
        if (sq == 0) {
            const float r1x = __ldg(t0 + 5 * i), r2x = __ldg(t0 + 5 * i + 1);
            s_rx[t][0] = r1x;
            s_rx[t][1] = r2x;
            if constexpr (NPHI == 3) {
                s_px2[t][0] = bc(1.f - r1x);
                s_px2[t][1] = bc(r1x - r2x);
                s_px2[t][2] = bc(r2x);
                s_px2[t][3] = bc(0.f);
            } else {
                s_px2[t][0] = bc(1.f);
                s_px2[t][1] = bc(0.f);
            }
        }
    }
    const V3<float> o = load3(verts, __ldg(faces + 3 * fy0));
    for (int i = tid; i < rows * Q; i += kLapThreads) {
        const int r = i / Q, sq = i - r * Q;
        const int64_t fy = fy0 + r;
        const float r1y = __ldg(t0 + 5 * (sq * Q) + 2), r2y = __ldg(t0 + 5 * (sq * Q) + 3);
        const V3<float> Y0 = load3(verts, __ldg(faces + 3 * fy)) - o;
        const V3<float> Y1 = load3(verts, __ldg(faces + 3 * fy + 1)) - o;
        const V3<float> Y2 = load3(verts, __ldg(faces + 3 * fy + 2)) - o;
        const V3<float> y = (1.f - r1y) * Y0 + (r1y - r2y) * Y1 + r2y * Y2;
        s_y2[r][3 * sq] = bc(y.x);
        s_y2[r][3 * sq + 1] = bc(y.y);
        s_y2[r][3 * sq + 2] = bc(y.z);
    }
    for (int r = tid; r < rows; r += kLapThreads) {
        const V3<float> nn = load3(normals, fy0 + r);
        s_n2[r][0] = bc(nn.x);
        s_n2[r][1] = bc(nn.y);
        s_n2[r][2] = bc(nn.z);
        s_n2[r][3] = bc(0.f);
        s_ay[r] = __ldg(areas + fy0 + r);
    }
    __syncthreads();
    // the x points of both faces, lane a = fxa, lane b = fxb (a face past the end repeats fxa)
    float2 xx[Q], xy[Q], xz[Q];
    float2 ax2 = bc(0.f);
    {
        const int64_t fa = fxa < nf ? fxa : 0, fb = fxb < nf ? fxb : fa;
        const V3<float> A0 = load3(verts, __ldg(faces + 3 * fa)) - o, A1 = load3(verts, __ldg(faces + 3 * fa + 1)) - o,
                        A2 = load3(verts, __ldg(faces + 3 * fa + 2)) - o;
        const V3<float> B0 = load3(verts, __ldg(faces + 3 * fb)) - o, B1 = load3(verts, __ldg(faces + 3 * fb + 1)) - o,
                        B2 = load3(verts, __ldg(faces + 3 * fb + 2)) - o;
#pragma unroll
        for (int t = 0; t < Q; ++t) {
            const float r1x = s_rx[t][0], r2x = s_rx[t][1];
            const V3<float> xa = (1.f - r1x) * A0 + (r1x - r2x) * A1 + r2x * A2;
            const V3<float> xb = (1.f - r1x) * B0 + (r1x - r2x) * B1 + r2x * B2;
            xx[t] = make_float2(xa.x, xb.x);
            xy[t] = make_float2(xa.y, xb.y);
            xz[t] = make_float2(xa.z, xb.z);
        }
        ax2 = make_float2(__ldg(areas + fa), __ldg(areas + fb));
    }
    const int64_t valid = (nf - col0) < W2 ? (nf - col0) : W2;
#pragma unroll 1
    for (int r = 0; r < rows; ++r) {
        const int64_t fy = fy0 + r;
        float2 acc[NN];
#pragma unroll
        for (int c = 0; c < NN; ++c) acc[c] = bc(0.f);
        float2 yv[Q * 3];
#pragma unroll
        for (int h = 0; h < Q * 3 / 2; ++h) {
            const float4 p = *reinterpret_cast<const float4*>(&s_y2[r][2 * h]);
            yv[2 * h] = make_float2(p.x, p.y);
            yv[2 * h + 1] = make_float2(p.z, p.w);
        }
        float2 NX = bc(0.f), NY = bc(0.f), NZ = bc(0.f);
        if constexpr (LAYER == 2) {
            const float4 p0 = *reinterpret_cast<const float4*>(&s_n2[r][0]);
            const float4 p1 = *reinterpret_cast<const float4*>(&s_n2[r][2]);
            NX = make_float2(p0.x, p0.y);
            NY = make_float2(p0.z, p0.w);
            NZ = make_float2(p1.x, p1.y);
        }
#pragma unroll
        for (int t = 0; t < Q; ++t) {
            float2 u[NPHI];
#pragma unroll
            for (int a = 0; a < NPHI; ++a) u[a] = bc(0.f);
            float2 wv[Q * NPHI];
#pragma unroll
            for (int h = 0; h < Q * NPHI / 2; ++h) {
                const float4 p = *reinterpret_cast<const float4*>(&s_w2[t][2 * h]);
                wv[2 * h] = make_float2(p.x, p.y);
                wv[2 * h + 1] = make_float2(p.z, p.w);
            }
#pragma unroll
            for (int sq = 0; sq < Q; ++sq) {
                const float2 dx = sub2(xx[t], yv[3 * sq]), dy = sub2(xy[t], yv[3 * sq + 1]),
                             dz = sub2(xz[t], yv[3 * sq + 2]);
                const float2 r2d = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
                float2 ri;
                ri.x = rsqrtf(r2d.x);
                ri.y = rsqrtf(r2d.y);
                float2 fr;
                if constexpr (LAYER == 1) {
                    fr = ri;
                } else {
                    const float2 dn = fma2(dz, NZ, fma2(dy, NY, mul2(dx, NX)));
                    fr = mul2(dn, mul2(ri, mul2(ri, ri)));
                }
#pragma unroll
                for (int a = 0; a < NPHI; ++a) u[a] = fma2(fr, wv[sq * NPHI + a], u[a]);
            }
            float2 pv[NP4];
#pragma unroll
            for (int h = 0; h < NP4 / 2; ++h) {
                const float4 p = *reinterpret_cast<const float4*>(&s_px2[t][2 * h]);
                pv[2 * h] = make_float2(p.x, p.y);
                pv[2 * h + 1] = make_float2(p.z, p.w);
            }
#pragma unroll
            for (int a = 0; a < NPHI; ++a)
#pragma unroll
                for (int b = 0; b < NPHI; ++b) acc[a * NPHI + b] = fma2(u[a], pv[b], acc[a * NPHI + b]);
        }
        float ra[NN], rb[NN];
        const float2 sc = mul2(bc(4.f * s_ay[r] * (float)kInv4Pi), ax2);
#pragma unroll
        for (int c = 0; c < NN; ++c) {
            ra[c] = acc[c].x * sc.x;
            rb[c] = acc[c].y * sc.y;
        }
        // row r goes through buffer r & 1: the barrier below also orders the reads of row
        // r - 1 before buffer (r + 1) & 1 is written again
        float* so = s_out[r & 1];
#pragma unroll
        for (int c = 0; c < NN; ++c) {
            so[tid * NN + c] = ra[c];
            so[(kLapThreads + tid) * NN + c] = rb[c];
        }
        const int64_t base = ((fy - row_begin) * nf + col0) * NN;
        if (bulk) {
            // one bulk store per row; before the barrier thread 0 waits until the store of
            // row r - 1 has read buffer (r + 1) & 1, which row r + 1 writes next
            lap_fence_async_smem();
            if (tid == 0) lap_bulk_wait_read();
            __syncthreads();
            if (tid == 0) lap_bulk_store(out_r + base, so, (unsigned)(valid * NN * sizeof(float)));
        } else {
            __syncthreads();
            for (int64_t c = tid; c < valid * NN; c += kLapThreads) out_r[base + c] = so[c];
        }
    }
    if (bulk && tid == 0) lap_bulk_wait_all();
}

// Pairs that share a vertex (relation 1, 2 or 3), when the caller passes the relation matrix:
// a block per row of the window.  The block scans the row's relation bytes (four per 32-bit
// word when the rows are 4-byte aligned, several loads in flight per thread) and appends
// every nonzero one to a list in shared memory; then groups of 8 lanes take pairs from the
// list (16 pairs at a time -- a typical row has about 13), lanes striding over the rows of
// the relation's table segment, a shuffle sum per entry, and overwrite the pair's entries
// (the tiled kernels wrote the separated rule there).  A row with more than kNearCap such
// pairs is evaluated from the whole row in rounds of 16.  Runs after the tiled kernel on
// the same stream.
constexpr int kNearCap = 256;
constexpr int kNearGroup = 8;

template <typename T, int NPHI, int KIND, int LAYER>
__global__ void __launch_bounds__(kLapThreads) laplace_near_rows_kernel(
    const T* __restrict__ verts, const int32_t* __restrict__ faces, const T* __restrict__ areas,
    const T* __restrict__ normals, const T* __restrict__ tab, int4 seg_lo, int seg_end,
    const uint8_t* __restrict__ rel, int64_t nf, int64_t row_begin, int words, T k, T* __restrict__ out_r,
    T* __restrict__ out_i) {
    constexpr int NN = NPHI * NPHI;
    constexpr int NG = kLapThreads / kNearGroup;  // pairs evaluated at a time
    __shared__ int s_cnt;
    __shared__ int32_t s_fx[kNearCap];
    __shared__ uint8_t s_rl[kNearCap];
    const int64_t fy = row_begin + blockIdx.x;
    const int tid = threadIdx.x, grp = tid / kNearGroup, gl = tid % kNearGroup;
    const uint8_t* rrow = rel + fy * nf;
    const T ay = __ldg(areas + fy);
    // pair (fy, fx) of relation rl by the 8 lanes of this group; active is uniform over the
    // group, every lane of the warp runs the shuffles
    auto pair = [&](bool active, int64_t fx, int rl) {
        T accr[NN], acci[NN];
#pragma unroll
        for (int c = 0; c < NN; ++c) { accr[c] = 0; acci[c] = 0; }
        if (active) {
            const int beg = rl == 1 ? seg_lo.y : rl == 2 ? seg_lo.z : seg_lo.w;
            const int end = rl == 1 ? seg_lo.z : rl == 2 ? seg_lo.w : seg_end;
            panel_pair_loop<T, NPHI, KIND, LAYER>(verts, faces, normals, tab, beg + gl, end, kNearGroup, fy, fx, k,
                                                  accr, acci);
        }
#pragma unroll
        for (int c = 0; c < NN; ++c) {
#pragma unroll
            for (int off = kNearGroup / 2; off > 0; off >>= 1) {
                accr[c] += __shfl_xor_sync(0xffffffffu, accr[c], off);
                if constexpr (KIND == 1) acci[c] += __shfl_xor_sync(0xffffffffu, acci[c], off);
            }
        }
        if (active) {
            const T scale = T(4) * ay * __ldg(areas + fx) * T(kInv4Pi);
            const int64_t o = ((fy - row_begin) * nf + fx) * NN;
#pragma unroll
            for (int c = 0; c < NN; ++c) {
                if (c % kNearGroup == gl) {
                    out_r[o + c] = accr[c] * scale;
                    if constexpr (KIND == 1) out_i[o + c] = acci[c] * scale;
                }
            }
        }
    };
    if (tid == 0) s_cnt = 0;
    __syncthreads();
    auto push = [&](int64_t fx, unsigned q) {
        const int pos = atomicAdd(&s_cnt, 1);
        if (pos < kNearCap) {
            s_fx[pos] = (int32_t)fx;
            s_rl[pos] = (uint8_t)q;
        }
    };
    if (words) {
        const uint32_t* wrow = reinterpret_cast<const uint32_t*>(rrow);
        const int64_t nw = nf >> 2;
        constexpr int U = 4;
        for (int64_t i0 = tid; i0 < nw; i0 += U * kLapThreads) {
            uint32_t w[U];
#pragma unroll
            for (int u = 0; u < U; ++u) w[u] = i0 + u * kLapThreads < nw ? __ldg(wrow + i0 + u * kLapThreads) : 0u;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (w[u] != 0u) {
#pragma unroll
                    for (int b = 0; b < 4; ++b)
                        if ((w[u] >> (8 * b)) & 0xffu) push(4 * (i0 + u * kLapThreads) + b, (w[u] >> (8 * b)) & 0xffu);
                }
            }
        }
    } else {
        for (int64_t fx = tid; fx < nf; fx += kLapThreads) {
            const unsigned q = __ldg(rrow + fx);
            if (q != 0u) push(fx, q);
        }
    }
    __syncthreads();
    const int total = s_cnt;
    if (total <= kNearCap) {
        for (int i0 = 0; i0 < total; i0 += NG) {
            const int i = i0 + grp;
            const bool act = i < total;
            pair(act, act ? s_fx[i] : 0, act ? s_rl[i] : 0);
        }
    } else {
        // more pairs than the list holds: rounds over the whole row, 16 columns at a time (one
        // per group); a pair's value does not depend on who computes it
        for (int64_t c0 = 0; c0 < nf; c0 += NG) {
            const int64_t fx = c0 + grp;
            const unsigned q = fx < nf ? (unsigned)__ldg(rrow + fx) : 0u;
            pair(q != 0u, fx, (int)q);
        }
    }
}

template <typename T>
int launch_laplace_panels(const T* verts, const int32_t* faces, int64_t nf, const T* areas,
                          const T* normals, const T* tab, const int* seg, const uint8_t* rel,
                          int layer, int order, int kind, double k, int64_t row_begin,
                          int64_t row_end, T* out_r, T* out_i, cudaStream_t stream) {
    if (nf <= 0 || row_end <= row_begin) return MB_OK;
    if (layer != 1 && layer != 2)
        return set_error(MB_ERR_UNSUPPORTED, "layer %d not supported (1 single, 2 double)", layer);
    if (order != 0 && order != 1) return set_error(MB_ERR_ARG, "order must be 0 or 1");
    if (kind != 0 && kind != 1) return set_error(MB_ERR_ARG, "kind must be 0 or 1");
    if (kind == 1 && out_i == nullptr) return set_error(MB_ERR_ARG, "Helmholtz kernel needs out_i");
    const int64_t col_blocks = (nf + kLapThreads - 1) / kLapThreads;
    const int64_t blocks = (row_end - row_begin) * col_blocks;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
    const int4 lo = make_int4(seg[0], seg[1], seg[2], seg[3]);
    const int se = seg[4];
    // the tiled kernel when the separated rule is a Q x Q product of a supported size
    int q = 0;
    for (int c = 1; c <= 16; ++c)
        if (c * c == seg[1] - seg[0]) q = c;
    // the tiled kernels when the separated rule is a Q x Q product of a supported size and the
    // relation matrix is given (its nonzero entries are then overwritten by the near kernel)
    if (rel != nullptr && (q == 4 || q == 9 || q == 1)) {
        const int64_t tiles = (row_end - row_begin + kLapTileRows - 1) / kLapTileRows;
        if (tiles * col_blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
        bool packed = false;
        if constexpr (sizeof(T) == 4) {
            if (q == 4 && kind == 0) {  // the packed two-faces-per-thread form
                packed = true;
                const int64_t cb2 = (nf + 2 * kLapThreads - 1) / (2 * kLapThreads);
                // bulk row stores need 16-byte aligned rows of the output: nf % 4 == 0
                const int bulk = (nf % 4 == 0 && reinterpret_cast<uintptr_t>(out_r) % 16 == 0) ? 1 : 0;
                const unsigned nb = (unsigned)(tiles * cb2);
#define MB_LAP2(NP, LY)                                                                                   \
    laplace_panels_pair2_kernel<NP, LY><<<nb, kLapThreads, 0, stream>>>(                                   \
        reinterpret_cast<const float*>(verts), faces, reinterpret_cast<const float*>(areas),                 \
        reinterpret_cast<const float*>(normals), reinterpret_cast<const float*>(tab), lo, nf, row_begin,     \
        row_end, cb2, bulk, reinterpret_cast<float*>(out_r))
                if (order == 1) {
                    if (layer == 1) MB_LAP2(3, 1); else MB_LAP2(3, 2);
                } else {
                    if (layer == 1) MB_LAP2(1, 1); else MB_LAP2(1, 2);
                }
#undef MB_LAP2
            }
        }
        if (!packed) {
            const unsigned tblocks = (unsigned)(tiles * col_blocks);
#define MB_LAPT(QQ, NP, KD, LY)                                                                        \
    laplace_panels_tiled_kernel<T, QQ, NP, KD, LY><<<tblocks, kLapThreads, 0, stream>>>(                \
        verts, faces, areas, normals, tab, lo, nf, row_begin, row_end, col_blocks, (T)k, out_r, out_i)
#define MB_LAPQ(QQ)                                                                                    \
    switch ((order == 1 ? 4 : 0) + kind * 2 + (layer - 1)) {                                           \
        case 0: MB_LAPT(QQ, 1, 0, 1); break;                                                           \
        case 1: MB_LAPT(QQ, 1, 0, 2); break;                                                           \
        case 2: MB_LAPT(QQ, 1, 1, 1); break;                                                           \
        case 3: MB_LAPT(QQ, 1, 1, 2); break;                                                           \
        case 4: MB_LAPT(QQ, 3, 0, 1); break;                                                           \
        case 5: MB_LAPT(QQ, 3, 0, 2); break;                                                           \
        case 6: MB_LAPT(QQ, 3, 1, 1); break;                                                           \
        case 7: MB_LAPT(QQ, 3, 1, 2); break;                                                           \
    }
            if (q == 1) { MB_LAPQ(1) } else if (q == 4) { MB_LAPQ(4) } else { MB_LAPQ(9) }
#undef MB_LAPQ
#undef MB_LAPT
        }
        int rc = check_launch(packed ? "laplace_panels_pair2" : "laplace_panels_tiled");
        if (rc != MB_OK) return rc;
        const int64_t nrows = row_end - row_begin;
        if (nrows > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
        if (nf > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
        // 32-bit scans of the relation rows when every row starts on a 4-byte boundary
        const int words = (nf % 4 == 0 && reinterpret_cast<uintptr_t>(rel) % 4 == 0) ? 1 : 0;
#define MB_LAPN(NP, KD, LY)                                                                            \
    laplace_near_rows_kernel<T, NP, KD, LY><<<(unsigned)nrows, kLapThreads, 0, stream>>>(               \
        verts, faces, areas, normals, tab, lo, se, rel, nf, row_begin, words, (T)k, out_r, out_i)
        switch ((order == 1 ? 4 : 0) + kind * 2 + (layer - 1)) {
            case 0: MB_LAPN(1, 0, 1); break;
            case 1: MB_LAPN(1, 0, 2); break;
            case 2: MB_LAPN(1, 1, 1); break;
            case 3: MB_LAPN(1, 1, 2); break;
            case 4: MB_LAPN(3, 0, 1); break;
            case 5: MB_LAPN(3, 0, 2); break;
            case 6: MB_LAPN(3, 1, 1); break;
            case 7: MB_LAPN(3, 1, 2); break;
        }
#undef MB_LAPN
        return check_launch("laplace_near_rows");
    }
#define MB_LAP(NP, KD, LY)                                                                          \
    laplace_panels_kernel<T, NP, KD, LY><<<(unsigned)blocks, kLapThreads, 0, stream>>>(             \
        verts, faces, areas, normals, tab, lo, se, rel, nf, row_begin, col_blocks, (T)k, out_r, out_i)
    const int sel = (order == 1 ? 4 : 0) + kind * 2 + (layer - 1);
    switch (sel) {
        case 0: MB_LAP(1, 0, 1); break;
        case 1: MB_LAP(1, 0, 2); break;
        case 2: MB_LAP(1, 1, 1); break;
        case 3: MB_LAP(1, 1, 2); break;
        case 4: MB_LAP(3, 0, 1); break;
        case 5: MB_LAP(3, 0, 2); break;
        case 6: MB_LAP(3, 1, 1); break;
        case 7: MB_LAP(3, 1, 2); break;
    }
#undef MB_LAP
    return check_launch("laplace_panels");
}

template int launch_laplace_panels<float>(const float*, const int32_t*, int64_t, const float*,
                                          const float*, const float*, const int*, const uint8_t*, int,
                                          int, int, double, int64_t, int64_t, float*, float*,
                                          cudaStream_t);
template int launch_laplace_panels<double>(const double*, const int32_t*, int64_t, const double*,
                                           const double*, const double*, const int*, const uint8_t*,
                                           int, int, int, double, int64_t, int64_t, double*, double*,
                                           cudaStream_t);

// pack_matrix_tight (src/utils/BEM_utils.py:314-357): packed[faces[fy,a], faces[fx,b]] +=
// M[fy, fx, a, b]; P0 spreads M[fy, fx]/9 over the nine vertex pairs.  packed is [V, V]
// (real) or interleaved complex [V, V] when m_i != nullptr; the caller zeroes it.
template <typename T>
__global__ void pack_tight_kernel(const T* __restrict__ m_r, const T* __restrict__ m_i,
                                  const int32_t* __restrict__ faces, int64_t nf, int64_t nv, int nphi,
                                  T* __restrict__ packed) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nf * nf) return;
    const int64_t fy = idx / nf, fx = idx % nf;
    const int32_t vy[3] = {faces[3 * fy], faces[3 * fy + 1], faces[3 * fy + 2]};
    const int32_t vx[3] = {faces[3 * fx], faces[3 * fx + 1], faces[3 * fx + 2]};
    const int nn = nphi * nphi;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            const int64_t src = idx * nn + (nphi == 3 ? a * 3 + b : 0);
            const T div = nphi == 3 ? T(1) : T(1) / T(9);
            const int64_t dst = (int64_t)vy[a] * nv + vx[b];
            if (m_i == nullptr) {
                atomicAdd(packed + dst, m_r[src] * div);
            } else {
                atomicAdd(packed + 2 * dst, m_r[src] * div);
                atomicAdd(packed + 2 * dst + 1, m_i[src] * div);
            }
        }
}

// Surface curls of the three P1 hat functions of face f (defined with the hypersingular
// operator below).
template <typename T>
__device__ __forceinline__ void face_curls(const T* verts, const int32_t* faces, int64_t f, V3<T> c[3]);

// Real P1 packing by test-face rows: block fy accumulates the three rows faces[fy, a] of
// its panels in shared memory (3 x V values, shared atomics over the ~6 faces that meet at
// a vertex), then adds them to the packed rows with 3 V global reductions -- 6x fewer than
// one global atomic per panel entry.  HS: the panels are the hypersingular ones, built on
// the fly from the P0 single layer m = V0 [F, F] and the faces' surface curls, so the
// [F, F, 3, 3] hypersingular panels are never stored.
constexpr int kPackRowThreads = 256;
constexpr int64_t kPackRowSmemMax = 160 * 1024;

template <typename T, bool HS>
__global__ void __launch_bounds__(kPackRowThreads)
    pack_rows_kernel(const T* __restrict__ m, const T* __restrict__ verts, const int32_t* __restrict__ faces,
                     int64_t nf, int64_t nv, T* __restrict__ packed) {
    extern __shared__ __align__(16) unsigned char pack_smem[];
    T* rows = reinterpret_cast<T*>(pack_smem);
    const int64_t fy = blockIdx.x;
    for (int64_t j = threadIdx.x; j < 3 * nv; j += blockDim.x) rows[j] = T(0);
    V3<T> cy[3];
    if constexpr (HS) face_curls(verts, faces, fy, cy);
    __syncthreads();
    for (int64_t fx = threadIdx.x; fx < nf; fx += blockDim.x) {
        const int32_t vx[3] = {__ldg(faces + 3 * fx), __ldg(faces + 3 * fx + 1), __ldg(faces + 3 * fx + 2)};
        if constexpr (HS) {
            V3<T> cx[3];
            face_curls(verts, faces, fx, cx);
            const T w = m[fy * nf + fx];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) atomicAdd(rows + a * nv + vx[b], dot(cy[a], cx[b]) * w);
        } else {
            const T* src = m + (fy * nf + fx) * 9;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) atomicAdd(rows + a * nv + vx[b], src[3 * a + b]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        T* dst = packed + (int64_t)__ldg(faces + 3 * fy + a) * nv;
        for (int64_t j = threadIdx.x; j < nv; j += blockDim.x) atomicAdd(dst + j, rows[a * nv + j]);
    }
}

template <typename T, bool HS>
int launch_pack_rows(const T* m, const T* verts, const int32_t* faces, int64_t nf, int64_t nv, T* packed,
                     cudaStream_t stream) {
    const int64_t smem = 3 * nv * (int64_t)sizeof(T);
    if (smem > kPackRowSmemMax) return set_error(MB_ERR_SIZE, "too many vertices for the row packing");
    if (nf > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(pack_rows_kernel<T, HS>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return set_error(MB_ERR_CUDA, cudaGetErrorString(e));
    }
    pack_rows_kernel<T, HS><<<(unsigned)nf, kPackRowThreads, (size_t)smem, stream>>>(m, verts, faces, nf, nv,
                                                                                     packed);
    return check_launch("pack_rows");
}

template <typename T>
int launch_pack_tight(const T* m_r, const T* m_i, const int32_t* faces, int64_t nf, int64_t nv,
                      int order, T* packed, cudaStream_t stream) {
    if (nf <= 0) return MB_OK;
    if (m_i == nullptr && order == 1 && 3 * nv * (int64_t)sizeof(T) <= kPackRowSmemMax)
        return launch_pack_rows<T, false>(m_r, nullptr, faces, nf, nv, packed, stream);
    const int threads = 256;
    const int64_t blocks = (nf * nf + threads - 1) / threads;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
    pack_tight_kernel<T><<<(unsigned)blocks, threads, 0, stream>>>(m_r, m_i, faces, nf, nv,
                                                                    order == 1 ? 3 : 1, packed);
    return check_launch("pack_tight");
}
template int launch_pack_tight<float>(const float*, const float*, const int32_t*, int64_t, int64_t, int,
                                      float*, cudaStream_t);
template int launch_pack_tight<double>(const double*, const double*, const int32_t*, int64_t, int64_t,
                                       int, double*, cudaStream_t);

// Hypersingular operator of the Laplace problem, P1 Galerkin, by Maue's integration by parts
// (J.-C. Nedelec 1982; O. Steinbach, Numerical Approximation Methods for Elliptic Boundary
// Value Problems, 2008, Thm 6.17):
//   <D phi_j, phi_i> = int int G(x, y) curl phi_j(y) . curl phi_i(x)  dS_y dS_x,
// and on a flat triangle (p0, p1, p2) with area A the surface curl n x grad phi_a of the P1
// hat function of vertex a is the constant (p_{a+1} - p_{a+2}) / (2 A).  So every face pair
// contributes curl_a(fy) . curl_b(fx) times the P0 single-layer integral V0[fy, fx].
// One thread per face pair; out[fy, fx, a, b] (same layout as the single / double layer).
template <typename T>
__device__ __forceinline__ void face_curls(const T* verts, const int32_t* faces, int64_t f, V3<T> c[3]) {
    const V3<T> p0 = load3(verts, faces[3 * f]), p1 = load3(verts, faces[3 * f + 1]),
                p2 = load3(verts, faces[3 * f + 2]);
    const V3<T> nr = cross(p1 - p0, p2 - p1);
    const T inv2a = T(1) / sqrt_t(dot(nr, nr));  // 1 / (2 A)
    c[0] = inv2a * (p1 - p2);
    c[1] = inv2a * (p2 - p0);
    c[2] = inv2a * (p0 - p1);
}

template <typename T>
__global__ void hypersingular_kernel(const T* __restrict__ verts, const int32_t* __restrict__ faces, int64_t nf,
                                     const T* __restrict__ v0, T* __restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nf * nf) return;
    const int64_t fy = idx / nf, fx = idx % nf;
    V3<T> cy[3], cx[3];
    face_curls(verts, faces, fy, cy);
    face_curls(verts, faces, fx, cx);
    const T w = v0[idx];
    T* o = out + 9 * idx;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) o[3 * a + b] = dot(cy[a], cx[b]) * w;
}

template <typename T>
int launch_hypersingular(const T* verts, const int32_t* faces, int64_t nf, const T* v0, T* out,
                         cudaStream_t stream) {
    if (nf <= 0) return MB_OK;
    const int threads = 256;
    const int64_t blocks = (nf * nf + threads - 1) / threads;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
    hypersingular_kernel<T><<<(unsigned)blocks, threads, 0, stream>>>(verts, faces, nf, v0, out);
    return check_launch("hypersingular");
}
template int launch_hypersingular<float>(const float*, const int32_t*, int64_t, const float*, float*,
                                         cudaStream_t);
template int launch_hypersingular<double>(const double*, const int32_t*, int64_t, const double*, double*,
                                          cudaStream_t);

// Packed P1 hypersingular matrix [V, V] straight from V0 [F, F] (the caller zeroes packed).
template <typename T>
int launch_hypersingular_tight(const T* verts, const int32_t* faces, int64_t nf, int64_t nv, const T* v0,
                               T* packed, cudaStream_t stream) {
    if (nf <= 0) return MB_OK;
    return launch_pack_rows<T, true>(v0, verts, faces, nf, nv, packed, stream);
}
template int launch_hypersingular_tight<float>(const float*, const int32_t*, int64_t, int64_t, const float*,
                                               float*, cudaStream_t);
template int launch_hypersingular_tight<double>(const double*, const int32_t*, int64_t, int64_t, const double*,
                                                double*, cudaStream_t);

// compute_panel_relation (src/utils/mesh_utils.py:700-725): shared-vertex count per pair.
__global__ void panel_relation_kernel(const int32_t* __restrict__ faces, int64_t nf,
                                      uint8_t* __restrict__ rel) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nf * nf) return;
    rel[idx] = (uint8_t)relation_of<float>(faces, idx / nf, idx % nf);
}

int launch_panel_relation(const int32_t* faces, int64_t nf, uint8_t* rel, cudaStream_t stream) {
    if (nf <= 0) return MB_OK;
    const int threads = 256;
    const int64_t blocks = (nf * nf + threads - 1) / threads;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for one launch");
    panel_relation_kernel<<<(unsigned)blocks, threads, 0, stream>>>(faces, nf, rel);
    return check_launch("panel_relation");
}

}  // namespace mb
