// spai.cu -- sparse approximate inverse (SAI) of the RWG impedance matrix, the near-field
// right preconditioner of the iterative solve (no counterpart in the reference, which
// factors Z densely: mesh_BEM_solver_3d.py:174).
//
// Column j of M (one RWG edge) minimises || Z[I_j, J_j] m - e_j || where
//   J_j = the edges of the faces that share a vertex with a face of edge j (the near-pair
//         list's rows of those faces: ~29 edges on a regular triangulation), and
//   I_j = the edges of the faces that share a vertex with a face of J_j (~70 edges),
// so Z M ~ I on the near field, where the EFIE's ill-conditioning (the hypersingular
// divergence term, growing like 1/(kh)^2) lives.  Far rows of Z[:, J_j] are left out of the
// fit (they are small and smooth).  On a 7680-unknown sphere at ka = 10 this cuts GMRES(50)
// steps to a 1e-4 error in J by about 13x.
//
// One 128-thread block per edge:
//   1. patterns: the face sets from the sorted near-pair list (binary search per face),
//      block-wide bitonic sort + unique in shared memory; sets above the caps keep the
//      edges nearest to edge j (midpoint distance, ties by edge id), and set a status bit;
//   2. the block A = Z[I, J] (<= 128 x 48 complex64) gathered into shared memory, stored
//      column-major with a padded column length (conflict-free lane-per-row access);
//   3. complex Householder QR in FP32 (one warp forms each reflector, four warps apply it
//      to the remaining columns and the right-hand side), back substitution by one warp;
//   4. the column written as (local edge id, value) pairs, width MB_SPAI_WIDTH.
// A second kernel turns the columns into rows (M[i, j] looked up in column j; the patterns
// are symmetric, i in J_j <=> j in J_i, unless a cap cut them), so that applying M is a
// plain gather: y_i = sum_q M[i, q] v[col(i, q)].
//
// FP32 is enough here: M only has to be a good preconditioner; the solve's accuracy comes
// from the FP64 refinement residual.  Several meshes are handled in one launch through a
// descriptor [n_mesh, 6] int64 = (first face, faces, first edge, edges, offset of Z_i in
// complex entries, row pitch of Z_i).
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace mb {

constexpr int kSpaiWidth = MB_SPAI_WIDTH;  // max |J_j|
constexpr int kSpaiRows = 128;             // max |I_j|
constexpr int kSpaiRowsP = kSpaiRows + 1;  // padded column length of A in shared memory
constexpr int kSpaiThreads = 128;
constexpr int kSpaiS1Cap = 128;            // faces around the edge's faces
constexpr int kSpaiCand = 2048;            // candidate buffer (sort) length

// status bits
constexpr int kSpaiTruncated = 1;  // a pattern above its cap was cut to the nearest edges
constexpr int kSpaiRankDef = 2;    // a least-squares block without full column rank
constexpr int kSpaiBadMap = 4;     // an edge id out of range, or an edge with 0 or > 2 faces

struct SpaiDesc {
    int64_t face0, nf, edge0, ne, zoff, pitch;
};

__device__ __forceinline__ SpaiDesc load_desc(const int64_t* d, int i) {
    return SpaiDesc{d[6 * i], d[6 * i + 1], d[6 * i + 2], d[6 * i + 3], d[6 * i + 4], d[6 * i + 5]};
}

// last mesh whose column `col` (0 = first face, 2 = first edge) is <= v
__device__ __forceinline__ int find_mesh(const int64_t* d, int n_mesh, int col, int64_t v) {
    int lo = 0, hi = n_mesh - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d[6 * mid + col] <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// [begin, end) of the near-pair rows whose first face is f (pairs sorted by first face)
__device__ __forceinline__ void pair_range(const int32_t* pairs, int64_t n, int32_t f, int64_t* b, int64_t* e) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (__ldg(pairs + 2 * mid) < f) lo = mid + 1; else hi = mid;
    }
    *b = lo;
    hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (__ldg(pairs + 2 * mid) <= f) lo = mid + 1; else hi = mid;
    }
    *e = lo;
}

__device__ __forceinline__ int pow2_at_least(int n) {
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

template <typename K>
__device__ void block_bitonic(K* a, int n) {  // n a power of two; ascending
    for (int k = 2; k <= n; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int p = i ^ j;
                if (p > i) {
                    const K x = a[i], y = a[p];
                    if ((x > y) == ((i & k) == 0)) {
                        a[i] = y;
                        a[p] = x;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Sorts a[0..n) (padding the power-of-two tail with INT_MAX) and compacts the distinct
// values in place; returns their count (same value in every thread).
__device__ int block_sort_unique(int* a, int n, int* s_count) {
    const int np = pow2_at_least(n < 2 ? 2 : n);
    for (int i = n + threadIdx.x; i < np; i += blockDim.x) a[i] = 0x7fffffff;
    __syncthreads();
    block_bitonic(a, np);
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int out = 0, prev = 0x7fffffff;
        for (int base = 0; base < n; base += 32) {
            const int idx = base + lane;
            const int v = idx < n ? a[idx] : 0x7fffffff;
            const int up = __shfl_up_sync(0xffffffffu, v, 1);
            const bool first = (lane == 0) ? (v != prev) : (v != up);
            const bool keep = idx < n && v != 0x7fffffff && first;
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            __syncwarp();
            if (keep) a[out + __popc(m & ((1u << lane) - 1u))] = v;
            out += __popc(m);
            prev = __shfl_sync(0xffffffffu, v, 31);
            __syncwarp();
        }
        if (lane == 0) *s_count = out;
    }
    __syncthreads();
    return *s_count;
}

// Keeps the `cap` edges of e[0..n) nearest to point c (squared midpoint distance, ties by
// id); keys is scratch of >= pow2(n) 64-bit words.  Returns cap.
__device__ int keep_nearest(int* e, int n, int cap, unsigned long long* keys, const float* verts,
                            const int32_t* faces, const int32_t* edge_fe, int64_t edge0, float cx, float cy,
                            float cz) {
    const int np = pow2_at_least(n);
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
        unsigned long long key = ~0ull;
        if (i < n) {
            const int32_t r = __ldg(edge_fe + 2 * (edge0 + e[i]));
            const int32_t f = r / 3, le = r - 3 * f;
            const int32_t a = __ldg(faces + 3 * f + (le + 1) % 3), b = __ldg(faces + 3 * f + (le + 2) % 3);
            const float mx = 0.5f * (__ldg(verts + 3 * a) + __ldg(verts + 3 * b)) - cx;
            const float my = 0.5f * (__ldg(verts + 3 * a + 1) + __ldg(verts + 3 * b + 1)) - cy;
            const float mz = 0.5f * (__ldg(verts + 3 * a + 2) + __ldg(verts + 3 * b + 2)) - cz;
            const float d2 = mx * mx + my * my + mz * mz;
            key = ((unsigned long long)__float_as_uint(d2) << 32) | (unsigned)e[i];
        }
        keys[i] = key;
    }
    __syncthreads();
    block_bitonic(keys, np);
    for (int i = threadIdx.x; i < cap; i += blockDim.x) e[i] = (int)(keys[i] & 0xffffffffull);
    __syncthreads();
    return cap;
}

struct SpaiSmem {
    float2 A[(kSpaiWidth + 1) * kSpaiRowsP];  // column-major, column length kSpaiRowsP
    int cand[kSpaiCand];
    int s1[kSpaiS1Cap];
    int s1_off[kSpaiS1Cap + 1];
    int J[kSpaiWidth];
    int I[kSpaiRows];
    float2 alpha[kSpaiWidth];
    float beta;
    int count, nJ, nI, pj, status;
};
static_assert(sizeof(unsigned long long) * kSpaiCand <= sizeof(float2) * (kSpaiWidth + 1) * kSpaiRowsP,
              "distance keys reuse the A buffer");

__device__ __forceinline__ float2 cmul_conj(float2 a, float2 b) {  // conj(a) * b
    return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kSpaiThreads) spai_column_kernel(
    const float* __restrict__ verts, const int32_t* __restrict__ faces, const int32_t* __restrict__ fei,
    const int32_t* __restrict__ edge_fe, const int32_t* __restrict__ pairs, int64_t n_pairs,
    const int64_t* __restrict__ desc, int n_mesh, const float* __restrict__ z, int32_t* __restrict__ out_cols,
    float2* __restrict__ out_vals, int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SpaiSmem& S = *reinterpret_cast<SpaiSmem*>(smem_raw);
    const int64_t g = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const SpaiDesc D = load_desc(desc, find_mesh(desc, n_mesh, 2, g));
    const int jl = (int)(g - D.edge0);
    const int32_t ra = __ldg(edge_fe + 2 * g), rb = __ldg(edge_fe + 2 * g + 1);
    if (ra < 0) {  // an edge without faces (bad map, already flagged): an empty column
        for (int c = tid; c < kSpaiWidth; c += kSpaiThreads) {
            out_cols[g * kSpaiWidth + c] = -1;
            out_vals[g * kSpaiWidth + c] = make_float2(0.f, 0.f);
        }
        return;
    }
    if (tid == 0) S.status = 0;
    // midpoint of edge j (distance reference of the caps)
    float cx, cy, cz;
    {
        const int32_t f = ra / 3, le = ra - 3 * f;
        const int32_t a = __ldg(faces + 3 * f + (le + 1) % 3), b = __ldg(faces + 3 * f + (le + 2) % 3);
        cx = 0.5f * (__ldg(verts + 3 * a) + __ldg(verts + 3 * b));
        cy = 0.5f * (__ldg(verts + 3 * a + 1) + __ldg(verts + 3 * b + 1));
        cz = 0.5f * (__ldg(verts + 3 * a + 2) + __ldg(verts + 3 * b + 2));
    }
    // ---- 1a. S1 = faces sharing a vertex with fa or fb -------------------------------------
    if (tid < 2) {
        const int32_t r = tid == 0 ? ra : rb;
        int64_t b = 0, e = 0;
        if (r >= 0) pair_range(pairs, n_pairs, r / 3, &b, &e);
        S.s1_off[tid] = (int)(e - b);
        S.s1_off[2 + tid] = (int)b;  // scratch: range starts
    }
    __syncthreads();
    {
        const int na = S.s1_off[0], nb = S.s1_off[1], ba = S.s1_off[2], bb = S.s1_off[3];
        int n = na + nb;
        if (n > kSpaiCand) n = kSpaiCand;
        for (int i = tid; i < n; i += kSpaiThreads)
            S.cand[i] = __ldg(pairs + 2 * (i < na ? (int64_t)ba + i : (int64_t)bb + (i - na)) + 1);
        __syncthreads();
        int n1 = block_sort_unique(S.cand, n, &S.count);
        if (n1 > kSpaiS1Cap) {
            n1 = kSpaiS1Cap;
            if (tid == 0) atomicOr(&S.status, kSpaiTruncated);
        }
        for (int i = tid; i < n1; i += kSpaiThreads) S.s1[i] = S.cand[i];
        if (tid == 0) S.count = n1;
        __syncthreads();
    }
    const int n1 = S.count;
    // ---- 1b. J = edges of S1 ---------------------------------------------------------------
    for (int i = tid; i < 3 * n1; i += kSpaiThreads) {
        const int32_t e = __ldg(fei + 3 * (int64_t)S.s1[i / 3] + i % 3);
        const bool ok = e >= 0 && e < D.ne;  // an id outside the mesh is dropped (and flagged)
        if (!ok) atomicOr(&S.status, kSpaiBadMap);
        S.cand[i] = ok ? e : 0x7fffffff;
    }
    __syncthreads();
    {
        int nJ = block_sort_unique(S.cand, 3 * n1, &S.count);
        if (nJ > kSpaiWidth) {
            nJ = keep_nearest(S.cand, nJ, kSpaiWidth, reinterpret_cast<unsigned long long*>(S.A), verts, faces,
                              edge_fe, D.edge0, cx, cy, cz);
            if (tid == 0) atomicOr(&S.status, kSpaiTruncated);
        }
        for (int i = tid; i < nJ; i += kSpaiThreads) S.J[i] = S.cand[i];
        if (tid == 0) S.nJ = nJ;
        __syncthreads();
    }
    // ---- 1c. S2 = faces sharing a vertex with a face of S1 ---------------------------------
    for (int i = tid; i < n1; i += kSpaiThreads) {
        int64_t b, e;
        pair_range(pairs, n_pairs, S.s1[i], &b, &e);
        S.s1_off[i + 1] = (int)(e - b);
        S.cand[kSpaiCand - 1 - i] = (int)b;  // range starts kept at the buffer's end
    }
    __syncthreads();
    if (tid == 0) {
        S.s1_off[0] = 0;
        for (int i = 0; i < n1; ++i) S.s1_off[i + 1] += S.s1_off[i];
    }
    __syncthreads();
    {
        int total = S.s1_off[n1];
        // the range starts occupy cand[kSpaiCand - n1, kSpaiCand): copy them out of the way
        int starts[kSpaiS1Cap / kSpaiThreads];
#pragma unroll
        for (int q = 0; q < kSpaiS1Cap / kSpaiThreads; ++q) {
            const int i = tid + q * kSpaiThreads;
            starts[q] = i < n1 ? S.cand[kSpaiCand - 1 - i] : 0;
        }
        __syncthreads();
        const int cap = kSpaiCand;
        if (total > cap) {
            total = cap;
            if (tid == 0) atomicOr(&S.status, kSpaiTruncated);
        }
#pragma unroll
        for (int q = 0; q < kSpaiS1Cap / kSpaiThreads; ++q) {
            const int i = tid + q * kSpaiThreads;
            if (i < n1) {
                const int o0 = S.s1_off[i], o1 = S.s1_off[i + 1];
                for (int o = o0; o < o1 && o < cap; ++o)
                    S.cand[o] = __ldg(pairs + 2 * ((int64_t)starts[q] + (o - o0)) + 1);
            }
        }
        __syncthreads();
        int n2 = block_sort_unique(S.cand, total, &S.count);
        // ---- 1d. I = edges of S2 (S2 kept in cand[0..n2); edges written after it) ----------
        int n2e = n2;
        if (3 * n2e > kSpaiCand) {
            n2e = kSpaiCand / 3;
            if (tid == 0) atomicOr(&S.status, kSpaiTruncated);
        }
        // write the edges back to front so no face id is overwritten before it is read
        __syncthreads();
        int fl[kSpaiCand / kSpaiThreads];
#pragma unroll
        for (int q = 0; q < kSpaiCand / kSpaiThreads; ++q) {
            const int i = tid + q * kSpaiThreads;
            fl[q] = i < n2e ? S.cand[i] : 0;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kSpaiCand / kSpaiThreads; ++q) {
            const int i = tid + q * kSpaiThreads;
            if (i < n2e) {
                for (int e3 = 0; e3 < 3; ++e3) {
                    const int32_t e = __ldg(fei + 3 * (int64_t)fl[q] + e3);
                    const bool ok = e >= 0 && e < D.ne;
                    if (!ok) atomicOr(&S.status, kSpaiBadMap);
                    S.cand[3 * i + e3] = ok ? e : 0x7fffffff;
                }
            }
        }
        __syncthreads();
        int nI = block_sort_unique(S.cand, 3 * n2e, &S.count);
        if (nI > kSpaiRows) {
            nI = keep_nearest(S.cand, nI, kSpaiRows, reinterpret_cast<unsigned long long*>(S.A), verts, faces,
                              edge_fe, D.edge0, cx, cy, cz);
            if (tid == 0) atomicOr(&S.status, kSpaiTruncated);
        }
        for (int i = tid; i < nI; i += kSpaiThreads) S.I[i] = S.cand[i];
        if (tid == 0) {
            S.nI = nI;
            S.pj = -1;
        }
        __syncthreads();
        for (int i = tid; i < nI; i += kSpaiThreads)
            if (S.I[i] == jl) S.pj = i;
        __syncthreads();
    }
    const int nJ = S.nJ, nI = S.nI, pj = S.pj;
    // ---- 2. A = Z[I, J] and the right-hand side e_j ---------------------------------------
    const float2* zb = reinterpret_cast<const float2*>(z) + D.zoff;
    for (int idx = tid; idx < nI * nJ; idx += kSpaiThreads) {
        const int r = idx / nJ, c = idx - r * nJ;
        S.A[c * kSpaiRowsP + r] = __ldg(zb + (int64_t)S.I[r] * D.pitch + S.J[c]);
    }
    for (int r = tid; r < nI; r += kSpaiThreads) S.A[nJ * kSpaiRowsP + r] = make_float2(r == pj ? 1.f : 0.f, 0.f);
    __syncthreads();
    // ---- 3. Householder QR, applied to the right-hand side as column nJ ---------------------
    const int ncol = nJ < nI ? nJ : nI;
    for (int k = 0; k < ncol; ++k) {
        if (warp == 0) {
            float s = 0.f;
            for (int r = k + lane; r < nI; r += 32) {
                const float2 a = S.A[k * kSpaiRowsP + r];
                s = fmaf(a.x, a.x, fmaf(a.y, a.y, s));
            }
            s = warp_sumf(s);
            if (lane == 0) {
                const float2 x0 = S.A[k * kSpaiRowsP + k];
                const float ax = sqrtf(x0.x * x0.x + x0.y * x0.y);
                const float an = sqrtf(s);
                if (an == 0.f) {
                    S.alpha[k] = make_float2(0.f, 0.f);
                    S.beta = 0.f;
                } else {
                    const float px = ax > 0.f ? x0.x / ax : 1.f, py = ax > 0.f ? x0.y / ax : 0.f;
                    const float2 al = make_float2(-px * an, -py * an);  // alpha = -phase(x0) |x|
                    S.alpha[k] = al;
                    S.A[k * kSpaiRowsP + k] = make_float2(x0.x - al.x, x0.y - al.y);
                    S.beta = 1.f / (an * (an + ax));  // 2 / |v|^2
                }
            }
        }
        __syncthreads();
        const float beta = S.beta;
        if (beta != 0.f) {
            for (int c = k + 1 + warp; c <= nJ; c += kSpaiThreads / 32) {
                float dr = 0.f, di = 0.f;
                for (int r = k + lane; r < nI; r += 32) {
                    const float2 p = cmul_conj(S.A[k * kSpaiRowsP + r], S.A[c * kSpaiRowsP + r]);
                    dr += p.x;
                    di += p.y;
                }
                dr = warp_sumf(dr) * beta;
                di = warp_sumf(di) * beta;
                for (int r = k + lane; r < nI; r += 32) {
                    const float2 v = S.A[k * kSpaiRowsP + r];
                    float2 a = S.A[c * kSpaiRowsP + r];
                    a.x -= dr * v.x - di * v.y;
                    a.y -= dr * v.y + di * v.x;
                    S.A[c * kSpaiRowsP + r] = a;
                }
            }
        }
        __syncthreads();
    }
    // ---- 4. back substitution R y = (Q^H e)[0:nJ] and the column of M ------------------------
    if (warp == 0) {
        float2 y[(kSpaiWidth + 31) / 32];
#pragma unroll
        for (int q = 0; q < (kSpaiWidth + 31) / 32; ++q) y[q] = make_float2(0.f, 0.f);
        bool rank_def = false;
        for (int c = ncol - 1; c >= 0; --c) {
            float sr = 0.f, si = 0.f;
#pragma unroll
            for (int q = 0; q < (kSpaiWidth + 31) / 32; ++q) {
                const int cc = lane + 32 * q;
                if (cc > c && cc < ncol) {
                    const float2 r = S.A[cc * kSpaiRowsP + c];  // R[c][cc]
                    sr += r.x * y[q].x - r.y * y[q].y;
                    si += r.x * y[q].y + r.y * y[q].x;
                }
            }
            sr = warp_sumf(sr);
            si = warp_sumf(si);
            const float2 b = S.A[nJ * kSpaiRowsP + c];
            const float2 al = S.alpha[c];
            const float den = al.x * al.x + al.y * al.y;
            float2 yc = make_float2(0.f, 0.f);
            if (den > 0.f) {
                const float nr = b.x - sr, ni = b.y - si;
                yc = make_float2((nr * al.x + ni * al.y) / den, (ni * al.x - nr * al.y) / den);
            } else {
                rank_def = true;
            }
            if ((c & 31) == lane) y[c >> 5] = yc;
        }
        int32_t* oc = out_cols + g * kSpaiWidth;
        float2* ov = out_vals + g * kSpaiWidth;
#pragma unroll
        for (int q = 0; q < (kSpaiWidth + 31) / 32; ++q) {
            const int c = lane + 32 * q;
            if (c < kSpaiWidth) {
                oc[c] = c < ncol ? S.J[c] : -1;
                ov[c] = c < ncol ? y[q] : make_float2(0.f, 0.f);
            }
        }
        if (lane == 0) {
            int st = S.status;
            if (rank_def || ncol < nJ) st |= kSpaiRankDef;
            if (pj < 0) st |= kSpaiBadMap;
            if (st) atomicOr(status, st);
        }
    }
}

// Row form: M[i, q] = value of column j = col(i, q) at row i (0 when i is not in J_j).
__global__ void spai_rows_kernel(const int64_t* __restrict__ desc, int n_mesh, int64_t total_edges,
                                 const int32_t* __restrict__ col_cols, const float2* __restrict__ col_vals,
                                 int32_t* __restrict__ m_cols, float2* __restrict__ m_vals) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total_edges * kSpaiWidth) return;
    const int64_t i = t / kSpaiWidth;
    const SpaiDesc D = load_desc(desc, find_mesh(desc, n_mesh, 2, i));
    const int32_t jl = __ldg(col_cols + t);
    float2 v = make_float2(0.f, 0.f);
    if (jl >= 0) {
        const int32_t il = (int32_t)(i - D.edge0);
        const int64_t jg = D.edge0 + jl;
        for (int q = 0; q < kSpaiWidth; ++q)
            if (__ldg(col_cols + jg * kSpaiWidth + q) == il) {
                v = col_vals[jg * kSpaiWidth + q];
                break;
            }
    }
    m_cols[t] = jl;
    m_vals[t] = v;
}

// edge_fe[2 g + s] = global face-edge rows 3 f + e of edge g's faces (smaller first, -1 if
// none); ef pre-filled with -1.
__global__ void edge_fe_kernel(const int32_t* __restrict__ fei, const int64_t* __restrict__ desc, int n_mesh,
                               int64_t total_faces, int32_t* __restrict__ ef, int* __restrict__ status) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= total_faces) return;
    const SpaiDesc D = load_desc(desc, find_mesh(desc, n_mesh, 0, f));
    for (int e = 0; e < 3; ++e) {
        const int32_t le = __ldg(fei + 3 * f + e);
        if (le < 0 || le >= D.ne) {
            atomicOr(status, kSpaiBadMap);
            continue;
        }
        const int64_t g = D.edge0 + le;
        const int32_t r = (int32_t)(3 * f + e);
        if (atomicCAS(ef + 2 * g, -1, r) != -1 && atomicCAS(ef + 2 * g + 1, -1, r) != -1)
            atomicOr(status, kSpaiBadMap);
    }
}

__global__ void edge_fe_order_kernel(int64_t total_edges, int32_t* __restrict__ ef, int* __restrict__ status) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total_edges) return;
    const int32_t a = ef[2 * g], b = ef[2 * g + 1];
    if (a < 0) {
        atomicOr(status, kSpaiBadMap);
        return;
    }
    if (b >= 0 && b < a) {
        ef[2 * g] = b;
        ef[2 * g + 1] = a;
    }
}

// y = M v (complex64 in and out; FP32 arithmetic) for one mesh; or y = M v in FP64 with
// complex128 v, y (the correction of the FP64 iterate).
template <typename VT>
__global__ void spai_apply_kernel(const int32_t* __restrict__ m_cols, const float2* __restrict__ m_vals, int64_t n,
                                  const VT* __restrict__ v, VT* __restrict__ y);

template <>
__global__ void spai_apply_kernel<float2>(const int32_t* __restrict__ m_cols, const float2* __restrict__ m_vals,
                                          int64_t n, const float2* __restrict__ v, float2* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float sr = 0.f, si = 0.f;
    for (int q = 0; q < kSpaiWidth; ++q) {
        const int32_t c = __ldg(m_cols + i * kSpaiWidth + q);
        if (c < 0) break;
        const float2 m = __ldg(m_vals + i * kSpaiWidth + q), x = __ldg(v + c);
        sr = fmaf(m.x, x.x, fmaf(-m.y, x.y, sr));
        si = fmaf(m.x, x.y, fmaf(m.y, x.x, si));
    }
    y[i] = make_float2(sr, si);
}

template <>
__global__ void spai_apply_kernel<double2>(const int32_t* __restrict__ m_cols, const float2* __restrict__ m_vals,
                                           int64_t n, const double2* __restrict__ v, double2* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double sr = 0.0, si = 0.0;
    for (int q = 0; q < kSpaiWidth; ++q) {
        const int32_t c = __ldg(m_cols + i * kSpaiWidth + q);
        if (c < 0) break;
        const float2 m = __ldg(m_vals + i * kSpaiWidth + q);
        const double2 x = __ldg(v + c);
        sr = fma((double)m.x, x.x, fma(-(double)m.y, x.y, sr));
        si = fma((double)m.x, x.y, fma((double)m.y, x.x, si));
    }
    y[i] = make_double2(sr, si);
}

// ---------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------
static size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

size_t spai_workspace_bytes(int64_t total_edges) {
    return al256(sizeof(int32_t) * 2 * (size_t)total_edges) + al256(sizeof(int32_t) * kSpaiWidth * (size_t)total_edges) +
           al256(sizeof(float2) * kSpaiWidth * (size_t)total_edges) + al256(sizeof(int));
}

struct SpaiWork {
    int32_t* ef;
    int32_t* ccols;
    float2* cvals;
    int* status;
};

static SpaiWork spai_carve(void* ws, int64_t ne) {
    char* p = static_cast<char*>(ws);
    SpaiWork w;
    w.ef = reinterpret_cast<int32_t*>(p);
    p += al256(sizeof(int32_t) * 2 * (size_t)ne);
    w.ccols = reinterpret_cast<int32_t*>(p);
    p += al256(sizeof(int32_t) * kSpaiWidth * (size_t)ne);
    w.cvals = reinterpret_cast<float2*>(p);
    p += al256(sizeof(float2) * kSpaiWidth * (size_t)ne);
    w.status = reinterpret_cast<int*>(p);
    return w;
}

int spai_build(const float* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc, int n_mesh,
               int64_t total_faces, int64_t total_edges, const int32_t* pairs, int64_t n_pairs, const float* z,
               int32_t* m_cols, float* m_vals, void* ws, size_t ws_bytes, cudaStream_t s) {
    if (!verts || !faces || !fei || !desc || !pairs || !z || !m_cols || !m_vals || !ws)
        return set_error(MB_ERR_ARG, "spai: null pointer");
    if (n_mesh < 1 || total_faces < 1 || total_edges < 1 || n_pairs < 1)
        return set_error(MB_ERR_ARG, "spai: empty input");
    if (total_edges > (int64_t)INT32_MAX || 3 * total_faces > (int64_t)INT32_MAX || n_pairs > (int64_t)INT32_MAX)
        return set_error(MB_ERR_SIZE, "spai: more than 2^31 edges, face-edge rows or near pairs");
    if (ws_bytes < spai_workspace_bytes(total_edges)) return set_error(MB_ERR_ARG, "spai: workspace too small");
    SpaiWork w = spai_carve(ws, total_edges);
    const int smem = (int)sizeof(SpaiSmem);
    cudaError_t e = cudaFuncSetAttribute(spai_column_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "spai smem attribute: %s", cudaGetErrorString(e));
    cudaMemsetAsync(w.status, 0, sizeof(int), s);
    cudaMemsetAsync(w.ef, 0xff, sizeof(int32_t) * 2 * (size_t)total_edges, s);
    edge_fe_kernel<<<(unsigned)((total_faces + 255) / 256), 256, 0, s>>>(fei, desc, n_mesh, total_faces, w.ef,
                                                                       w.status);
    edge_fe_order_kernel<<<(unsigned)((total_edges + 255) / 256), 256, 0, s>>>(total_edges, w.ef, w.status);
    spai_column_kernel<<<(unsigned)total_edges, kSpaiThreads, smem, s>>>(verts, faces, fei, w.ef, pairs, n_pairs, desc,
                                                                        n_mesh, z, w.ccols, w.cvals, w.status);
    const int64_t nt = total_edges * kSpaiWidth;
    spai_rows_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(desc, n_mesh, total_edges, w.ccols, w.cvals,
                                                                  m_cols, reinterpret_cast<float2*>(m_vals));
    return check_launch("spai_build");
}

int spai_status(const void* ws, int64_t total_edges, int32_t* out, cudaStream_t s) {
    SpaiWork w = spai_carve(const_cast<void*>(ws), total_edges);
    cudaError_t e = cudaMemcpyAsync(out, w.status, sizeof(int), cudaMemcpyDefault, s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "spai status: %s", cudaGetErrorString(e));
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "spai status: %s", cudaGetErrorString(e));
    return MB_OK;
}

int spai_apply_c64(const int32_t* m_cols, const float* m_vals, int64_t n, const float* v, float* y, cudaStream_t s) {
    if (n <= 0) return MB_OK;
    spai_apply_kernel<float2><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        m_cols, reinterpret_cast<const float2*>(m_vals), n, reinterpret_cast<const float2*>(v),
        reinterpret_cast<float2*>(y));
    return check_launch("spai_apply_c64");
}

int spai_apply_c128(const int32_t* m_cols, const float* m_vals, int64_t n, const double* v, double* y,
                    cudaStream_t s) {
    if (n <= 0) return MB_OK;
    spai_apply_kernel<double2><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        m_cols, reinterpret_cast<const float2*>(m_vals), n, reinterpret_cast<const double2*>(v),
        reinterpret_cast<double2*>(y));
    return check_launch("spai_apply_c128");
}

}  // namespace mb
