// mgmres.cu -- GMRES(restart) for many right-hand sides in lockstep, Z X = B, with every
// Arnoldi step's m matrix-vector products done as one product Z [v_1 .. v_m] (the split-TF32
// tensor-core GEMM, or the block-diagonal product of many meshes) instead of m HBM-bound
// matvecs.
//
// Each column is an independent GMRES process (its own Hessenberg matrix, Givens rotations
// and residual estimate); only the product is shared.  The Krylov basis is stored in
// complex64 and the two Gram-Schmidt passes (CGS2) run in FP32 arithmetic with FP64 sums
// across rows: GB300's FP64 rate (~1.25 TFLOP/s) would bound an FP64 Gram-Schmidt at a
// quarter of HBM bandwidth, and the FP32-class product already sets the attainable residual
// (~1e-7 relative).  The Hessenberg matrix, the Givens rotations and the iterate X stay
// FP64.  A column whose estimate reaches tol / 2, or whose new basis vector vanishes, stops
// (its later basis vectors are zero) while the others continue.  Every restart cycle starts
// from the residual B - Z X computed with the same product on the complex64 rounding of X.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "tc_common.cuh"

namespace mb {

size_t cgemm_workspace_bytes(int64_t n, int64_t m);
int cgemm_tf32x3(const float* z_hi, const float* z_lo, int64_t n, const float* x, int64_t m, float* y, void* ws,
                 size_t ws_bytes, cudaStream_t s);

constexpr int kMgMaxRestart = 160;

struct MgWork {
    float2* V;      // [(r+1), n, m] complex64 Krylov basis (V_j is the product's input at step j)
    float2* w;      // [n, m] complex64 working vector (also the complex64 X at a restart)
    float2* y32;    // [n, m] complex64 product output
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
    int* crow;      // [m] rows of each column (block-diagonal systems; rows beyond are zero)
    float* scale;   // [m] 1 / |v| of the next basis vector (0 for inactive columns)
    int* count;     // [4]
    int* status;    // [4] mbarrier time-outs of the streamed kernels (0 = none)
    int* colsteps;  // [m] Arnoldi steps each column took (while active), over all cycles
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
    W->V = static_cast<float2*>(take(8 * nm * (r + 1)));
    W->w = static_cast<float2*>(take(8 * nm));
    W->y32 = static_cast<float2*>(take(8 * nm));
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
    W->crow = static_cast<int*>(take(4 * m));
    W->scale = static_cast<float*>(take(4 * m));
    W->count = static_cast<int*>(take(16));
    W->status = static_cast<int*>(take(16));
    W->colsteps = static_cast<int*>(take(4 * m));
    return off;
}

// internal width: m rounded up to even (TMA row strides are multiples of 16 bytes)
static int64_t padded_width(int64_t m) { return m + (m & 1); }

size_t gmres_multi_workspace_bytes(int64_t n, int64_t m, int r) {
    MgWork W;
    return mg_layout(n, padded_width(m), r, cgemm_workspace_bytes(n, padded_width(m)), nullptr, &W);
}

// (the product's slot holds the per-mesh tensor maps of the streamed variant: one per column
// is more than enough)
// and, after them, the preconditioned variant's buffers: the preconditioned basis vector
// [n, mp] complex64 and the cycle's update before M, [n, m] complex128)
static size_t bd_maps_bytes(int64_t m) { return a256(128 * (size_t)std::max<int64_t>(m, 1)); }
static size_t bd_prod_bytes(int64_t n, int64_t m) {
    return bd_maps_bytes(m) + a256(8 * (size_t)n * padded_width(m)) + a256(16 * (size_t)n * m);
}
size_t gmres_blockdiag_workspace_bytes(int64_t n, int64_t m, int r) {
    MgWork W;
    return mg_layout(n, padded_width(m), r, bd_prod_bytes(n, m), nullptr, &W);
}

// ---- kernels ---------------------------------------------------------------------------
// Column-blocked kernels use 256-thread blocks of 32 columns (threadIdx.x) x 8 row lanes
// (threadIdx.y); crow (optional) limits column c to rows k < crow[c].
__device__ __forceinline__ int64_t rows_of(const int* __restrict__ crow, int64_t c, int64_t n) {
    return crow ? (int64_t)__ldg(crow + c) : n;
}

// complex128 X [n, m] -> complex64 [n, mp] (padding columns zero); 32 x 8 blocks
__global__ void mg_to_c64(const double2* __restrict__ src, int64_t n, int64_t m, int64_t mp, float2* __restrict__ dst) {
    const int64_t c = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (c >= mp) return;
    for (int64_t k = blockIdx.y * blockDim.y + threadIdx.y; k < n; k += (int64_t)gridDim.y * blockDim.y) {
        const double2 v = c < m ? src[k * m + c] : make_double2(0.0, 0.0);
        dst[k * mp + c] = make_float2((float)v.x, (float)v.y);
    }
}

// Sum of the 8 row lanes' values of a 32 x 8 block, added to out[c] (FP64 atomics).
__device__ __forceinline__ void col_sum_add(double v, int64_t c, int64_t m, double* __restrict__ out) {
    __shared__ double s[8][33];
    s[threadIdx.y][threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.y == 0 && c < m) {
        double t = 0.0;
#pragma unroll
        for (int q = 0; q < 8; ++q) t += s[q][threadIdx.x];
        atomicAdd(out + c, t);
    }
}

// R = B - Y (B complex128 [n, m], Y complex64 [n, mp] from the product), complex64 into V_0
// [n, mp]; per-column |R|^2 (of the FP64 difference) into sq (pre-zeroed).
__global__ void mg_residual(const double2* __restrict__ b, const float2* __restrict__ y, int64_t n, int64_t m,
                            int64_t mp, float2* __restrict__ r, double* __restrict__ sq) {
    const int64_t c = (int64_t)blockIdx.x * 32 + threadIdx.x;
    double acc = 0.0;
    if (c < mp) {
        for (int64_t k = blockIdx.y * blockDim.y + threadIdx.y; k < n; k += (int64_t)gridDim.y * blockDim.y) {
            const float2 yv = y[k * mp + c];
            const double2 bv = c < m ? b[k * m + c] : make_double2(0.0, 0.0);
            const double re = bv.x - (double)yv.x, im = bv.y - (double)yv.y;
            r[k * mp + c] = make_float2((float)re, (float)im);
            acc += re * re + im * im;
        }
    }
    col_sum_add(acc, c, mp, sq);
}

// per-column |x|^2 of a complex128 [n, m] block into sq (pre-zeroed)
__global__ void mg_colnorm2(const double2* __restrict__ x, int64_t n, int64_t m, double* __restrict__ sq) {
    const int64_t c = (int64_t)blockIdx.x * 32 + threadIdx.x;
    double acc = 0.0;
    if (c < m) {
        for (int64_t k = blockIdx.y * blockDim.y + threadIdx.y; k < n; k += (int64_t)gridDim.y * blockDim.y) {
            const double2 v = x[k * m + c];
            acc += v.x * v.x + v.y * v.y;
        }
    }
    col_sum_add(acc, c, m, sq);
}

// ---- streamed Gram-Schmidt ------------------------------------------------------------------
// The two bandwidth kernels of an Arnoldi step read every basis vector V_0 .. V_{nb-1} once.
// Their tiles (64 rows x 32 columns of complex64, 16 KB) come from TMA into an S-stage ring
// in shared memory (two 16-column boxes per tile, 128-byte swizzle), loaded by one producer
// warp and read by 8 consumer warps; full / empty mbarriers, every wait bounded (a time-out
// sets *status and ends the block).  Consumer lane = 4 ly + lx of warp w owns column
// 4 w + lx and rows ly + 8 t (t < 8) of the tile, so a sum over the tile's rows is a shuffle
// reduction inside the warp and the 8 warps never combine partial sums.  grid.x = column
// groups of 32, grid.y = blocks along the rows (persistent).  The internal width mp is even
// (16-byte TMA row strides).
constexpr int kGsRows = 64;
constexpr int kGsStage = 16384;
constexpr int kGsThreads = 288;  // 8 consumer warps + 1 producer warp
constexpr long long kGsBudget = 1ll << 30;  // SM clocks per wait (~0.5 s)

struct GsMaps {
    CUtensorMap v;    // basis: (mp, n, r+1) 8-byte elements, box (16, 64, 1)
    CUtensorMap src;  // w or y: (mp, n), box (16, 64)
};

// byte offset of (row r, column cc) in a stage: box cc / 16, 128-byte rows, 16-byte chunk
// index XOR (row % 8)
__device__ __forceinline__ uint32_t gs_off(int r, int cc) {
    const int q = cc & 15;
    return (uint32_t)((cc >> 4) * 8192 + r * 128 + (((q >> 1) ^ (r & 7)) << 4) + ((q & 1) << 3));
}

template <int S>
constexpr size_t gs_smem(size_t aux) {
    return 1024 + (size_t)S * kGsStage + 16 * S + aux;
}

struct GsRing {
    unsigned char* stage;
    uint64_t* full;
    uint64_t* empty;
    unsigned char* aux;
};

template <int S>
__device__ __forceinline__ GsRing gs_ring(unsigned char* smem) {
    GsRing g;
    g.stage = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem) + 1023) & ~uintptr_t(1023));
    g.full = reinterpret_cast<uint64_t*>(g.stage + (size_t)S * kGsStage);
    g.empty = g.full + S;
    g.aux = reinterpret_cast<unsigned char*>(g.empty + S);
    return g;
}

// Producer: items p < count, item_of(p) -> (row tile q, basis index i; -1 = the src matrix).
// After the loop it waits for the last use of every stage, so no copy is in flight at exit.
template <int S, typename ItemOf>
__device__ void gs_produce(const GsMaps& maps, const GsRing& g, int64_t count, int c0, ItemOf item_of,
                           int* status) {
    int64_t p = 0;
    for (; p < count; ++p) {
        const int s = (int)(p % S);
        const int64_t use = p / S;
        if (use > 0 && !tc::mbar_wait(&g.empty[s], (uint32_t)((use - 1) & 1), kGsBudget, status, 1)) break;
        int64_t q;
        int i;
        item_of(p, q, i);
        unsigned char* dst = g.stage + (size_t)s * kGsStage;
        tc::mbar_arrive_expect_tx(&g.full[s], kGsStage);
        const int y = (int)(q * kGsRows);
        if (i < 0) {
            tc::tma_load_2d(dst, &maps.src, &g.full[s], c0, y);
            tc::tma_load_2d(dst + 8192, &maps.src, &g.full[s], c0 + 16, y);
        } else {
            tc::tma_load_3d(dst, &maps.v, &g.full[s], c0, y, i);
            tc::tma_load_3d(dst + 8192, &maps.v, &g.full[s], c0 + 16, y, i);
        }
    }
    for (int s = 0; s < S; ++s) {
        const int64_t uses = p > s ? (p - s + S - 1) / S : 0;
        if (uses > 0) tc::mbar_wait(&g.full[s], (uint32_t)((uses - 1) & 1), kGsBudget, status, 2);
    }
}

template <int S>
__device__ __forceinline__ void gs_init(const GsRing& g) {
    if (threadIdx.x == 256) {
        for (int s = 0; s < S; ++s) {
            tc::mbar_init(&g.full[s], 1);
            tc::mbar_init(&g.empty[s], 8);
        }
        tc::fence_mbar_init();
    }
}

// hc[i][c] += sum_k conj(V_i[k][c]) w[k][c] for i < nb (hc pre-zeroed).  A block's work is a
// contiguous range of the sequence (row tile q, item i = -1 .. nb-1), item -1 being w (kept
// in registers for the tile); FP32 products over a thread's 8 rows and the warp's 8 row
// lanes, FP64 sums per (i, column) in shared memory across the block's tiles, FP64 atomics
// once per block.
template <int S>
__global__ void __launch_bounds__(kGsThreads) mg_dots(const __grid_constant__ GsMaps maps,
                                                      const float2* __restrict__ w, int64_t n, int64_t mp, int nb,
                                                      double* __restrict__ hc, int* __restrict__ status) {
    extern __shared__ unsigned char gs_raw[];
    const GsRing g = gs_ring<S>(gs_raw);
    double2* acc_s = reinterpret_cast<double2*>(g.aux);  // [nb][32]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, lx = lane & 3, ly = lane >> 2;
    const int c0 = blockIdx.x * 32;
    const int L = nb + 1;
    const int64_t tiles = (n + kGsRows - 1) / kGsRows;
    const int64_t items = tiles * L;
    const int64_t p0 = items * blockIdx.y / gridDim.y, p1 = items * (blockIdx.y + 1) / gridDim.y;
    if (p0 >= p1) return;
    gs_init<S>(g);
    for (int e = tid; e < nb * 32; e += kGsThreads) acc_s[e] = make_double2(0.0, 0.0);
    __syncthreads();
    if (warp == 8) {
        if (lane == 0) {
            tc::prefetch_tmap(&maps.v);
            tc::prefetch_tmap(&maps.src);
            gs_produce<S>(maps, g, p1 - p0, c0,
                          [&](int64_t p, int64_t& q, int& i) {
                              const int64_t a = p0 + p;
                              q = a / L;
                              i = (int)(a - q * L) - 1;
                          },
                          status);
        }
    } else {
        const int cc = warp * 4 + lx;
        const int64_t c = c0 + cc;
        float2 wv[8];
        {
            // a range that starts inside a tile reads that tile's w directly
            const int64_t q = p0 / L;
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int64_t k = q * kGsRows + ly + 8 * t;
                wv[t] = (k < n && c < mp) ? w[k * mp + c] : make_float2(0.f, 0.f);
            }
        }
        for (int64_t p = 0; p < p1 - p0; ++p) {
            const int s = (int)(p % S);
            if (!tc::mbar_wait(&g.full[s], (uint32_t)((p / S) & 1), kGsBudget, status, 4)) break;
            const unsigned char* st = g.stage + (size_t)s * kGsStage;
            const int i = (int)((p0 + p) % L) - 1;
            if (i < 0) {
#pragma unroll
                for (int t = 0; t < 8; ++t) wv[t] = *reinterpret_cast<const float2*>(st + gs_off(ly + 8 * t, cc));
            } else {
                float ar = 0.f, ai = 0.f;
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const float2 v = *reinterpret_cast<const float2*>(st + gs_off(ly + 8 * t, cc));
                    ar = fmaf(v.x, wv[t].x, fmaf(v.y, wv[t].y, ar));
                    ai = fmaf(v.x, wv[t].y, fmaf(-v.y, wv[t].x, ai));
                }
#pragma unroll
                for (int o = 4; o < 32; o <<= 1) {
                    ar += __shfl_xor_sync(0xffffffffu, ar, o);
                    ai += __shfl_xor_sync(0xffffffffu, ai, o);
                }
                if (ly == 0) {
                    double2& a = acc_s[i * 32 + cc];
                    a.x += (double)ar;
                    a.y += (double)ai;
                }
            }
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&g.empty[s]);
        }
    }
    __syncthreads();
    for (int e = tid; e < nb * 32; e += kGsThreads) {
        const int i = e / 32, cc = e % 32;
        if (c0 + cc >= mp) continue;
        double* h = hc + 2 * ((int64_t)i * mp + c0 + cc);
        atomicAdd(h, acc_s[e].x);
        atomicAdd(h + 1, acc_s[e].y);
    }
}

// dst[k][c] = src[k][c] + sign * sum_{i<nb} V_i[k][c] coef[i][c] (FP32 products and sums;
// dst may alias src).  MODE 0: src / dst complex64 [n, mp] (src streamed as item -1 of each
// tile); MODE 1: the same, plus per-column |dst|^2 added to sq (pre-zeroed); MODE 2: the
// iterate X, complex128 [n, m] read and written directly (columns c < m).  A block owns row
// tiles q = blockIdx.y + j gridDim.y of its column group; the group's coefficients sit in
// shared memory.
template <int S, int MODE>
__global__ void __launch_bounds__(kGsThreads) mg_combine(const __grid_constant__ GsMaps maps,
                                                         const double* __restrict__ coef, int64_t n, int64_t mp,
                                                         int64_t m, int nb, float sign, void* dst_v,
                                                         double* __restrict__ sq, int* __restrict__ status) {
    constexpr bool kStream = MODE != 2;
    extern __shared__ unsigned char gs_raw[];
    const GsRing g = gs_ring<S>(gs_raw);
    float2* s_coef = reinterpret_cast<float2*>(g.aux);  // [nb][32]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, lx = lane & 3, ly = lane >> 2;
    const int c0 = blockIdx.x * 32;
    const int L = nb + (kStream ? 1 : 0);
    const int64_t tiles = (n + kGsRows - 1) / kGsRows;
    const int64_t my_tiles = tiles > blockIdx.y ? (tiles - blockIdx.y + gridDim.y - 1) / gridDim.y : 0;
    if (my_tiles == 0) return;
    const int64_t count = my_tiles * L;
    gs_init<S>(g);
    for (int e = tid; e < nb * 32; e += kGsThreads) {
        const int i = e / 32, cc = e % 32;
        const int64_t q = 2 * ((int64_t)i * mp + c0 + cc);
        s_coef[e] = c0 + cc < mp ? make_float2(sign * (float)coef[q], sign * (float)coef[q + 1]) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (warp == 8) {
        if (lane == 0) {
            tc::prefetch_tmap(&maps.v);
            if (kStream) tc::prefetch_tmap(&maps.src);
            gs_produce<S>(maps, g, count, c0,
                          [&](int64_t p, int64_t& q, int& i) {
                              const int64_t j = p / L;
                              q = blockIdx.y + j * gridDim.y;
                              i = (int)(p - j * L) - (kStream ? 1 : 0);
                          },
                          status);
        }
    } else {
        const int cc = warp * 4 + lx;
        const int64_t c = c0 + cc;
        float2 acc[8];
        float nrm = 0.f;
        for (int64_t p = 0; p < count; ++p) {
            const int s = (int)(p % S);
            if (!tc::mbar_wait(&g.full[s], (uint32_t)((p / S) & 1), kGsBudget, status, 4)) break;
            const unsigned char* st = g.stage + (size_t)s * kGsStage;
            const int64_t j = p / L;
            const int i = (int)(p - j * L) - (kStream ? 1 : 0);
            if (p - j * L == 0) {
#pragma unroll
                for (int t = 0; t < 8; ++t) acc[t] = make_float2(0.f, 0.f);
            }
            if (i < 0) {
#pragma unroll
                for (int t = 0; t < 8; ++t) acc[t] = *reinterpret_cast<const float2*>(st + gs_off(ly + 8 * t, cc));
            } else {
                const float2 h = s_coef[i * 32 + cc];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const float2 v = *reinterpret_cast<const float2*>(st + gs_off(ly + 8 * t, cc));
                    acc[t].x = fmaf(h.x, v.x, fmaf(-h.y, v.y, acc[t].x));
                    acc[t].y = fmaf(h.x, v.y, fmaf(h.y, v.x, acc[t].y));
                }
            }
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&g.empty[s]);
            if (i == nb - 1) {  // tile complete
                const int64_t q = blockIdx.y + j * gridDim.y;
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const int64_t k = q * kGsRows + ly + 8 * t;
                    if (k >= n) continue;
                    if (MODE == 2) {
                        if (c < m) {
                            double2* x = static_cast<double2*>(dst_v) + k * m + c;
                            double2 o = *x;
                            o.x += (double)acc[t].x;
                            o.y += (double)acc[t].y;
                            *x = o;
                        }
                    } else if (c < mp) {
                        static_cast<float2*>(dst_v)[k * mp + c] = acc[t];
                        if (MODE == 1) nrm += acc[t].x * acc[t].x + acc[t].y * acc[t].y;
                    }
                }
            }
        }
        if (MODE == 1) {
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
            if (ly == 0 && c < mp) atomicAdd(sq + c, (double)nrm);
        }
    }
    __syncthreads();
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
// rotation, the residual estimate, the scale of the next basis vector; inactive columns are
// left untouched (their scale stays 0).
__global__ void mg_givens(double* __restrict__ H, double* __restrict__ cs, double* __restrict__ sn,
                          double* __restrict__ g, const double* __restrict__ hn2, const double* __restrict__ bnorm,
                          int j, int r, int64_t m, double tol, int* __restrict__ active, int* __restrict__ jend,
                          int* __restrict__ count, float* __restrict__ scale, int* __restrict__ colsteps) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m || !active[c]) return;
    colsteps[c] += 1;
    auto hre = [&](int i) -> double& { return H[2 * (((int64_t)i * r + j) * m + c)]; };
    auto him = [&](int i) -> double& { return H[2 * (((int64_t)i * r + j) * m + c) + 1]; };
    const double hn = sqrt(hn2[c]);
    // the rotated column: a carries entry i through the loop.  The rotations and the entries
    // below come in chunks of 4, all loaded before the chunk's stores (each load otherwise
    // waits for the previous store to the same array).
    double ar = hre(0), ai = him(0);
    for (int i0 = 0; i0 < j; i0 += 4) {
        double2 cv[4], sv[4], bv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = i0 + u;
            if (i < j) {
                cv[u] = make_double2(cs[2 * ((int64_t)i * m + c)], cs[2 * ((int64_t)i * m + c) + 1]);
                sv[u] = make_double2(sn[2 * ((int64_t)i * m + c)], sn[2 * ((int64_t)i * m + c) + 1]);
                bv[u] = make_double2(hre(i + 1), him(i + 1));
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = i0 + u;
            if (i >= j) break;
            const double cr = cv[u].x, ci = cv[u].y, sr = sv[u].x, si = sv[u].y, br = bv[u].x, bi = bv[u].y;
            // t = conj(c) a + conj(s) b ;  b' = -s a + c b
            hre(i) = cr * ar + ci * ai + sr * br + si * bi;
            him(i) = cr * ai - ci * ar + sr * bi - si * br;
            const double nbr = -(sr * ar - si * ai) + (cr * br - ci * bi);
            const double nbi = -(sr * ai + si * ar) + (cr * bi + ci * br);
            ar = nbr;
            ai = nbi;
        }
    }
    const double br = hn, bi = 0.0;
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
    const double e1 = -(sr * gr - si * gi), e2 = -(sr * gi + si * gr);
    g[2 * ((int64_t)(j + 1) * m + c)] = e1;
    g[2 * ((int64_t)(j + 1) * m + c) + 1] = e2;
    g[2 * ((int64_t)j * m + c)] = cr * gr + ci * gi;
    g[2 * ((int64_t)j * m + c) + 1] = cr * gi - ci * gr;
    const double est = sqrt(e1 * e1 + e2 * e2) / bnorm[c];
    jend[c] = j + 1;
    if (est <= 0.5 * tol || hn <= 1e-300 || j + 1 == r) {
        active[c] = 0;
        scale[c] = 0.f;
    } else {
        scale[c] = (float)(1.0 / hn);
        atomicAdd(count, 1);
    }
}

// dst[k][c] = scale[c] src[k][c] for k < the column's rows, 0 beyond: the next basis vector
// (src = w) and the start of a cycle (src = dst = V_0).
__global__ void mg_scale_cols(const float2* src, const float* __restrict__ scale, const int* __restrict__ crow,
                              int64_t n, int64_t m, float2* dst) {
    const int64_t c = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (c >= m) return;
    const int64_t nr = rows_of(crow, c, n);
    const float s = scale[c];
    for (int64_t k = blockIdx.y * blockDim.y + threadIdx.y; k < n; k += (int64_t)gridDim.y * blockDim.y) {
        const float2 v = src[k * m + c];
        dst[k * m + c] = k < nr ? make_float2(v.x * s, v.y * s) : make_float2(0.f, 0.f);
    }
}

// column c of mesh i (nc columns each) has E_i rows
// (padding columns c >= m have no rows)
__global__ void mg_column_rows(const int64_t* __restrict__ desc, int64_t m, int64_t mp, int nc,
                               int* __restrict__ crow) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < mp) crow[c] = c < m ? (int)desc[6 * (c / nc) + 2] : 0;
}

// Start of a cycle, per column: g = (beta, 0, ..), active = beta / |b| > tol, scale = 1 / beta.
__global__ void mg_init_g(const double* __restrict__ beta2, const double* __restrict__ bnorm, int r, int64_t m,
                          double tol, double* __restrict__ g, int* __restrict__ jend, int* __restrict__ count,
                          int* __restrict__ active, float* __restrict__ scale) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m) return;
    for (int i = 0; i <= r; ++i) {
        g[2 * ((int64_t)i * m + c)] = 0.0;
        g[2 * ((int64_t)i * m + c) + 1] = 0.0;
    }
    const double beta = sqrt(beta2[c]);
    g[2 * c] = beta;
    jend[c] = 0;
    const bool act = beta / bnorm[c] > tol;
    active[c] = act ? 1 : 0;
    scale[c] = act ? (float)(1.0 / beta) : 0.f;
    if (act) atomicAdd(count, 1);
}

// back substitution per column (upper-triangular jend x jend), then y into yv.  One warp per
// block; the solution being built stays in shared memory ([r][32] complex128).
__global__ void __launch_bounds__(32) mg_backsolve(const double* __restrict__ H, const double* __restrict__ g,
                                                   const int* __restrict__ jend, int r, int64_t m,
                                                   double* __restrict__ yv) {
    extern __shared__ double2 s_y[];
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m) return;
    const int k = jend[c];
    double2* y = s_y + threadIdx.x;  // y[q * 32]
    for (int i = k - 1; i >= 0; --i) {
        double ar = g[2 * ((int64_t)i * m + c)], ai = g[2 * ((int64_t)i * m + c) + 1];
        for (int q = i + 1; q < k; ++q) {
            const double hr = H[2 * (((int64_t)i * r + q) * m + c)], hi = H[2 * (((int64_t)i * r + q) * m + c) + 1];
            const double2 yq = y[q * 32];
            ar -= hr * yq.x - hi * yq.y;
            ai -= hr * yq.y + hi * yq.x;
        }
        const double dr = H[2 * (((int64_t)i * r + i) * m + c)], di = H[2 * (((int64_t)i * r + i) * m + c) + 1];
        const double den = dr * dr + di * di;
        y[i * 32] = den > 0.0 ? make_double2((ar * dr + ai * di) / den, (ai * dr - ar * di) / den)
                              : make_double2(0.0, 0.0);
    }
    for (int i = 0; i < r; ++i) {
        const double2 v = i < k ? y[i * 32] : make_double2(0.0, 0.0);
        yv[2 * ((int64_t)i * m + c)] = v.x;
        yv[2 * ((int64_t)i * m + c) + 1] = v.y;
    }
}

// ---- block-diagonal product (many meshes) ------------------------------------------------
// desc[i] = (face offset, faces, edges E_i, offset of Z_i in the flat array (complex entries),
// -, first right-hand-side column); Z_i is stored row-major with the even row pitch
// P_i = E_i + (E_i & 1), so every row starts on a 16-byte boundary.  goff[i] = first work
// unit of mesh i (a unit owns ROWS rows), goff[n_mesh] = total units.
// y[r, col + c] = sum_l Z_i[r, l] x[l, col + c] for the NC columns of mesh i; x, y:
// [rows_max, ld] interleaved complex64; FP32 products and sums.  Rows of the padded block
// beyond E_i are never written.
__device__ __forceinline__ int seg_of(const int64_t* __restrict__ off, int n, int64_t v) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// A mesh is live while any of its nc columns (first column co) is still iterating in the
// current cycle (cact = the solver's per-column flags; null: every mesh is live).  The
// products of an Arnoldi step skip the other meshes: their columns' next basis vectors are
// scaled by 0, so their (stale, finite) product rows are never used.
__device__ __forceinline__ bool mesh_live(const int* __restrict__ cact, int64_t co, int nc) {
    if (!cact) return true;
    for (int c = 0; c < nc; ++c)
        if (cact[co + c]) return true;
    return false;
}

template <int ROWS, int NC>
__global__ void __launch_bounds__(256) blockdiag_matvec_kernel(const float* __restrict__ z,
                                                               const int64_t* __restrict__ desc,
                                                               const int64_t* __restrict__ goff, int n_mesh,
                                                               const float* __restrict__ x, int64_t ld,
                                                               float* __restrict__ y, const int* __restrict__ cact) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= __ldg(goff + n_mesh)) return;
    const int i = seg_of(goff, n_mesh, w);
    const int64_t E = __ldg(desc + 6 * i + 2), zo = __ldg(desc + 6 * i + 3), co = __ldg(desc + 6 * i + 5);
    if (!mesh_live(cact, co, NC)) return;  // warp-uniform
    const int64_t P = E + (E & 1);
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
                const float2 a = __ldcs(zc + (r0 + q) * P + l);
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

// Streamed variant (ROWS = 32): a block takes units u = blockIdx.x + j gridDim.x; per unit and
// chunk of 64 columns a producer warp loads, by TMA, the 32 x 64 tile of Z_i (one tensor map
// per mesh, in global memory: rows of pitch P_i, zero fill beyond E_i) and the 64 x 8 tile
// of x at the mesh's columns (64-byte swizzle) into a kBdStages ring; 8 consumer warps own
// 4 rows each and lanes stride over the chunk's columns, both operands from shared memory.
// Waits are bounded (a time-out sets *status and ends the block).
constexpr int kBdRows = 32, kBdCols = 64, kBdZBytes = kBdRows * kBdCols * 8, kBdXBytes = kBdCols * 64;
constexpr int kBdStage = kBdZBytes + kBdXBytes, kBdStages = 4;
constexpr int kBdThreads = 288;
constexpr size_t kBdSmem = 1024 + (size_t)kBdStages * kBdStage + 16 * kBdStages;

// byte offset of x tile element (row j, byte column cb) under the 64-byte swizzle
__device__ __forceinline__ uint32_t bd_xoff(int j, int cb) {
    return (uint32_t)(j * 64 + ((((cb >> 4) ^ (j >> 1)) & 3) << 4) + (cb & 15));
}

template <int NC>
__global__ void __launch_bounds__(kBdThreads) blockdiag_stream_kernel(const CUtensorMap* __restrict__ zmaps,
                                                                      const __grid_constant__ CUtensorMap xmap,
                                                                      const int64_t* __restrict__ desc,
                                                                      const int64_t* __restrict__ uoff, int n_mesh,
                                                                      int64_t ld, float* __restrict__ y,
                                                                      int* __restrict__ status,
                                                                      const int* __restrict__ cact) {
    extern __shared__ unsigned char bd_raw[];
    unsigned char* stage =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(bd_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(stage + (size_t)kBdStages * kBdStage);
    uint64_t* empty = full + kBdStages;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t units = __ldg(uoff + n_mesh);
    if (threadIdx.x == 256) {
        for (int s = 0; s < kBdStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 8);
        }
        tc::fence_mbar_init();
    }
    __syncthreads();
    if (warp == 8) {
        if (lane == 0) {
            tc::prefetch_tmap(&xmap);
            int64_t p = 0;
            bool ok = true;
            for (int64_t u = blockIdx.x; u < units && ok; u += gridDim.x) {
                const int i = seg_of(uoff, n_mesh, u);
                const int64_t E = __ldg(desc + 6 * i + 2), co = __ldg(desc + 6 * i + 5);
                if (!mesh_live(cact, co, NC)) continue;  // the consumers skip the same units
                const int r0 = (int)((u - __ldg(uoff + i)) * kBdRows);
                const CUtensorMap* zm = zmaps + i;
                for (int64_t l0 = 0; l0 < E; l0 += kBdCols, ++p) {
                    const int s = (int)(p % kBdStages);
                    const int64_t use = p / kBdStages;
                    if (use > 0 && !tc::mbar_wait(&empty[s], (uint32_t)((use - 1) & 1), kGsBudget, status, 8)) {
                        ok = false;
                        break;
                    }
                    unsigned char* st = stage + (size_t)s * kBdStage;
                    tc::mbar_arrive_expect_tx(&full[s], kBdStage);
                    tc::tma_load_2d(st, zm, &full[s], (int)l0, r0);
                    tc::tma_load_2d(st + kBdZBytes, &xmap, &full[s], (int)(co & ~1ll), (int)l0);
                }
            }
            for (int s = 0; s < kBdStages; ++s) {
                const int64_t uses = p > s ? (p - s + kBdStages - 1) / kBdStages : 0;
                if (uses > 0) tc::mbar_wait(&full[s], (uint32_t)((uses - 1) & 1), kGsBudget, status, 16);
            }
        }
    } else {
        int64_t p = 0;
        bool ok = true;
        for (int64_t u = blockIdx.x; u < units && ok; u += gridDim.x) {
            const int i = seg_of(uoff, n_mesh, u);
            const int64_t E = __ldg(desc + 6 * i + 2), co = __ldg(desc + 6 * i + 5);
            if (!mesh_live(cact, co, NC)) continue;
            const int64_t r0 = (u - __ldg(uoff + i)) * kBdRows + warp * 4;
            const int cb0 = (int)(co & 1) * 8;  // byte column of the mesh's first column in the x tile
            float ar[4][NC], ai[4][NC];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int c = 0; c < NC; ++c) ar[q][c] = ai[q][c] = 0.f;
            for (int64_t l0 = 0; l0 < E; l0 += kBdCols, ++p) {
                const int s = (int)(p % kBdStages);
                if (!tc::mbar_wait(&full[s], (uint32_t)((p / kBdStages) & 1), kGsBudget, status, 32)) {
                    ok = false;
                    break;
                }
                const unsigned char* st = stage + (size_t)s * kBdStage;
                const float2* zt = reinterpret_cast<const float2*>(st);
                const unsigned char* xt = st + kBdZBytes;
#pragma unroll
                for (int t = 0; t < kBdCols / 32; ++t) {
                    const int j = lane + 32 * t;
                    if (l0 + j >= E) break;
                    float2 xv[NC];
                    if (NC % 2 == 0 && cb0 == 0) {
#pragma unroll
                        for (int c = 0; c < NC / 2; ++c) {
                            const float4 v = *reinterpret_cast<const float4*>(xt + bd_xoff(j, 16 * c));
                            xv[2 * c] = make_float2(v.x, v.y);
                            xv[2 * c + 1] = make_float2(v.z, v.w);
                        }
                    } else {
#pragma unroll
                        for (int c = 0; c < NC; ++c) xv[c] = *reinterpret_cast<const float2*>(xt + bd_xoff(j, cb0 + 8 * c));
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float2 a = zt[(warp * 4 + q) * kBdCols + j];
#pragma unroll
                        for (int c = 0; c < NC; ++c) {
                            ar[q][c] = fmaf(a.x, xv[c].x, fmaf(-a.y, xv[c].y, ar[q][c]));
                            ai[q][c] = fmaf(a.x, xv[c].y, fmaf(a.y, xv[c].x, ai[q][c]));
                        }
                    }
                }
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&empty[s]);
            }
            if (!ok) break;
#pragma unroll
            for (int q = 0; q < 4; ++q)
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
    }
    __syncthreads();
}

int tmap_encode(CUtensorMap* map, CUtensorMapDataType type, int rank, const void* ptr, const uint64_t* dims,
                const uint64_t* strides, const uint32_t* box, CUtensorMapSwizzle swizzle);

// Per-mesh tensor maps of the flat block-diagonal array (host desc copy), written to dev.
static int bd_zmaps(const float* z, const int64_t* desc_h, int n_mesh, CUtensorMap* dev, cudaStream_t s) {
    std::vector<CUtensorMap> maps((size_t)n_mesh);
    for (int i = 0; i < n_mesh; ++i) {
        const int64_t E = desc_h[6 * i + 2], zo = desc_h[6 * i + 3], P = E + (E & 1);
        if (zo & 1) return set_error(MB_ERR_ARG, "block-diagonal product: Z_%d offset must be even", i);
        const uint64_t dims[2] = {(uint64_t)P, (uint64_t)E};
        const uint64_t strides[1] = {(uint64_t)P * 8};
        const uint32_t box[2] = {(uint32_t)kBdCols, (uint32_t)kBdRows};
        int rc = tmap_encode(&maps[i], CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, z + 2 * zo, dims, strides, box,
                             CU_TENSOR_MAP_SWIZZLE_NONE);
        if (rc) return rc;
    }
    cudaError_t e = cudaMemcpyAsync(dev, maps.data(), sizeof(CUtensorMap) * n_mesh, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "block-diagonal product: tensor maps: %s", cudaGetErrorString(e));
    return MB_OK;
}

static int bd_xmap(CUtensorMap* map, const float* x, int64_t n_rows, int64_t ld) {
    if (ld & 1) return set_error(MB_ERR_ARG, "block-diagonal product (streamed): ld must be even");
    const uint64_t dims[2] = {(uint64_t)ld, (uint64_t)n_rows};
    const uint64_t strides[1] = {(uint64_t)ld * 8};
    const uint32_t box[2] = {8, (uint32_t)kBdCols};
    return tmap_encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, x, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_64B);
}

static int bd_launch(const CUtensorMap* zmaps, const float* x, int64_t n_rows, const int64_t* desc,
                     const int64_t* goff, int n_mesh, int64_t total_units, int64_t ld, int nc, float* y, int* status,
                     cudaStream_t s, const int* cact = nullptr) {
    CUtensorMap xm;
    int rc = bd_xmap(&xm, x, n_rows, ld);
    if (rc) return rc;
    int sms = 152, dev = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
#define MB_BDS(C)                                                                                               \
    if (nc == C) {                                                                                              \
        cudaFuncSetAttribute(blockdiag_stream_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBdSmem); \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, blockdiag_stream_kernel<C>, kBdThreads, kBdSmem);   \
        const int64_t g = std::max<int64_t>(1, std::min<int64_t>(total_units, (int64_t)std::max(per_sm, 1) * sms)); \
        blockdiag_stream_kernel<C><<<(unsigned)g, kBdThreads, kBdSmem, s>>>(zmaps, xm, desc, goff, n_mesh, ld, y,  \
                                                                           status, cact);                       \
        return check_launch("blockdiag_matvec (streamed)");                                                     \
    }
    MB_BDS(1) MB_BDS(2) MB_BDS(4) MB_BDS(8)
#undef MB_BDS
    return set_error(MB_ERR_UNSUPPORTED, "block-diagonal product: columns per mesh in {1, 2, 4, 8}");
}

int blockdiag_matvec(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                     const float* x, int64_t ld, int nc, int rows, float* y, cudaStream_t s, const int* cact) {
    if (n_mesh <= 0 || total_warps <= 0) return MB_OK;
    if (rows == kBdRows) {
        // standalone call: the tensor maps and the time-out word in stream-ordered buffers of
        // this call, the word checked here
        if (reinterpret_cast<uintptr_t>(z) & 15) return set_error(MB_ERR_ARG, "z must be 16-byte aligned");
        std::vector<int64_t> dh((size_t)6 * n_mesh);
        cudaMemcpyAsync(dh.data(), desc, 48 * (size_t)n_mesh, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return check_launch("blockdiag_matvec: descriptors");
        void* buf = nullptr;
        const size_t map_bytes = sizeof(CUtensorMap) * (size_t)n_mesh;
        if (cudaMallocAsync(&buf, map_bytes + 256, s) != cudaSuccess)
            return set_error(MB_ERR_CUDA, "block-diagonal product: scratch");
        CUtensorMap* maps = static_cast<CUtensorMap*>(buf);
        int* own = reinterpret_cast<int*>(static_cast<char*>(buf) + map_bytes);
        int rc = bd_zmaps(z, dh.data(), n_mesh, maps, s);
        int64_t rows_max = 0;
        for (int i = 0; i < n_mesh; ++i) rows_max = std::max(rows_max, dh[6 * i + 2]);
        if (!rc) {
            cudaMemsetAsync(own, 0, 4, s);
            rc = bd_launch(maps, x, rows_max, desc, goff, n_mesh, total_warps, ld, nc, y, own, s);
        }
        int hs = 0;
        if (!rc) cudaMemcpyAsync(&hs, own, 4, cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(buf, s);
        const cudaError_t e = cudaStreamSynchronize(s);
        if (rc) return rc;
        if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "blockdiag_matvec: %s", cudaGetErrorString(e));
        if (hs) return set_error(MB_ERR_CUDA, "blockdiag_matvec: wait timed out (code %d)", hs);
        return MB_OK;
    }
    const int64_t blocks = (total_warps * 32 + 255) / 256;
    if (blocks > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "batch too large for one launch");
#define MB_BD(R, C)                                                                                           \
    if (rows == R && nc == C) {                                                                               \
        blockdiag_matvec_kernel<R, C><<<(unsigned)blocks, 256, 0, s>>>(z, desc, goff, n_mesh, x, ld, y, cact); \
        return check_launch("blockdiag_matvec");                                                              \
    }
    MB_BD(1, 1) MB_BD(2, 1) MB_BD(4, 1) MB_BD(8, 1)
    MB_BD(1, 2) MB_BD(2, 2) MB_BD(4, 2) MB_BD(8, 2)
    MB_BD(1, 4) MB_BD(2, 4) MB_BD(4, 4) MB_BD(8, 4)
    MB_BD(1, 8) MB_BD(2, 8) MB_BD(4, 8)
#undef MB_BD
    return set_error(MB_ERR_UNSUPPORTED, "block-diagonal product: rows per warp in {1, 2, 4, 8} (8 with up to 4 "
                                         "columns) or 32 (streamed), columns per mesh in {1, 2, 4, 8}");
}

// ---- host driver -------------------------------------------------------------------------
static int mg_sync(cudaStream_t s, const char* what) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return check_launch(what);
}

int tmap_encode(CUtensorMap* map, CUtensorMapDataType type, int rank, const void* ptr, const uint64_t* dims,
                const uint64_t* strides, const uint32_t* box, CUtensorMapSwizzle swizzle);

// Tensor maps of the streamed kernels: the basis (mp, n, r+1) and one [n, mp] matrix.
static int gs_maps(GsMaps* g, const float2* V, const float2* src, int64_t n, int64_t mp, int r) {
    const uint64_t dv[3] = {(uint64_t)mp, (uint64_t)n, (uint64_t)(r + 1)};
    const uint64_t sv[2] = {(uint64_t)mp * 8, (uint64_t)n * mp * 8};
    const uint32_t bv[3] = {16, (uint32_t)kGsRows, 1};
    int rc = tmap_encode(&g->v, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, V, dv, sv, bv, CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
    return tmap_encode(&g->src, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, src, dv, sv, bv, CU_TENSOR_MAP_SWIZZLE_128B);
}

// ---------------------------------------------------------------------------------------
// Near-field right preconditioner of the batched (block-diagonal) systems: column c belongs to
// mesh i = c / nc and is preconditioned by M_i, rows eoff[i] .. eoff[i] + E_i of the ELL rows
// of MB_SPAI_WIDTH (local column, value) pairs that mb_spai_build_c64 builds for the batch.
// Each Arnoldi step multiplies Z by M V_j; each cycle's update V y goes through M before it
// is added to X.
// ---------------------------------------------------------------------------------------
struct BdPrecond {
    const int32_t* cols;
    const float2* vals;
    const int64_t* desc;  // the batch descriptor (E_i in column 2, offset of Z_i in column 3)
    const int64_t* eoff;  // [n_mesh] first global edge of each mesh
    int n_mesh;
    int nc;
    const float2* z;      // the flat block-diagonal Z (row pitch E_i rounded up to even)
    float2* z32;          // [n, mp] M V_j
    double2* u;           // [n, m] the cycle's update before M (the split X at a cycle start)
};

// X (complex128 [n, m]) -> FP32 (hi, lo) parts, float4 [n, m]
__global__ void bd_split_kernel(const double2* __restrict__ x, int64_t count, float4* __restrict__ xs) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const double2 v = x[k];
    const float hr = (float)v.x, hi = (float)v.y;
    xs[k] = make_float4(hr, hi, (float)(v.x - (double)hr), (float)(v.y - (double)hi));
}

__device__ __forceinline__ void bd_two_sum(float& s, float t, float& e) {
    const float u = __fadd_rn(s, t);
    const float bb = __fsub_rn(u, s);
    e = __fadd_rn(__fsub_rn(s, __fsub_rn(u, bb)), __fsub_rn(t, bb));
    s = u;
}

// Refinement residual of the block-diagonal systems, R = B - Z X with X given by its FP32
// split: compensated FP32 dot products (exact products by TwoProduct, exact running sums by
// TwoSum, the rounding terms and the x_lo products summed beside them, lane sums combined in
// FP64) -- FP64-class accuracy at FP32 instruction speed.  One warp per Z row (global row g:
// mesh i, local row k) and all NC columns of the mesh; R (complex64) into V_0 [n, mp] (the
// caller zeroes it) and |R|^2 per column into sq.
template <int NC>
__global__ void __launch_bounds__(256) bd_residual_kernel(BdPrecond P, int64_t total_rows, int64_t m, int64_t mp,
                                                          const float4* __restrict__ xs, const double2* __restrict__ b,
                                                          float2* __restrict__ r, double* __restrict__ sq) {
    const int64_t g = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (g >= total_rows) return;
    int lo = 0, hi = P.n_mesh - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.eoff[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const int i = lo;
    const int64_t e = P.desc[6 * i + 2], k = g - P.eoff[i];
    const float2* zr = P.z + P.desc[6 * i + 3] + k * (e + (e & 1));
    const int64_t c0 = (int64_t)i * NC;
    float sr[NC], si[NC], cr[NC], ci[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) sr[q] = si[q] = cr[q] = ci[q] = 0.f;
    for (int64_t j = lane; j < e; j += 32) {
        const float2 a = __ldcs(zr + j);
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            const float4 x = __ldg(xs + j * m + c0 + q);
            const float p1 = __fmul_rn(a.x, x.x), e1 = fmaf(a.x, x.x, -p1);
            const float p2 = __fmul_rn(-a.y, x.y), e2 = fmaf(-a.y, x.y, -p2);
            const float p3 = __fmul_rn(a.x, x.y), e3 = fmaf(a.x, x.y, -p3);
            const float p4 = __fmul_rn(a.y, x.x), e4 = fmaf(a.y, x.x, -p4);
            float t1, t2, t3, t4;
            bd_two_sum(sr[q], p1, t1);
            bd_two_sum(sr[q], p2, t2);
            bd_two_sum(si[q], p3, t3);
            bd_two_sum(si[q], p4, t4);
            cr[q] += (t1 + t2) + (e1 + e2) + fmaf(a.x, x.z, -a.y * x.w);
            ci[q] += (t3 + t4) + (e3 + e4) + fmaf(a.x, x.w, a.y * x.z);
        }
    }
#pragma unroll
    for (int q = 0; q < NC; ++q) {
        double ar = (double)sr[q] + (double)cr[q], ai = (double)si[q] + (double)ci[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ar += __shfl_xor_sync(0xffffffffu, ar, o);
            ai += __shfl_xor_sync(0xffffffffu, ai, o);
        }
        if (lane == 0) {
            const int64_t c = c0 + q;
            const double2 bv = b[k * m + c];
            const double re = bv.x - ar, im = bv.y - ai;
            r[k * mp + c] = make_float2((float)re, (float)im);
            atomicAdd(sq + c, re * re + im * im);
        }
    }
}

static int bd_residual(const BdPrecond& P, int64_t total_rows, int64_t n, int64_t m, int64_t mp, const double* x,
                       const double* b, float2* v0, double* sq, cudaStream_t s) {
    bd_split_kernel<<<(unsigned)((n * m + 255) / 256), 256, 0, s>>>(reinterpret_cast<const double2*>(x), n * m,
                                                                     reinterpret_cast<float4*>(P.u));
    cudaMemsetAsync(v0, 0, 8 * (size_t)n * mp, s);
    const unsigned blocks = (unsigned)((total_rows + 7) / 8);
    const float4* xs = reinterpret_cast<const float4*>(P.u);
    const double2* b2 = reinterpret_cast<const double2*>(b);
    switch (P.nc) {
        case 1: bd_residual_kernel<1><<<blocks, 256, 0, s>>>(P, total_rows, m, mp, xs, b2, v0, sq); break;
        case 2: bd_residual_kernel<2><<<blocks, 256, 0, s>>>(P, total_rows, m, mp, xs, b2, v0, sq); break;
        case 4: bd_residual_kernel<4><<<blocks, 256, 0, s>>>(P, total_rows, m, mp, xs, b2, v0, sq); break;
        case 8: bd_residual_kernel<8><<<blocks, 256, 0, s>>>(P, total_rows, m, mp, xs, b2, v0, sq); break;
        default: return set_error(MB_ERR_UNSUPPORTED, "preconditioned batch solve: nc must be 1, 2, 4 or 8");
    }
    return check_launch("bd_residual");
}

// z = M v on the padded [n, mp] complex64 layout (FP32); rows beyond E_i and padding columns 0
__global__ void __launch_bounds__(256) bd_precond_kernel(BdPrecond P, int64_t n, int64_t m, int64_t mp,
                                                         const float2* __restrict__ v, float2* __restrict__ z) {
    const int64_t c = (int64_t)blockIdx.x * 32 + (threadIdx.x & 31);
    const int64_t r = (int64_t)blockIdx.y * 8 + (threadIdx.x >> 5);
    if (r >= n || c >= mp) return;
    float sr = 0.f, si = 0.f;
    if (c < m) {
        const int i = (int)(c / P.nc);
        if (r < P.desc[6 * i + 2]) {
            const int64_t g = P.eoff[i] + r;
            for (int q = 0; q < MB_SPAI_WIDTH; ++q) {
                const int32_t col = __ldg(P.cols + g * MB_SPAI_WIDTH + q);
                if (col < 0) break;
                const float2 mq = __ldg(P.vals + g * MB_SPAI_WIDTH + q), x = v[col * mp + c];
                sr = fmaf(mq.x, x.x, fmaf(-mq.y, x.y, sr));
                si = fmaf(mq.x, x.y, fmaf(mq.y, x.x, si));
            }
        }
    }
    z[r * mp + c] = make_float2(sr, si);
}

// x += M u on the [n, m] complex128 layout (FP64)
__global__ void __launch_bounds__(256) bd_update_kernel(BdPrecond P, int64_t n, int64_t m,
                                                        const double2* __restrict__ u, double2* __restrict__ x) {
    const int64_t c = (int64_t)blockIdx.x * 32 + (threadIdx.x & 31);
    const int64_t r = (int64_t)blockIdx.y * 8 + (threadIdx.x >> 5);
    if (r >= n || c >= m) return;
    const int i = (int)(c / P.nc);
    if (r >= P.desc[6 * i + 2]) return;
    const int64_t g = P.eoff[i] + r;
    double sr = 0.0, si = 0.0;
    for (int q = 0; q < MB_SPAI_WIDTH; ++q) {
        const int32_t col = __ldg(P.cols + g * MB_SPAI_WIDTH + q);
        if (col < 0) break;
        const float2 mq = __ldg(P.vals + g * MB_SPAI_WIDTH + q);
        const double2 y = u[col * m + c];
        sr = fma((double)mq.x, y.x, fma(-(double)mq.y, y.y, sr));
        si = fma((double)mq.x, y.y, fma((double)mq.y, y.x, si));
    }
    double2 o = x[r * m + c];
    o.x += sr;
    o.y += si;
    x[r * m + c] = o;
}

// The lockstep driver.  prod(v, y, stream, cact) computes Y = Z V for [n, mp] complex64 blocks
// (cact: the per-column active flags of an Arnoldi step, or null for every column)
// (mp = m rounded up to even; the padding column has b = 0 and stays inactive).
// desc / nc (optional): block-diagonal layout, column c of mesh c / nc has desc[.][2] rows.
// With use_graph, the r Arnoldi steps of a cycle are captured once as a CUDA graph and
// replayed every cycle (no host synchronisation inside a cycle; a cycle always runs its r
// steps, columns that converged early are inactive).
// pc (optional): right preconditioner of the block-diagonal systems (see BdPrecond).
// ---- augmentation subspace (deflation) ---------------------------------------------------
// Per mesh i a fixed subspace U_i of K vectors of x-space (K in {4, 8, 16}) enters every
// cycle.  The caller factors C_i = Z_i U_i = Q_i R_i (thin QR) and passes Q_i and
// Ut_i = U_i R_i^{-1} (so Z_i Ut_i = Q_i), complex64 [n_rows, ld] with mesh i's K columns at
// i K and zero rows beyond E_i.  The Arnoldi operator becomes (I - Q Q^H) Z M: step j keeps
// b_j = Q^H Z M v_j (K values per column) and removes Q b_j from the product; a cycle start
// adds Ut Q^H r to X and removes Q Q^H r from r (at the first cycle: the residual-minimising
// combination of U, the initial guess); a cycle's update is X += M V y - Ut (B y), so the
// minimised residual is again the true one (GCRO with a fixed recycled space).
constexpr int kAugChunks = 64;

struct AugSpace {
    const float2* q;
    const float2* ut;
    int64_t ld;      // row pitch of q and ut (complex entries)
    int k;           // vectors per mesh
    int nc;          // columns per mesh
    double2* part;   // [kAugChunks][mp][k] chunk partials of Q^H y
    double2* bq;     // [r][mp][k] b_j of the cycle's steps
    double2* coef;   // [mp][k]
};

// part[chunk][c][q] = sum over the chunk's rows of conj(Q[row, mesh(c) K + q]) src[row, c]
template <int K>
__global__ void __launch_bounds__(128) aug_coef_kernel(AugSpace A, const float2* __restrict__ src,
                                                       const int* __restrict__ crow, int64_t n, int64_t m,
                                                       int64_t mp) {
    const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (c >= m) return;
    const int64_t nr = rows_of(crow, c, n);
    const int64_t rpc = (n + kAugChunks - 1) / kAugChunks;
    const int64_t k0 = (int64_t)blockIdx.y * rpc, k1 = k0 + rpc < nr ? k0 + rpc : nr;
    const float2* qc = A.q + (c / A.nc) * K;
    float ar[K], ai[K];
#pragma unroll
    for (int q = 0; q < K; ++q) { ar[q] = 0.f; ai[q] = 0.f; }
    for (int64_t k = k0; k < k1; ++k) {
        const float2 v = src[k * mp + c];
        const float2* qk = qc + k * A.ld;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const float2 w = __ldg(qk + q);
            ar[q] = fmaf(w.x, v.x, fmaf(w.y, v.y, ar[q]));
            ai[q] = fmaf(w.x, v.y, fmaf(-w.y, v.x, ai[q]));
        }
    }
    double2* p = A.part + ((int64_t)blockIdx.y * mp + c) * K;
#pragma unroll
    for (int q = 0; q < K; ++q) p[q] = make_double2(ar[q], ai[q]);
}

// dst[c][q] = sum of the chunk partials in chunk order (columns c >= m get 0)
__global__ void aug_reduce_kernel(AugSpace A, int64_t m, int64_t mp, double2* __restrict__ dst) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= mp * A.k) return;
    double sr = 0.0, si = 0.0;
    if (t / A.k < m) {
        for (int ch = 0; ch < kAugChunks; ++ch) {
            const double2 v = A.part[(int64_t)ch * mp * A.k + t];
            sr += v.x;
            si += v.y;
        }
    }
    dst[t] = make_double2(sr, si);
}

// y[row, c] -= sum_q Q[row, mesh(c) K + q] coef[c][q] (complex64 y [n, mp])
template <int K>
__global__ void __launch_bounds__(128) aug_sub_kernel(AugSpace A, const double2* __restrict__ coef,
                                                      const int* __restrict__ crow, int64_t n, int64_t m, int64_t mp,
                                                      float2* __restrict__ y) {
    const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (c >= m) return;
    const int64_t nr = rows_of(crow, c, n);
    const int64_t rpc = (n + gridDim.y - 1) / gridDim.y;
    const int64_t k0 = (int64_t)blockIdx.y * rpc, k1 = k0 + rpc < nr ? k0 + rpc : nr;
    float cr[K], ci[K];
#pragma unroll
    for (int q = 0; q < K; ++q) {
        const double2 v = coef[c * K + q];
        cr[q] = (float)v.x;
        ci[q] = (float)v.y;
    }
    const float2* qc = A.q + (c / A.nc) * K;
    for (int64_t k = k0; k < k1; ++k) {
        const float2* qk = qc + k * A.ld;
        float sr = 0.f, si = 0.f;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const float2 w = __ldg(qk + q);
            sr = fmaf(w.x, cr[q], fmaf(-w.y, ci[q], sr));
            si = fmaf(w.x, ci[q], fmaf(w.y, cr[q], si));
        }
        float2 v = y[k * mp + c];
        v.x -= sr;
        v.y -= si;
        y[k * mp + c] = v;
    }
}

// x[row, c] += sgn sum_q Ut[row, mesh(c) K + q] coef[c][q] in FP64 (complex128 x [n, m])
template <int K>
__global__ void __launch_bounds__(128) aug_x_kernel(AugSpace A, const double2* __restrict__ coef, double sgn,
                                                    const int* __restrict__ crow, int64_t n, int64_t m,
                                                    double2* __restrict__ x) {
    const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (c >= m) return;
    const int64_t nr = rows_of(crow, c, n);
    const int64_t rpc = (n + gridDim.y - 1) / gridDim.y;
    const int64_t k0 = (int64_t)blockIdx.y * rpc, k1 = k0 + rpc < nr ? k0 + rpc : nr;
    double cr[K], ci[K];
#pragma unroll
    for (int q = 0; q < K; ++q) {
        const double2 v = coef[c * K + q];
        cr[q] = sgn * v.x;
        ci[q] = sgn * v.y;
    }
    const float2* uc = A.ut + (c / A.nc) * K;
    for (int64_t k = k0; k < k1; ++k) {
        const float2* uk = uc + k * A.ld;
        double sr = 0.0, si = 0.0;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const float2 w = __ldg(uk + q);
            sr += (double)w.x * cr[q] - (double)w.y * ci[q];
            si += (double)w.x * ci[q] + (double)w.y * cr[q];
        }
        double2 v = x[k * m + c];
        v.x += sr;
        v.y += si;
        x[k * m + c] = v;
    }
}

// coef[c][q] = sum_{j < r} bq[j][c][q] yv[j][c]  (yv is zero beyond the column's last step)
__global__ void aug_by_kernel(AugSpace A, const double* __restrict__ yv, int r, int64_t m, int64_t mp) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= mp * A.k) return;
    const int64_t c = t / A.k;
    double sr = 0.0, si = 0.0;
    if (c < m) {
        for (int j = 0; j < r; ++j) {
            const double2 bv = A.bq[(int64_t)j * mp * A.k + t];
            const double yr = yv[2 * ((int64_t)j * mp + c)], yi = yv[2 * ((int64_t)j * mp + c) + 1];
            sr += bv.x * yr - bv.y * yi;
            si += bv.x * yi + bv.y * yr;
        }
    }
    A.coef[t] = make_double2(sr, si);
}

// sq[c] = sum_rows |v[row, c]|^2 (FP64), complex64 v [n, mp]
__global__ void aug_colnorm2_kernel(const float2* __restrict__ v, int64_t n, int64_t m, int64_t mp,
                                    double* __restrict__ sq) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m) return;
    double a = 0.0;
    for (int64_t k = 0; k < n; ++k) {
        const float2 w = v[k * mp + c];
        a += (double)w.x * w.x + (double)w.y * w.y;
    }
    sq[c] = a;
}

// Q^H src into dst (via the chunk partials), then src -= Q dst
static int aug_project(const AugSpace& A, float2* src, const int* crow, int64_t n, int64_t m, int64_t mp,
                       double2* dst, cudaStream_t s) {
    const unsigned cbk = (unsigned)((m + 127) / 128);
    const dim3 g(cbk, kAugChunks);
    const unsigned rb = (unsigned)((mp * A.k + 255) / 256);
    const dim3 gs(cbk, (unsigned)std::max<int64_t>(1, std::min<int64_t>(n, 256)));
    switch (A.k) {
        case 4: aug_coef_kernel<4><<<g, 128, 0, s>>>(A, src, crow, n, m, mp); break;
        case 8: aug_coef_kernel<8><<<g, 128, 0, s>>>(A, src, crow, n, m, mp); break;
        default: aug_coef_kernel<16><<<g, 128, 0, s>>>(A, src, crow, n, m, mp); break;
    }
    aug_reduce_kernel<<<rb, 256, 0, s>>>(A, m, mp, dst);
    switch (A.k) {
        case 4: aug_sub_kernel<4><<<gs, 128, 0, s>>>(A, dst, crow, n, m, mp, src); break;
        case 8: aug_sub_kernel<8><<<gs, 128, 0, s>>>(A, dst, crow, n, m, mp, src); break;
        default: aug_sub_kernel<16><<<gs, 128, 0, s>>>(A, dst, crow, n, m, mp, src); break;
    }
    return check_launch("gmres_blockdiag augmentation projection");
}

static int aug_update_x(const AugSpace& A, const double2* coef, double sgn, const int* crow, int64_t n, int64_t m,
                        double* x, cudaStream_t s) {
    const dim3 gs((unsigned)((m + 127) / 128), (unsigned)std::max<int64_t>(1, std::min<int64_t>(n, 256)));
    double2* xd = reinterpret_cast<double2*>(x);
    switch (A.k) {
        case 4: aug_x_kernel<4><<<gs, 128, 0, s>>>(A, coef, sgn, crow, n, m, xd); break;
        case 8: aug_x_kernel<8><<<gs, 128, 0, s>>>(A, coef, sgn, crow, n, m, xd); break;
        default: aug_x_kernel<16><<<gs, 128, 0, s>>>(A, coef, sgn, crow, n, m, xd); break;
    }
    return check_launch("gmres_blockdiag augmentation update");
}

template <typename Prod>
static int gmres_lockstep(Prod prod, int64_t n, const double* b, double* x, int64_t m, int r, int max_iters,
                          double tol, size_t prod_ws, const int64_t* desc, int nc, void* workspace, size_t ws_bytes,
                          bool use_graph, int64_t* iters_out, int64_t* cycles_out, double* max_relres_out,
                          int* status_out, cudaStream_t s, const BdPrecond* pc = nullptr,
                          const AugSpace* aug = nullptr) {
    if (n <= 0 || m <= 0) return set_error(MB_ERR_ARG, "n and m must be > 0");
    if (((uintptr_t)x | (uintptr_t)b) & 15) return set_error(MB_ERR_ARG, "b and x must be 16-byte aligned");
    if (r < 1 || r > kMgMaxRestart) return set_error(MB_ERR_ARG, "restart must be in [1, %d]", kMgMaxRestart);
    if (max_iters < 1 || !(tol > 0)) return set_error(MB_ERR_ARG, "bad max_iters / tol");
    if (n > (1ll << 30)) return set_error(MB_ERR_SIZE, "gmres: too many rows");
    const int64_t mp = padded_width(m);
    MgWork W;
    if (ws_bytes < mg_layout(n, mp, r, prod_ws, nullptr, &W)) return set_error(MB_ERR_ARG, "workspace too small");
    mg_layout(n, mp, r, prod_ws, workspace, &W);
    const int64_t nm = n * mp;
    const unsigned cb = (unsigned)((mp + 31) / 32);  // per-column FP64 kernels: one warp per block
    const unsigned colb = (unsigned)((mp + 31) / 32);
    const dim3 rblk(32, 8);
    int sms = 152;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    // row blocks per column group for the reductions: enough blocks to fill the GPU
    const unsigned ky = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 63) / 64, (sms * 16 + colb - 1) / colb));
    const dim3 rgrid(colb, ky);
    // streamed Gram-Schmidt: tensor maps and persistent grids (as many blocks as stay resident)
    constexpr int kS = 4;
    auto dots_k = mg_dots<kS>;
    auto comb_k = mg_combine<kS, 0>;
    auto combn_k = mg_combine<kS, 1>;
    auto upd_k = mg_combine<kS, 2>;
    GsMaps maps_y, maps_w;
    int rc;
    if ((rc = gs_maps(&maps_y, W.V, W.y32, n, mp, r)) || (rc = gs_maps(&maps_w, W.V, W.w, n, mp, r))) return rc;
    const size_t dots_max = gs_smem<kS>((size_t)(r + 1) * 32 * 16), comb_max = gs_smem<kS>((size_t)(r + 1) * 32 * 8);
    cudaFuncSetAttribute(dots_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dots_max);
    for (auto k : {comb_k, combn_k, upd_k})
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)comb_max);
    cudaFuncSetAttribute(mg_backsolve, cudaFuncAttributeMaxDynamicSharedMemorySize, r * 32 * 16);
    int dots_per_sm = 0, comb_per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dots_per_sm, dots_k, kGsThreads, dots_max);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&comb_per_sm, combn_k, kGsThreads, comb_max);
    const int64_t tiles = (n + kGsRows - 1) / kGsRows;
    const dim3 dgrid(colb, (unsigned)std::max<int64_t>(
                               1, std::min<int64_t>(tiles, ((int64_t)std::max(dots_per_sm, 1) * sms) / colb)));
    const dim3 cgrid(colb, (unsigned)std::max<int64_t>(
                               1, std::min<int64_t>(tiles, ((int64_t)std::max(comb_per_sm, 1) * sms) / colb)));
    const int* crow = nullptr;
    if (desc) {
        if (nc < 1 || m % nc) return set_error(MB_ERR_ARG, "gmres: m must be a multiple of nc");
        mg_column_rows<<<cb, 32, 0, s>>>(desc, m, mp, nc, W.crow);
        crow = W.crow;
    }
    if (aug && !crow) return set_error(MB_ERR_ARG, "gmres: an augmentation subspace needs the batch descriptor");
    int64_t pc_rows = 0;  // sum of E_i (the preconditioned block-diagonal residual's rows)
    if (pc) {
        std::vector<int64_t> dh((size_t)6 * pc->n_mesh);
        cudaMemcpyAsync(dh.data(), pc->desc, 48 * (size_t)pc->n_mesh, cudaMemcpyDeviceToHost, s);
        if ((rc = mg_sync(s, "gmres_blockdiag descriptor"))) return rc;
        for (int i = 0; i < pc->n_mesh; ++i) pc_rows += dh[(size_t)6 * i + 2];
    }
    std::vector<double> hb(mp);
    cudaMemsetAsync(W.y32, 0, 8 * (size_t)nm, s);  // rows a product does not write stay 0
    cudaMemsetAsync(W.bnorm, 0, 8 * mp, s);
    cudaMemsetAsync(W.status, 0, 16, s);
    cudaMemsetAsync(W.colsteps, 0, 4 * mp, s);
    mg_colnorm2<<<rgrid, rblk, 0, s>>>(reinterpret_cast<const double2*>(b), n, m, W.bnorm);
    cudaMemcpyAsync(hb.data(), W.bnorm, 8 * mp, cudaMemcpyDeviceToHost, s);
    if ((rc = mg_sync(s, "gmres_multi |b|"))) return rc;
    for (auto& v : hb) v = v > 0 ? std::sqrt(v) : 1.0;
    cudaMemcpyAsync(W.bnorm, hb.data(), 8 * mp, cudaMemcpyHostToDevice, s);
    int64_t iters = 0, cycles = 0;
    double worst = 0.0;
    int status = 1;
    std::vector<double> hbeta(mp);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;  // capture needs a stream other than the legacy default stream
    auto step = [&](int j, cudaStream_t st) -> int {
        int e;
        const int nb = j + 1;
        const size_t dsm = gs_smem<kS>((size_t)nb * 32 * 16), csm = gs_smem<kS>((size_t)nb * 32 * 8);
        const float2* vj = W.V + (size_t)j * nm;
        if (pc) {
            bd_precond_kernel<<<dim3((unsigned)((mp + 31) / 32), (unsigned)((n + 7) / 8)), 256, 0, st>>>(
                *pc, n, m, mp, vj, pc->z32);
            vj = pc->z32;
        }
        // an Arnoldi step's product skips the meshes none of whose columns is still iterating
        if ((e = prod(reinterpret_cast<const float*>(vj), reinterpret_cast<float*>(W.y32), st, W.active))) return e;
        if (aug && (e = aug_project(*aug, W.y32, crow, n, m, mp, aug->bq + (size_t)j * mp * aug->k, st))) return e;
        // CGS2: pass 1 projects the product output y into w, pass 2 re-orthogonalises w and
        // accumulates |w|^2
        cudaMemsetAsync(W.hc, 0, 16 * (size_t)nb * mp, st);
        dots_k<<<dgrid, kGsThreads, dsm, st>>>(maps_y, W.y32, n, mp, nb, W.hc, W.status);
        comb_k<<<cgrid, kGsThreads, csm, st>>>(maps_y, W.hc, n, mp, mp, nb, -1.f, W.w, nullptr, W.status);
        mg_accum_h<<<(unsigned)((nb * mp + 255) / 256), 256, 0, st>>>(W.hc, nb, j, r, mp, W.H);
        cudaMemsetAsync(W.hc, 0, 16 * (size_t)nb * mp, st);
        dots_k<<<dgrid, kGsThreads, dsm, st>>>(maps_w, W.w, n, mp, nb, W.hc, W.status);
        cudaMemsetAsync(W.hn, 0, 8 * mp, st);
        combn_k<<<cgrid, kGsThreads, csm, st>>>(maps_w, W.hc, n, mp, mp, nb, -1.f, W.w, W.hn, W.status);
        mg_accum_h<<<(unsigned)((nb * mp + 255) / 256), 256, 0, st>>>(W.hc, nb, j, r, mp, W.H);
        cudaMemsetAsync(W.count, 0, 4, st);
        mg_givens<<<cb, 32, 0, st>>>(W.H, W.cs, W.sn, W.g, W.hn, W.bnorm, j, r, mp, tol, W.active, W.jend, W.count,
                                     W.scale, W.colsteps);
        mg_scale_cols<<<rgrid, rblk, 0, st>>>(W.w, W.scale, crow, n, mp, W.V + (size_t)(j + 1) * nm);
        return check_launch("gmres_multi step");
    };
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
    };
    auto check_status = [&]() -> int {
        int hs = 0;
        cudaMemcpyAsync(&hs, W.status, 4, cudaMemcpyDeviceToHost, s);
        int e = mg_sync(s, "gmres_multi status");
        if (e) return e;
        if (hs) return set_error(MB_ERR_CUDA, "gmres_multi: streamed kernel wait timed out (code %d)", hs);
        return MB_OK;
    };
    while (true) {
        // residual of the current iterate through the same product (w holds complex64 X)
        if (pc) {  // compensated refinement residual of the block-diagonal systems
            cudaMemsetAsync(W.beta, 0, 8 * mp, s);
            if ((rc = bd_residual(*pc, pc_rows, n, m, mp, x, b, W.V, W.beta, s))) return cleanup(), rc;
        } else {
            mg_to_c64<<<rgrid, rblk, 0, s>>>(reinterpret_cast<const double2*>(x), n, m, mp, W.w);
            if ((rc = prod(reinterpret_cast<const float*>(W.w), reinterpret_cast<float*>(W.y32), s, nullptr)))
                return cleanup(), rc;
            cudaMemsetAsync(W.beta, 0, 8 * mp, s);
            mg_residual<<<rgrid, rblk, 0, s>>>(reinterpret_cast<const double2*>(b), W.y32, n, m, mp, W.V, W.beta);
        }
        if (aug) {  // X += Ut Q^H r, r -= Q Q^H r, then |r|^2 again
            if ((rc = aug_project(*aug, W.V, crow, n, m, mp, aug->coef, s)) ||
                (rc = aug_update_x(*aug, aug->coef, 1.0, crow, n, m, x, s)))
                return cleanup(), rc;
            aug_colnorm2_kernel<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(W.V, n, m, mp, W.beta);
        }
        cudaMemcpyAsync(hbeta.data(), W.beta, 8 * mp, cudaMemcpyDeviceToHost, s);
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
        mg_init_g<<<cb, 32, 0, s>>>(W.beta, W.bnorm, r, mp, tol, W.g, W.jend, W.count, W.active, W.scale);
        mg_scale_cols<<<rgrid, rblk, 0, s>>>(W.V, W.scale, crow, n, mp, W.V);
        cudaMemsetAsync(W.H, 0, 16 * (size_t)(r + 1) * r * mp, s);
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
        mg_backsolve<<<cb, 32, (size_t)r * 32 * 16, s>>>(W.H, W.g, W.jend, r, mp, W.yv);
        if (j > 0 && pc) {
            cudaMemsetAsync(pc->u, 0, 16 * (size_t)n * m, s);
            upd_k<<<cgrid, kGsThreads, gs_smem<kS>((size_t)j * 32 * 8), s>>>(maps_w, W.yv, n, mp, m, j, 1.f, pc->u,
                                                                           nullptr, W.status);
            bd_update_kernel<<<dim3((unsigned)((m + 31) / 32), (unsigned)((n + 7) / 8)), 256, 0, s>>>(
                *pc, n, m, pc->u, reinterpret_cast<double2*>(x));
        } else if (j > 0) {
            upd_k<<<cgrid, kGsThreads, gs_smem<kS>((size_t)j * 32 * 8), s>>>(maps_w, W.yv, n, mp, m, j, 1.f, x,
                                                                           nullptr, W.status);
        }
        if (j > 0 && aug) {  // X -= Ut (B y)
            aug_by_kernel<<<(unsigned)((mp * aug->k + 255) / 256), 256, 0, s>>>(*aug, W.yv, j, m, mp);
            if ((rc = aug_update_x(*aug, aug->coef, -1.0, crow, n, m, x, s))) return cleanup(), rc;
        }
        if ((rc = check_status())) return cleanup(), rc;
    }
    cleanup();
    if (iters_out) *iters_out = iters;
    if (cycles_out) *cycles_out = cycles;
    if (max_relres_out) *max_relres_out = worst;
    if (status_out) *status_out = status;
    return MB_OK;
}

// Per-column Arnoldi step counts of the last solve that used `workspace` (int32 [m], to a
// device or host pointer).
static int column_steps(const void* workspace, int64_t n, int64_t m, int r, size_t prod_ws, int32_t* out,
                        cudaStream_t s) {
    MgWork W;
    mg_layout(n, padded_width(m), r, prod_ws, const_cast<void*>(workspace), &W);
    const cudaError_t e = cudaMemcpyAsync(out, W.colsteps, 4 * (size_t)m, cudaMemcpyDefault, s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "column steps: %s", cudaGetErrorString(e));
    return MB_OK;
}
int gmres_multi_column_steps(const void* ws, int64_t n, int64_t m, int r, int32_t* out, cudaStream_t s) {
    return column_steps(ws, n, m, r, cgemm_workspace_bytes(n, padded_width(m)), out, s);
}
int gmres_blockdiag_column_steps(const void* ws, int64_t n, int64_t m, int r, int32_t* out, cudaStream_t s) {
    return column_steps(ws, n, m, r, bd_prod_bytes(n, m), out, s);
}

int gmres_multi(const float* z_hi, const float* z_lo, int64_t n, const double* b, double* x, int64_t m, int r,
                int max_iters, double tol, void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out,
                double* max_relres_out, int* status_out, cudaStream_t s) {
    const int64_t mp = padded_width(m);
    const size_t gws = cgemm_workspace_bytes(n, mp);
    MgWork W;
    if (ws_bytes < mg_layout(n, mp, r, gws, nullptr, &W)) return set_error(MB_ERR_ARG, "workspace too small");
    mg_layout(n, mp, r, gws, workspace, &W);
    void* gemm_ws = W.gemm_ws;
    auto prod = [&](const float* v32, float* y32, cudaStream_t st, const int*) {
        return cgemm_tf32x3(z_hi, z_lo, n, v32, mp, y32, gemm_ws, gws, st);
    };
    return gmres_lockstep(prod, n, b, x, m, r, max_iters, tol, gws, nullptr, 1, workspace, ws_bytes, false,
                          iters_out, cycles_out, max_relres_out, status_out, s);
}

// Many meshes, each with its own Z_i and nc right-hand sides: the block-diagonal system on
// the padded [n_rows, m] layout (m = n_mesh * nc columns).
static int blockdiag_solve(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                           int rows_per_warp, int nc, int64_t n_rows, const double* b, double* x, int r,
                           int max_iters, double tol, bool use_graph, void* workspace, size_t ws_bytes,
                           int64_t* iters_out, int64_t* cycles_out, double* max_relres_out, int* status_out,
                           cudaStream_t s, const int32_t* m_cols, const float* m_vals, const int64_t* eoff,
                           const float* aug_q = nullptr, const float* aug_ut = nullptr, int aug_k = 0) {
    const int64_t m = (int64_t)n_mesh * nc, mp = padded_width(m);
    MgWork W;
    const size_t map_bytes = bd_prod_bytes(n_rows, m);  // tensor maps (>= n_mesh) + preconditioner buffers
    if (ws_bytes < mg_layout(n_rows, mp, r, map_bytes, nullptr, &W)) return set_error(MB_ERR_ARG, "workspace too small");
    mg_layout(n_rows, mp, r, map_bytes, workspace, &W);
    BdPrecond pc{};
    if (m_cols) {
        char* q = static_cast<char*>(W.gemm_ws) + bd_maps_bytes(m);
        pc = BdPrecond{m_cols, reinterpret_cast<const float2*>(m_vals), desc, eoff, n_mesh, nc,
                       reinterpret_cast<const float2*>(z), reinterpret_cast<float2*>(q),
                       reinterpret_cast<double2*>(q + a256(8 * (size_t)n_rows * mp))};
    }
    int* status = W.status;
    const CUtensorMap* zmaps = static_cast<const CUtensorMap*>(W.gemm_ws);
    if (rows_per_warp == kBdRows) {
        if (reinterpret_cast<uintptr_t>(z) & 15) return set_error(MB_ERR_ARG, "z must be 16-byte aligned");
        std::vector<int64_t> dh((size_t)6 * n_mesh);
        cudaMemcpyAsync(dh.data(), desc, 48 * (size_t)n_mesh, cudaMemcpyDeviceToHost, s);
        int rc = bd_zmaps(z, dh.data(), n_mesh, static_cast<CUtensorMap*>(W.gemm_ws), s);
        if (rc) return rc;
    }
    auto prod = [&](const float* v32, float* y32, cudaStream_t st, const int* cact) {
        if (rows_per_warp == kBdRows)
            return bd_launch(zmaps, v32, n_rows, desc, goff, n_mesh, total_warps, mp, nc, y32, status, st, cact);
        return blockdiag_matvec(z, desc, goff, n_mesh, total_warps, v32, mp, nc, rows_per_warp, y32, st, cact);
    };
    if (!aug_q)
        return gmres_lockstep(prod, n_rows, b, x, m, r, max_iters, tol, map_bytes, desc, nc, workspace, ws_bytes,
                              use_graph, iters_out, cycles_out, max_relres_out, status_out, s, m_cols ? &pc : nullptr);
    if (r < 1 || r > kMgMaxRestart) return set_error(MB_ERR_ARG, "restart must be in [1, %d]", kMgMaxRestart);
    // the subspace's coefficients: chunk partials, the cycle's b_j and one scratch set
    const size_t per = (size_t)mp * aug_k * sizeof(double2);
    char* abuf = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void**>(&abuf), per * (kAugChunks + r + 1), s) != cudaSuccess) {
        cudaGetLastError();
        return set_error(MB_ERR_CUDA, "gmres_blockdiag: augmentation buffers could not be allocated");
    }
    AugSpace A{reinterpret_cast<const float2*>(aug_q), reinterpret_cast<const float2*>(aug_ut), (int64_t)n_mesh * aug_k,
               aug_k, nc, reinterpret_cast<double2*>(abuf), reinterpret_cast<double2*>(abuf + per * kAugChunks),
               reinterpret_cast<double2*>(abuf + per * (kAugChunks + r))};
    const int rc = gmres_lockstep(prod, n_rows, b, x, m, r, max_iters, tol, map_bytes, desc, nc, workspace, ws_bytes,
                                  use_graph, iters_out, cycles_out, max_relres_out, status_out, s,
                                  m_cols ? &pc : nullptr, &A);
    cudaFreeAsync(abuf, s);
    return rc;
}

int gmres_blockdiag(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                    int rows_per_warp, int nc, int64_t n_rows, const double* b, double* x, int r, int max_iters,
                    double tol, bool use_graph, void* workspace, size_t ws_bytes, int64_t* iters_out,
                    int64_t* cycles_out, double* max_relres_out, int* status_out, cudaStream_t s) {
    return blockdiag_solve(z, desc, goff, n_mesh, total_warps, rows_per_warp, nc, n_rows, b, x, r, max_iters, tol,
                           use_graph, workspace, ws_bytes, iters_out, cycles_out, max_relres_out, status_out, s,
                           nullptr, nullptr, nullptr);
}

int gmres_blockdiag_pc(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                       int rows_per_warp, int nc, int64_t n_rows, const int32_t* m_cols, const float* m_vals,
                       const int64_t* eoff, const double* b, double* x, int r, int max_iters, double tol,
                       bool use_graph, void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out,
                       double* max_relres_out, int* status_out, cudaStream_t s) {
    if (!m_cols || !m_vals || !eoff) return set_error(MB_ERR_ARG, "gmres_blockdiag_pc: null preconditioner");
    return blockdiag_solve(z, desc, goff, n_mesh, total_warps, rows_per_warp, nc, n_rows, b, x, r, max_iters, tol,
                           use_graph, workspace, ws_bytes, iters_out, cycles_out, max_relres_out, status_out, s, m_cols,
                           m_vals, eoff);
}

int gmres_blockdiag_aug(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                        int rows_per_warp, int nc, int64_t n_rows, const int32_t* m_cols, const float* m_vals,
                        const int64_t* eoff, const float* aug_q, const float* aug_ut, int aug_k, const double* b,
                        double* x, int r, int max_iters, double tol, bool use_graph, void* workspace, size_t ws_bytes,
                        int64_t* iters_out, int64_t* cycles_out, double* max_relres_out, int* status_out,
                        cudaStream_t s) {
    if (!aug_q || !aug_ut) return set_error(MB_ERR_ARG, "gmres_blockdiag_aug: null subspace");
    if (aug_k != 4 && aug_k != 8 && aug_k != 16) return set_error(MB_ERR_UNSUPPORTED, "subspace size must be 4, 8 or 16");
    if ((m_cols != nullptr) != (m_vals != nullptr) || (m_cols != nullptr) != (eoff != nullptr))
        return set_error(MB_ERR_ARG, "gmres_blockdiag_aug: give all of m_cols, m_vals, edge_offsets or none");
    return blockdiag_solve(z, desc, goff, n_mesh, total_warps, rows_per_warp, nc, n_rows, b, x, r, max_iters, tol,
                           use_graph, workspace, ws_bytes, iters_out, cycles_out, max_relres_out, status_out, s, m_cols,
                           m_vals, eoff, aug_q, aug_ut, aug_k);
}

}  // namespace mb
