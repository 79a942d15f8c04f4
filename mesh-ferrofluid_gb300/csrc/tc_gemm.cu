// tc_gemm.cu -- complex multi-right-hand-side product Y = Z X on the 5th-generation tensor
// cores (tcgen05, kind::tf32) with the split-TF32 x 3 scheme, FP32 accumulation in TMEM.
//
// Real form: Z complex64 [E, E] is read as the real matrix A [E, 2E] (interleaved re/im),
// X complex64 [E, m] becomes Bt [2m, 2E] with
//     Bt[2j][2k] = Re X[k][j],  Bt[2j][2k+1] = -Im X[k][j],
//     Bt[2j+1][2k] = Im X[k][j], Bt[2j+1][2k+1] = Re X[k][j],
// so D = A Bt^T [E, 2m] is Y complex64 [E, m] (8 E^2 m real FLOP per product).
// Split: a = a_hi + a_lo with a_hi = a rounded to TF32 (10-bit mantissa) and a_lo = a - a_hi;
// D = A_hi B_hi + A_hi B_lo + A_lo B_hi (the dropped A_lo B_lo is ~2^-22 relative), which
// keeps FP32-class accuracy on TF32 tensor cores.
//
// Kernel: one CTA per 128 x 256 output tile; one thread issues the TMA loads of the four
// K-major tiles (A_hi, A_lo 128 x 32, B_hi, B_lo 256 x 32 fp32, 128-byte swizzle) into a
// 2-stage ring (96 KB per stage), one thread issues 12 tcgen05.mma (3 products x 4 K steps
// of 8) per stage into one of two 128 x 256 fp32 TMEM accumulators and commits each stage
// back to the producer; every 4 stages the accumulators swap and eight warps add the
// finished one into FP32 registers (round to nearest) -- see tc_gemm_tf32x3_kernel.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "tc_common.cuh"

namespace mb {

using namespace tc;

constexpr int kTcBM = 128, kTcBN = 256, kTcBK = 32, kTcStages = 2;
constexpr uint32_t kTileA = kTcBM * kTcBK * 4;  // 16 KB
constexpr uint32_t kTileB = kTcBN * kTcBK * 4;  // 32 KB
constexpr uint32_t kStageBytes = 2 * kTileA + 2 * kTileB;
constexpr uint32_t kTcSmem = kTcStages * kStageBytes + 1024 /*alignment slack*/ + 256 /*barriers*/;
constexpr long long kWaitBudget = 4000000000LL;  // SM clocks (~2 s at 2 GHz)

enum TcStatus { kTcTimeoutFull = 1, kTcTimeoutEmpty = 2, kTcTimeoutDone = 4 };

// ---------------------------------------------------------------------------------------
// self-test: one 128 x 256 x 32 tile, operands staged by plain stores in the swizzled layout
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) tc_selftest_kernel(const float* __restrict__ a, const float* __restrict__ b,
                                                          float* __restrict__ d, int* __restrict__ status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~uintptr_t(1023));
    float* sa = reinterpret_cast<float*>(base);
    float* sb = reinterpret_cast<float*>(base + kTileA);
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + kTileA + kTileB);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(base + kTileA + kTileB + 64);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    for (int e = t; e < kTcBM * kTcBK; e += 128) {
        const int r = e / kTcBK, k = e % kTcBK;
        *reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(sa) + sw128_offset(r, k)) = a[e];
    }
    for (int e = t; e < kTcBN * kTcBK; e += 128) {
        const int r = e / kTcBK, k = e % kTcBK;
        *reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(sb) + sw128_offset(r, k)) = b[e];
    }
    if (t == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    fence_proxy_async_smem();
    if (warp == 0) tmem_alloc(tslot, 256);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tslot;
    if (t == 0) {
        const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
        for (int k = 0; k < kTcBK / 8; ++k)
            mma_tf32(taddr, sw128_kmajor_desc(a0 + 32 * k), sw128_kmajor_desc(b0 + 32 * k), idesc_tf32(kTcBM, kTcBN),
                     k > 0);
        mma_commit(bar);
    }
    // every lane of a warp takes the same branch before the warp-collective TMEM loads
    const bool ok = __all_sync(0xffffffffu, mbar_wait(bar, 0, kWaitBudget, status, kTcTimeoutDone));
    tc_fence_after();
    if (ok) {
        const int row = 32 * warp + lane;
        for (int c = 0; c < kTcBN; c += 16) {
            float v[16];
            tmem_ld16(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) d[row * kTcBN + c + i] = v[i];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(taddr, 256);
}

// ---------------------------------------------------------------------------------------
// split and operand preparation
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__global__ void split_tf32_kernel(const float* __restrict__ src, int64_t count, float* __restrict__ hi,
                                  float* __restrict__ lo) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const float x = src[i];
        const float h = to_tf32(x);
        hi[i] = h;
        lo[i] = to_tf32(x - h);
    }
}

// X complex64 [n, m] -> Bt_hi, Bt_lo [2m, 2n] (layout in the file header), through a 32 x 32
// shared-memory transpose so both the reads of X and the writes of Bt are coalesced.
__global__ void build_bt_kernel(const float* __restrict__ x, int64_t n, int64_t m, float* __restrict__ bt_hi,
                                float* __restrict__ bt_lo) {
    __shared__ float2 tile[32][33];
    const int64_t k0 = (int64_t)blockIdx.y * 32, j0 = (int64_t)blockIdx.x * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t k = k0 + r, j = j0 + threadIdx.x;
        float2 v = make_float2(0.f, 0.f);
        if (k < n && j < m) v = reinterpret_cast<const float2*>(x)[k * m + j];
        tile[r][threadIdx.x] = v;
    }
    __syncthreads();
    const int64_t ld = 2 * n;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t j = j0 + r, k = k0 + threadIdx.x;
        if (j >= m || k >= n) continue;
        const float2 v = tile[threadIdx.x][r];
        const float rh = to_tf32(v.x), rl = to_tf32(v.x - rh);
        const float ih = to_tf32(v.y), il = to_tf32(v.y - ih);
        float2* h0 = reinterpret_cast<float2*>(bt_hi + (2 * j) * ld + 2 * k);
        float2* h1 = reinterpret_cast<float2*>(bt_hi + (2 * j + 1) * ld + 2 * k);
        float2* l0 = reinterpret_cast<float2*>(bt_lo + (2 * j) * ld + 2 * k);
        float2* l1 = reinterpret_cast<float2*>(bt_lo + (2 * j + 1) * ld + 2 * k);
        *h0 = make_float2(rh, -ih);
        *h1 = make_float2(ih, rh);
        *l0 = make_float2(rl, -il);
        *l1 = make_float2(il, rl);
    }
}

// ---------------------------------------------------------------------------------------
// the GEMM: D [M, N] = A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T, A [M, K], B [N, K] K-major
// ---------------------------------------------------------------------------------------
struct TcMaps {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;
};

// Warp roles (320 threads): warps 0-7 drain the accumulator and write the tile (warp w owns
// TMEM lanes 32 (w % 4) .. +31 and columns 128 (w / 4) .. +127), warp 8 lane 0 issues the
// TMA loads, warp 9 allocates TMEM (512 columns: two 256-column accumulators) and its lane 0
// issues the MMAs.  The tensor core rounds toward zero when it adds into the accumulator, a
// bias that grows with the number of accumulations; so every kTcChunk K-blocks the MMA warp
// switches accumulator and the drain warps add the finished one into FP32 registers with
// round-to-nearest, overlapped with the MMAs of the next chunk.
constexpr int kTcChunk = 4;
constexpr int kTcDrainWarps = 8;
constexpr int kTcThreads = 32 * (kTcDrainWarps + 2);

__global__ void __launch_bounds__(kTcThreads, 1)
    tc_gemm_tf32x3_kernel(const __grid_constant__ TcMaps maps, int M, int N, int K, float* __restrict__ d,
                          int* __restrict__ status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(base + kTcStages * kStageBytes);
    uint64_t* empty = full + kTcStages;
    uint64_t* accf = empty + kTcStages;  // [2] chunk accumulated (MMA -> drain)
    uint64_t* acce = accf + 2;           // [2] accumulator drained (drain -> MMA)
    uint32_t* tslot = reinterpret_cast<uint32_t*>(acce + 2);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int n0 = blockIdx.x * kTcBN, m0 = blockIdx.y * kTcBM;
    // split K: this CTA owns K-blocks [kb0, kb0 + nk) of the tile
    const int nk_all = (K + kTcBK - 1) / kTcBK;
    const int kb0 = (int)(((int64_t)nk_all * blockIdx.z) / gridDim.z);
    const int nk = (int)(((int64_t)nk_all * (blockIdx.z + 1)) / gridDim.z) - kb0;
    const bool split = gridDim.z > 1;
    const int nchunks = (nk + kTcChunk - 1) / kTcChunk;
    if (t == 0) {
        prefetch_tmap(&maps.a_hi);
        prefetch_tmap(&maps.a_lo);
        prefetch_tmap(&maps.b_hi);
        prefetch_tmap(&maps.b_lo);
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(accf + b, 1);
            mbar_init(acce + b, kTcDrainWarps);
        }
        fence_mbar_init();
    }
    if (warp == kTcDrainWarps + 1) tmem_alloc(tslot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tslot;
    auto stage_ptr = [&](int s, int which) -> unsigned char* {
        // which: 0 A_hi, 1 A_lo, 2 B_hi, 3 B_lo
        const uint32_t off = which < 2 ? which * kTileA : 2 * kTileA + (which - 2) * kTileB;
        return base + s * kStageBytes + off;
    };
    if (warp == kTcDrainWarps) {
        if (lane == 0) {
            for (int kb = 0; kb < nk; ++kb) {
                const int s = kb % kTcStages;
                const uint32_t ph = (uint32_t)(kb / kTcStages) & 1u;
                if (!mbar_wait(empty + s, ph ^ 1u, kWaitBudget, status, kTcTimeoutEmpty)) break;
                mbar_arrive_expect_tx(full + s, kStageBytes);
                const int kx = (kb0 + kb) * kTcBK;
                tma_load_2d(stage_ptr(s, 0), &maps.a_hi, full + s, kx, m0);
                tma_load_2d(stage_ptr(s, 1), &maps.a_lo, full + s, kx, m0);
                tma_load_2d(stage_ptr(s, 2), &maps.b_hi, full + s, kx, n0);
                tma_load_2d(stage_ptr(s, 3), &maps.b_lo, full + s, kx, n0);
            }
        }
        __syncwarp();
    } else if (warp == kTcDrainWarps + 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_tf32(kTcBM, kTcBN);
            for (int kb = 0; kb < nk; ++kb) {
                const int c = kb / kTcChunk, buf = c & 1;
                const bool first = (kb % kTcChunk) == 0;
                if (first) {
                    if (!mbar_wait(acce + buf, ((uint32_t)(c >> 1) & 1u) ^ 1u, kWaitBudget, status,
                                   kTcTimeoutDone))
                        break;
                    tc_fence_after();
                }
                const int s = kb % kTcStages;
                const uint32_t ph = (uint32_t)(kb / kTcStages) & 1u;
                if (!mbar_wait(full + s, ph, kWaitBudget, status, kTcTimeoutFull)) break;
                tc_fence_after();
                const uint32_t acc = taddr + (uint32_t)(buf * kTcBN);
                const uint32_t ah = smem_u32(stage_ptr(s, 0)), al = smem_u32(stage_ptr(s, 1));
                const uint32_t bh = smem_u32(stage_ptr(s, 2)), bl = smem_u32(stage_ptr(s, 3));
#pragma unroll
                for (int k = 0; k < kTcBK / 8; ++k) {
                    const uint32_t o = 32u * k;
                    mma_tf32(acc, sw128_kmajor_desc(ah + o), sw128_kmajor_desc(bh + o), idesc, !(first && k == 0));
                    mma_tf32(acc, sw128_kmajor_desc(ah + o), sw128_kmajor_desc(bl + o), idesc, 1u);
                    mma_tf32(acc, sw128_kmajor_desc(al + o), sw128_kmajor_desc(bh + o), idesc, 1u);
                }
                mma_commit(empty + s);
                if ((kb % kTcChunk) == kTcChunk - 1 || kb == nk - 1) mma_commit(accf + buf);
            }
        }
        __syncwarp();
    } else {
        // drain warps
        const int lane_base = 32 * (warp & 3), col_base = 128 * (warp >> 2);
        float acc[128];
#pragma unroll
        for (int i = 0; i < 128; ++i) acc[i] = 0.f;
        bool ok = true;
        for (int c = 0; c < nchunks; ++c) {
            const int buf = c & 1;
            ok = __all_sync(0xffffffffu, mbar_wait(accf + buf, (uint32_t)(c >> 1) & 1u, kWaitBudget, status,
                                                   kTcTimeoutDone));
            if (!ok) break;
            tc_fence_after();
            const uint32_t src = taddr + ((uint32_t)lane_base << 16) + (uint32_t)(buf * kTcBN + col_base);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                uint32_t r[32];
                tmem_ld16_nowait(src + (uint32_t)(32 * h), r);
                tmem_ld16_nowait(src + (uint32_t)(32 * h + 16), r + 16);
                tmem_ld_wait();
#pragma unroll
                for (int i = 0; i < 32; ++i) acc[32 * h + i] = __fadd_rn(acc[32 * h + i], __uint_as_float(r[i]));
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce + buf);
        }
        if (ok) {
            const int row = m0 + lane_base + lane;
            if (row < M) {
                float* drow = d + (int64_t)row * N;
                const int col0 = n0 + col_base;
                if ((N & 3) == 0 && col0 + 128 <= N) {
                    float4* d4 = reinterpret_cast<float4*>(drow + col0);
#pragma unroll
                    for (int q = 0; q < 32; ++q) {
                        const float4 v = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
                        if (split)
                            atomicAdd(d4 + q, v);  // partial sums of the K split (D zeroed by the host)
                        else
                            d4[q] = v;
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 128; ++i)
                        if (col0 + i < N) {
                            if (split)
                                atomicAdd(drow + col0 + i, acc[i]);
                            else
                                drow[col0 + i] = acc[i];
                        }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kTcDrainWarps + 1) tmem_dealloc(taddr, 512);
}

// ---------------------------------------------------------------------------------------
// host side: tensor maps through the driver entry point (no link against libcuda)
// ---------------------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// General tiled tensor map (rank <= 5): dims / box innermost first, strides in bytes for
// dimensions 1 .. rank-1.
int tmap_encode(CUtensorMap* map, CUtensorMapDataType type, int rank, const void* ptr, const uint64_t* dims,
                const uint64_t* strides, const uint32_t* box, CUtensorMapSwizzle swizzle) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return set_error(MB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t d[5], st[4];
    cuuint32_t b[5], e[5];
    for (int i = 0; i < rank; ++i) {
        d[i] = dims[i];
        b[i] = box[i];
        e[i] = 1;
        if (i + 1 < rank) st[i] = strides[i];
    }
    const CUresult r = fn(map, type, (cuuint32_t)rank, const_cast<void*>(ptr), d, st, b, e,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(MB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MB_OK;
}

// rows x cols fp32 row-major matrix, box of box_rows x 32 columns, 128-byte swizzle.
static int make_map(CUtensorMap* m, const float* ptr, int64_t rows, int64_t cols, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return set_error(MB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)cols * 4};
    const cuuint32_t box[2] = {(cuuint32_t)kTcBK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(ptr), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(MB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MB_OK;
}

size_t cgemm_workspace_bytes(int64_t n, int64_t m) {
    const size_t bt = (size_t)(2 * m) * (size_t)(2 * n) * 4;
    return 2 * ((bt + 255) & ~size_t(255)) + 256;
}

int split_tf32(const float* src, int64_t count, float* hi, float* lo, cudaStream_t s) {
    if (count <= 0) return MB_OK;
    const int64_t blocks = std::min<int64_t>((count + 255) / 256, 152 * 32);
    split_tf32_kernel<<<(unsigned)blocks, 256, 0, s>>>(src, count, hi, lo);
    return check_launch("split_tf32");
}

static int* cgemm_status_ptr(void* ws, int64_t n, int64_t m) {
    return reinterpret_cast<int*>(static_cast<char*>(ws) + cgemm_workspace_bytes(n, m) - 256);
}

int cgemm_status(void* ws, int64_t n, int64_t m, int* out, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(out, cgemm_status_ptr(ws, n, m), sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "cgemm status: %s", cudaGetErrorString(e));
    return MB_OK;
}

// Y [n, m] complex64 = Z X, Z given as its split real view (z_hi, z_lo: [n, 2n] fp32).
// The workspace holds Bt_hi, Bt_lo and a status word (mbarrier time-outs; 0 = none).
int cgemm_tf32x3(const float* z_hi, const float* z_lo, int64_t n, const float* x, int64_t m, float* y,
                 void* ws, size_t ws_bytes, cudaStream_t s) {
    if (n <= 0 || m <= 0) return MB_OK;
    if (n & 1) return set_error(MB_ERR_ARG, "n must be even (TMA row strides are multiples of 16 bytes)");
    if (n > (1LL << 28) || m > (1LL << 20)) return set_error(MB_ERR_SIZE, "matrix too large");
    if (ws_bytes < cgemm_workspace_bytes(n, m)) return set_error(MB_ERR_ARG, "workspace too small");
    for (const void* p : {(const void*)z_hi, (const void*)z_lo, (const void*)ws})
        if (reinterpret_cast<uintptr_t>(p) & 15) return set_error(MB_ERR_ARG, "operands must be 16-byte aligned");
    const size_t bt = (((size_t)(2 * m) * (size_t)(2 * n) * 4) + 255) & ~size_t(255);
    float* bt_hi = static_cast<float*>(ws);
    float* bt_lo = reinterpret_cast<float*>(static_cast<char*>(ws) + bt);
    build_bt_kernel<<<dim3((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32)), dim3(32, 8), 0, s>>>(x, n, m, bt_hi,
                                                                                                    bt_lo);
    int* status = cgemm_status_ptr(ws, n, m);
    cudaMemsetAsync(status, 0, sizeof(int), s);
    TcMaps maps;
    const int64_t M = n, N = 2 * m, K = 2 * n;
    int rc;
    if ((rc = make_map(&maps.a_hi, z_hi, M, K, kTcBM))) return rc;
    if ((rc = make_map(&maps.a_lo, z_lo, M, K, kTcBM))) return rc;
    if ((rc = make_map(&maps.b_hi, bt_hi, N, K, kTcBN))) return rc;
    if ((rc = make_map(&maps.b_lo, bt_lo, N, K, kTcBN))) return rc;
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        attr_err = cudaFuncSetAttribute(tc_gemm_tf32x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    });
    if (attr_err != cudaSuccess) return set_error(MB_ERR_CUDA, "smem attribute: %s", cudaGetErrorString(attr_err));
    // One CTA per SM.  Split K so the number of work items fills whole waves of the SMs
    // (at least 16 K-blocks per item); split partials are added with vector atomics.
    const int64_t tiles = ((N + kTcBN - 1) / kTcBN) * ((M + kTcBM - 1) / kTcBM);
    const int64_t nk_all = (K + kTcBK - 1) / kTcBK;
    int sms = 152;
    {
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    int ksplit = 1;
    double best = 0.0;
    for (int ks = 1; ks <= 8; ++ks) {
        if (ks > 1 && nk_all / ks < 16) break;
        const double waves = (double)(tiles * ks) / sms;
        const double eff = waves / std::ceil(waves);
        if (eff > best + 0.02) {
            best = eff;
            ksplit = ks;
        }
    }
    if (ksplit > 1) cudaMemsetAsync(y, 0, (size_t)M * N * 4, s);
    const dim3 grid((unsigned)((N + kTcBN - 1) / kTcBN), (unsigned)((M + kTcBM - 1) / kTcBM), (unsigned)ksplit);
    if (grid.y > 65535) return set_error(MB_ERR_SIZE, "too many row tiles");
    tc_gemm_tf32x3_kernel<<<grid, kTcThreads, kTcSmem, s>>>(maps, (int)M, (int)N, (int)K, y, status);
    return check_launch("cgemm_tf32x3");
}

static float tf32_trunc(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u &= 0xFFFFE000u;
    std::memcpy(&x, &u, 4);
    return x;
}

int tc_selftest(double* max_rel_err, cudaStream_t s) {
    std::vector<float> ha(kTcBM * kTcBK), hb(kTcBN * kTcBK), hd(kTcBM * kTcBN, 0.f);
    uint32_t seed = 12345u;
    auto rnd = [&seed]() {
        seed = seed * 1664525u + 1013904223u;
        return ((seed >> 8) & 0xFFFF) / 32768.0f - 1.0f;
    };
    for (auto& v : ha) v = tf32_trunc(rnd());
    for (auto& v : hb) v = tf32_trunc(rnd());
    float *da = nullptr, *db = nullptr, *dd = nullptr;
    int* dstat = nullptr;
    cudaError_t e = cudaMalloc(&da, ha.size() * 4);
    if (e == cudaSuccess) e = cudaMalloc(&db, hb.size() * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dd, hd.size() * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dstat, 4);
    if (e == cudaSuccess) e = cudaMemcpyAsync(da, ha.data(), ha.size() * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(db, hb.data(), hb.size() * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dd, 0, hd.size() * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dstat, 0, 4, s);
    const int smem = (int)(kTileA + kTileB + 1024 + 256);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int status = 0;
    if (e == cudaSuccess) {
        tc_selftest_kernel<<<1, 128, smem, s>>>(da, db, dd, dstat);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hd.data(), dd, hd.size() * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, dstat, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(da);
    cudaFree(db);
    cudaFree(dd);
    cudaFree(dstat);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "tensor-core self-test: %s", cudaGetErrorString(e));
    if (status) return set_error(MB_ERR_CUDA, "tensor-core self-test: mbarrier wait timed out (status %d)", status);
    double worst = 0.0;
    for (int i = 0; i < kTcBM; ++i)
        for (int j = 0; j < kTcBN; ++j) {
            double ref = 0.0, mag = 0.0;
            for (int k = 0; k < kTcBK; ++k) {
                ref += (double)ha[i * kTcBK + k] * hb[j * kTcBK + k];
                mag += std::fabs((double)ha[i * kTcBK + k] * hb[j * kTcBK + k]);
            }
            worst = std::fmax(worst, std::fabs(hd[i * kTcBN + j] - ref) / (mag + 1e-30));
        }
    *max_rel_err = worst;
    return MB_OK;
}

}  // namespace mb
