// near_pairs.cu -- the list of ordered face pairs that share at least one vertex (each face
// with itself included), sorted by first face and then second face: the nonzeros of the
// reference's dense shared-vertex relation (compute_panel_relation, src/utils/mesh_utils.py:
// 700-725) in row-major order, built in O(F) memory and a handful of launches.
//
//   1. vertex valences (atomics), exclusive scan -> CSR offsets
//   2. vertex -> incident faces (atomics), each vertex's list sorted by face id
//   3. per face: the union of its three vertices' sorted lists (3-way merge, duplicates
//      dropped) -> a count, exclusive scan -> output offsets, total to the host
//   4. per face: the same merge, written at its offset.
// Deterministic: the output is the same for every run and equals the sorted unique list.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace mb {

constexpr int kScanThreads = 1024;

// ---- exclusive scan of int32 counts into int64 offsets (out[n] = total) ----------------
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* s_warp, int64_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        int64_t w = lane < nw ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) s_warp[lane] = w;
    }
    __syncthreads();
    const int64_t warp_base = warp > 0 ? s_warp[warp - 1] : 0;
    *total = s_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_base + x - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_block_sums(const int32_t* __restrict__ in, int64_t n,
                                                                int64_t* __restrict__ bsum) {
    __shared__ int64_t s_warp[32];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total;
    block_exclusive_scan(i < n ? in[i] : 0, s_warp, &total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// One block: exclusive scan of the block sums in place, in chunks of kScanThreads.
__global__ void __launch_bounds__(kScanThreads) scan_bsums(int64_t* __restrict__ bsum, int64_t nb) {
    __shared__ int64_t s_warp[32];
    int64_t carry = 0;
    for (int64_t c0 = 0; c0 < nb; c0 += blockDim.x) {
        const int64_t i = c0 + threadIdx.x;
        const int64_t v = i < nb ? bsum[i] : 0;
        int64_t total;
        const int64_t ex = block_exclusive_scan(v, s_warp, &total);
        if (i < nb) bsum[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_apply(const int32_t* __restrict__ in, int64_t n,
                                                           const int64_t* __restrict__ bsum,
                                                           int64_t* __restrict__ out) {
    __shared__ int64_t s_warp[32];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t v = i < n ? in[i] : 0;
    int64_t total;
    const int64_t ex = block_exclusive_scan(v, s_warp, &total) + bsum[blockIdx.x];
    if (i < n) out[i] = ex;
    if (i == n - 1) out[n] = ex + v;
}

static int64_t scan_blocks(int64_t n) { return (n + kScanThreads - 1) / kScanThreads; }

static void exclusive_scan(const int32_t* in, int64_t n, int64_t* bsum, int64_t* out, cudaStream_t s) {
    const int64_t nb = scan_blocks(n);
    scan_block_sums<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, bsum);
    scan_bsums<<<1, kScanThreads, 0, s>>>(bsum, nb);
    scan_apply<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, bsum, out);
}

// ---- vertex -> faces CSR ---------------------------------------------------------------
__global__ void nv_valence(const int32_t* __restrict__ faces, int64_t n3, int64_t nv, int32_t* __restrict__ val,
                           int32_t* __restrict__ status) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n3) return;
    const int32_t v = faces[t];
    if (v < 0 || v >= nv) {
        atomicOr(status, 1);
        return;
    }
    atomicAdd(val + v, 1);
}

__global__ void nv_fill(const int32_t* __restrict__ faces, int64_t n3, int64_t nv, const int64_t* __restrict__ vstart,
                        int32_t* __restrict__ cursor, int32_t* __restrict__ list) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n3) return;
    const int32_t v = faces[t];
    if (v < 0 || v >= nv) return;
    const int32_t slot = atomicAdd(cursor + v, 1);
    list[vstart[v] + slot] = (int32_t)(t / 3);
}

// Sorts each vertex's face list by face id (Shell sort with Knuth's gaps 1, 4, 13, ...:
// insertion sort for the usual valences of 4-8, and no quadratic blow-up for a vertex that
// fans out to very many faces).  A face listing a vertex twice appears twice; the merge
// below drops the duplicate.
__global__ void nv_sort(const int64_t* __restrict__ vstart, int64_t nv, int32_t* __restrict__ list) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    int32_t* a = list + vstart[v];
    const int64_t n = vstart[v + 1] - vstart[v];
    int64_t h = 1;
    while (h < n / 3) h = 3 * h + 1;
    for (; h >= 1; h /= 3) {
        for (int64_t i = h; i < n; ++i) {
            const int32_t x = a[i];
            int64_t j = i;
            while (j >= h && a[j - h] > x) {
                a[j] = a[j - h];
                j -= h;
            }
            a[j] = x;
        }
    }
}

// ---- per face: union of the three sorted vertex lists ----------------------------------
template <bool WRITE>
__global__ void nv_face_union(const int32_t* __restrict__ faces, int64_t nf, int64_t nv,
                              const int64_t* __restrict__ vstart, const int32_t* __restrict__ list,
                              int32_t* __restrict__ fcount, const int64_t* __restrict__ foff,
                              int32_t* __restrict__ pairs) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int64_t p[3], e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int32_t v = faces[3 * f + k];
        const bool ok = v >= 0 && v < nv;
        p[k] = ok ? vstart[v] : 0;
        e[k] = ok ? vstart[v + 1] : 0;
    }
    int64_t out = WRITE ? foff[f] : 0;
    int32_t count = 0, last = -1;
    for (;;) {
        int32_t m = 0x7fffffff;
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (p[k] < e[k] && list[p[k]] < m) m = list[p[k]];
        if (m == 0x7fffffff) break;
#pragma unroll
        for (int k = 0; k < 3; ++k)
            while (p[k] < e[k] && list[p[k]] == m) ++p[k];
        if (m != last) {
            if (WRITE) {
                pairs[2 * out] = (int32_t)f;
                pairs[2 * out + 1] = m;
                ++out;
            }
            ++count;
            last = m;
        }
    }
    if (!WRITE) fcount[f] = count;
}

struct NearWorkspace {
    int32_t* val;     // [nv] valences, then the fill cursors
    int64_t* vstart;  // [nv + 1]
    int32_t* list;    // [3 nf]
    int32_t* fcount;  // [nf]
    int64_t* foff;    // [nf + 1]
    int64_t* bsum;    // [max(scan blocks)]
    int32_t* status;  // [1]
};

static int64_t align256(int64_t b) { return (b + 255) / 256 * 256; }

int64_t near_pairs_workspace_bytes(int64_t nf, int64_t nv) {
    const int64_t nb = scan_blocks(nv > nf ? nv + 1 : nf + 1);
    return align256(4 * nv) + align256(8 * (nv + 1)) + align256(12 * nf) + align256(4 * nf) + align256(8 * (nf + 1)) +
           align256(8 * nb) + align256(4);
}

static NearWorkspace carve(void* ws, int64_t nf, int64_t nv) {
    char* p = static_cast<char*>(ws);
    NearWorkspace w;
    w.val = reinterpret_cast<int32_t*>(p);
    p += align256(4 * nv);
    w.vstart = reinterpret_cast<int64_t*>(p);
    p += align256(8 * (nv + 1));
    w.list = reinterpret_cast<int32_t*>(p);
    p += align256(12 * nf);
    w.fcount = reinterpret_cast<int32_t*>(p);
    p += align256(4 * nf);
    w.foff = reinterpret_cast<int64_t*>(p);
    p += align256(8 * (nf + 1));
    w.bsum = reinterpret_cast<int64_t*>(p);
    p += align256(8 * scan_blocks(nv > nf ? nv + 1 : nf + 1));
    w.status = reinterpret_cast<int32_t*>(p);
    return w;
}

// Phase 1: CSR, per-face counts and offsets in the workspace; *n_pairs = the list length
// (the stream is synchronised to read it).
int near_pairs_count(const int32_t* faces, int64_t nf, int64_t nv, void* ws, int64_t ws_bytes, int64_t* n_pairs,
                     cudaStream_t s) {
    *n_pairs = 0;
    if (nf <= 0) return MB_OK;
    if (nv <= 0) return set_error(MB_ERR_ARG, "faces given without vertices");
    if (ws_bytes < near_pairs_workspace_bytes(nf, nv)) return set_error(MB_ERR_ARG, "workspace too small");
    if (3 * nf > 0x7fffffffLL || nv > 0x7fffffffLL) return set_error(MB_ERR_SIZE, "mesh too large for int32 ids");
    const NearWorkspace w = carve(ws, nf, nv);
    const int64_t n3 = 3 * nf;
    const int threads = 256;
    cudaMemsetAsync(w.val, 0, 4 * nv, s);
    cudaMemsetAsync(w.status, 0, 4, s);
    nv_valence<<<(unsigned)((n3 + threads - 1) / threads), threads, 0, s>>>(faces, n3, nv, w.val, w.status);
    exclusive_scan(w.val, nv, w.bsum, w.vstart, s);
    cudaMemsetAsync(w.val, 0, 4 * nv, s);
    nv_fill<<<(unsigned)((n3 + threads - 1) / threads), threads, 0, s>>>(faces, n3, nv, w.vstart, w.val, w.list);
    nv_sort<<<(unsigned)((nv + threads - 1) / threads), threads, 0, s>>>(w.vstart, nv, w.list);
    nv_face_union<false><<<(unsigned)((nf + threads - 1) / threads), threads, 0, s>>>(
        faces, nf, nv, w.vstart, w.list, w.fcount, nullptr, nullptr);
    exclusive_scan(w.fcount, nf, w.bsum, w.foff, s);
    int rc = check_launch("near_pairs_count");
    if (rc != MB_OK) return rc;
    int32_t status = 0;
    cudaMemcpyAsync(n_pairs, w.foff + nf, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&status, w.status, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, cudaGetErrorString(e));
    if (status) return set_error(MB_ERR_ARG, "faces reference vertex ids outside [0, n_verts)");
    return MB_OK;
}

// Phase 2: writes the list (pairs [n_pairs, 2]) from the workspace of phase 1.
int near_pairs_fill(const int32_t* faces, int64_t nf, int64_t nv, void* ws, int32_t* pairs, cudaStream_t s) {
    if (nf <= 0) return MB_OK;
    const NearWorkspace w = carve(ws, nf, nv);
    const int threads = 256;
    nv_face_union<true><<<(unsigned)((nf + threads - 1) / threads), threads, 0, s>>>(
        faces, nf, nv, w.vstart, w.list, nullptr, w.foff, pairs);
    return check_launch("near_pairs_fill");
}

}  // namespace mb
