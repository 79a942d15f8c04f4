// rayquery.cu -- closest-hit ray queries against the triangle mesh (a CUDA replacement of
// the reference's Vulkan ray-query plugin: src/vulkan_ray_tracing/ray_query_App.hpp:881-1000,
// shaders/raygen.rgen:23-64, closesthit.rchit, miss.rmiss).
//
// Semantics of the plugin: rays start at origin[row] along the normalised dir[row, col];
// opaque geometry, no face culling, hits with t in [tmin, tmax] (the shader uses 0.001 and
// 10000); each ray returns (face index, 0, 0, distance to the hit) or (-1, 0, 0, -1).
//
// Acceleration structure: a linear BVH (T. Karras, "Maximizing parallelism in the
// construction of BVHs, octrees, and k-d trees", HPG 2012):
//   1. 30-bit Morton codes of triangle centroids in the centroid box; 2. radix sort (CUB);
//   3. one thread per internal node finds its key range and split from common-prefix
//      lengths (ties broken by index); 4. boxes are merged bottom-up, the second child to
//      arrive at a node (atomic counter) computes its union; 5. every internal node is
//      packed into one 64-byte record holding both child boxes and both child ids, and every
//      leaf into 48 bytes (v0, e1 = v1 - v0, e2 = v2 - v0, face id), in leaf order.
// After the build the query reads only the packed records (the mesh arrays may go).
// Traversal: one thread per ray, explicit stack of 64 node ids (bounded; an overflow sets
// an error flag and ends that ray's traversal; so does a visit count above 2n), slab tests
// against both child boxes of a node (nearer child first, pruned by the best hit),
// Moller-Trumbore tests on leaves
// (Moller & Trumbore, J. Graphics Tools 2(1), 1997).  Equal distances keep the lower face id.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cub/device/device_radix_sort.cuh>

#include "common.cuh"

namespace mb {

constexpr int kRayStack = 64;
constexpr uint32_t kLeafBit = 0x80000000u;

struct BvhLayout {
    float4* nodes;      // [m][4]: (lmin xyz, lmax x) (lmax yz, rmin xy) (rmin z, rmax xyz) (left, right, -, -)
    float4* tris;       // [n][3]: (v0 xyz, face id bits) (e1 xyz, 0) (e2 xyz, 0)
    int32_t* status;    // [1] traversal stack overflow flag
    uint32_t* keys_in;  // build scratch from here on
    uint32_t* keys_out;
    int32_t* ids_in;
    int32_t* ids_out;   // sorted triangle ids (leaf i -> triangle ids_out[i])
    int32_t* left;      // [m] child (leaf if kLeafBit set)
    int32_t* right;     // [m]
    int32_t* parent;    // [m internal] then [n leaves] at parent + n - 1
    int32_t* flags;     // [m] arrival counters
    float* ibox;        // [m][6] internal boxes (min xyz, max xyz)
    float* lbox;        // [n][6] leaf boxes
    uint32_t* bounds;   // [6] centroid box, ordered-uint encoding
    void* sort_tmp;
    size_t sort_bytes;
};

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

static size_t sort_temp_bytes(int64_t n) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (const int32_t*)nullptr, (int32_t*)nullptr, (int)n, 0, 30);
    return b;
}

// Carves the caller's buffer; with base == nullptr it only sums the sizes.
static size_t carve_bvh(void* base, int64_t n, BvhLayout* L) {
    const size_t m = n > 1 ? (size_t)(n - 1) : 1, un = (size_t)n;
    size_t off = 0;
    char* p = static_cast<char*>(base);
    auto take = [&](size_t bytes) {
        void* at = p ? p + off : nullptr;
        off += align256(bytes);
        return at;
    };
    L->nodes = static_cast<float4*>(take(64 * m));
    L->tris = static_cast<float4*>(take(48 * un));
    L->status = static_cast<int32_t*>(take(4));
    L->keys_in = static_cast<uint32_t*>(take(4 * un));
    L->keys_out = static_cast<uint32_t*>(take(4 * un));
    L->ids_in = static_cast<int32_t*>(take(4 * un));
    L->ids_out = static_cast<int32_t*>(take(4 * un));
    L->left = static_cast<int32_t*>(take(4 * m));
    L->right = static_cast<int32_t*>(take(4 * m));
    L->parent = static_cast<int32_t*>(take(4 * (m + un)));
    L->flags = static_cast<int32_t*>(take(4 * m));
    L->ibox = static_cast<float*>(take(24 * m));
    L->lbox = static_cast<float*>(take(24 * un));
    L->bounds = static_cast<uint32_t*>(take(24));
    L->sort_bytes = sort_temp_bytes(n);
    L->sort_tmp = take(L->sort_bytes);
    return off;
}

size_t bvh_bytes(int64_t n) {
    BvhLayout L;
    return carve_bvh(nullptr, n, &L);
}

__device__ __forceinline__ uint32_t ord(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o ^ 0x80000000u) : ~o);
}

__global__ void bvh_init_kernel(uint32_t* bounds, int32_t* status) {
    if (threadIdx.x < 3) bounds[threadIdx.x] = 0xffffffffu;      // min
    else if (threadIdx.x < 6) bounds[threadIdx.x] = 0u;          // max
    if (threadIdx.x == 0) *status = 0;
}

__device__ __forceinline__ V3<float> centroid(const float* verts, const int32_t* faces, int64_t f) {
    const V3<float> a = load3(verts, faces[3 * f]), b = load3(verts, faces[3 * f + 1]),
                    c = load3(verts, faces[3 * f + 2]);
    return v3<float>((a.x + b.x + c.x) / 3.f, (a.y + b.y + c.y) / 3.f, (a.z + b.z + c.z) / 3.f);
}

__global__ void bvh_bounds_kernel(const float* __restrict__ verts, const int32_t* __restrict__ faces, int64_t n,
                                  uint32_t* __restrict__ bounds) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    const V3<float> c = centroid(verts, faces, f);
    const float c3[3] = {c.x, c.y, c.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        atomicMin(bounds + d, ord(c3[d]));
        atomicMax(bounds + 3 + d, ord(c3[d]));
    }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void bvh_morton_kernel(const float* __restrict__ verts, const int32_t* __restrict__ faces, int64_t n,
                                  const uint32_t* __restrict__ bounds, uint32_t* __restrict__ keys,
                                  int32_t* __restrict__ ids) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    const V3<float> c = centroid(verts, faces, f);
    const float c3[3] = {c.x, c.y, c.z};
    uint32_t code = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float lo = unord(bounds[d]), hi = unord(bounds[3 + d]);
        const float ext = hi - lo;
        float u = ext > 0.f ? (c3[d] - lo) / ext : 0.5f;
        u = fminf(fmaxf(u * 1024.f, 0.f), 1023.f);
        code |= spread10((uint32_t)u) << (2 - d);
    }
    keys[f] = code;
    ids[f] = (int32_t)f;
}

// Length of the common prefix of (key, index) pairs i and j; -1 outside [0, n).
__device__ __forceinline__ int delta(const uint32_t* keys, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = keys[i], b = keys[j];
    if (a != b) return __clz(a ^ b);
    return __clzll((unsigned long long)(i ^ j));  // = 32 + clz32(i ^ j): ties broken by index
}

__global__ void bvh_internal_kernel(const uint32_t* __restrict__ keys, int64_t n, int32_t* __restrict__ left,
                                    int32_t* __restrict__ right, int32_t* __restrict__ parent,
                                    int32_t* __restrict__ flags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int64_t lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;  // ends once i + lmax d leaves [0, n)
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int64_t j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int64_t s = 0;
    int64_t t = l;
    do {
        t = (t + 1) / 2;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int64_t g = i + s * d + (d < 0 ? d : 0);
    const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
    const int32_t lc = (lo == g) ? (int32_t)(g | kLeafBit) : (int32_t)g;
    const int32_t rc = (hi == g + 1) ? (int32_t)((g + 1) | kLeafBit) : (int32_t)(g + 1);
    left[i] = lc;
    right[i] = rc;
    // parent table: internal nodes at [0, n-1), leaves at [n-1, 2n-1)
    parent[(lc & kLeafBit) ? (n - 1) + (lc & ~kLeafBit) : lc] = (int32_t)i;
    parent[(rc & kLeafBit) ? (n - 1) + (rc & ~kLeafBit) : rc] = (int32_t)i;
    flags[i] = 0;
}

// Leaf boxes and packed triangles, then the bottom-up climb.  The climb has no waits: the
// first child to reach a node stops, the second (which sees the first's box through the
// fence + L2 loads) merges and continues; at most n - 1 steps.
__global__ void bvh_boxes_kernel(const float* __restrict__ verts, const int32_t* __restrict__ faces,
                                 const int32_t* __restrict__ ids, int64_t n, const int32_t* __restrict__ left,
                                 const int32_t* __restrict__ right, const int32_t* __restrict__ parent,
                                 int32_t* __restrict__ flags, float* __restrict__ ibox, float* __restrict__ lbox,
                                 float4* __restrict__ tris) {
    const int64_t leaf = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= n) return;
    const int32_t f = ids[leaf];
    const V3<float> a = load3(verts, faces[3 * (int64_t)f]), b = load3(verts, faces[3 * (int64_t)f + 1]),
                    c = load3(verts, faces[3 * (int64_t)f + 2]);
    const V3<float> e1 = b - a, e2 = c - a;
    tris[3 * leaf + 0] = make_float4(a.x, a.y, a.z, __int_as_float(f));
    tris[3 * leaf + 1] = make_float4(e1.x, e1.y, e1.z, 0.f);
    tris[3 * leaf + 2] = make_float4(e2.x, e2.y, e2.z, 0.f);
    float* lb = lbox + 6 * leaf;
    lb[0] = fminf(a.x, fminf(b.x, c.x)); lb[1] = fminf(a.y, fminf(b.y, c.y)); lb[2] = fminf(a.z, fminf(b.z, c.z));
    lb[3] = fmaxf(a.x, fmaxf(b.x, c.x)); lb[4] = fmaxf(a.y, fmaxf(b.y, c.y)); lb[5] = fmaxf(a.z, fmaxf(b.z, c.z));
    if (n == 1) return;
    __threadfence();
    int64_t node = parent[(n - 1) + leaf];
    for (int64_t guard = 0; guard < n; ++guard) {
        if (atomicAdd(flags + node, 1) == 0) return;  // first child to arrive stops here
        __threadfence();
        const int32_t lc = left[node], rc = right[node];
        const float* bl = (lc & kLeafBit) ? lbox + 6 * (int64_t)(lc & ~kLeafBit) : ibox + 6 * (int64_t)lc;
        const float* br = (rc & kLeafBit) ? lbox + 6 * (int64_t)(rc & ~kLeafBit) : ibox + 6 * (int64_t)rc;
        float* o = ibox + 6 * node;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            o[d] = fminf(__ldcg(bl + d), __ldcg(br + d));
            o[3 + d] = fmaxf(__ldcg(bl + 3 + d), __ldcg(br + 3 + d));
        }
        __threadfence();
        if (node == 0) return;
        node = parent[node];
    }
}

__global__ void bvh_pack_kernel(int64_t n, const int32_t* __restrict__ left, const int32_t* __restrict__ right,
                                const float* __restrict__ ibox, const float* __restrict__ lbox,
                                float4* __restrict__ nodes) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int32_t lc = left[i], rc = right[i];
    const float* bl = (lc & kLeafBit) ? lbox + 6 * (int64_t)(lc & ~kLeafBit) : ibox + 6 * (int64_t)lc;
    const float* br = (rc & kLeafBit) ? lbox + 6 * (int64_t)(rc & ~kLeafBit) : ibox + 6 * (int64_t)rc;
    nodes[4 * i + 0] = make_float4(bl[0], bl[1], bl[2], bl[3]);
    nodes[4 * i + 1] = make_float4(bl[4], bl[5], br[0], br[1]);
    nodes[4 * i + 2] = make_float4(br[2], br[3], br[4], br[5]);
    nodes[4 * i + 3] = make_float4(__int_as_float(lc), __int_as_float(rc), 0.f, 0.f);
}

// Slab test of the ray against [lo, hi]; enter distance in *t0.  Zero direction components
// are replaced by +-1e-20 before inverting, so 0 * inf never appears.
__device__ __forceinline__ bool slab(float lx, float ly, float lz, float hx, float hy, float hz, const V3<float>& o,
                                     const V3<float>& inv, float tmax, float* tenter) {
    float t0 = (lx - o.x) * inv.x, t1 = (hx - o.x) * inv.x;
    float tn = fminf(t0, t1), tf = fmaxf(t0, t1);
    t0 = (ly - o.y) * inv.y; t1 = (hy - o.y) * inv.y;
    tn = fmaxf(tn, fminf(t0, t1)); tf = fminf(tf, fmaxf(t0, t1));
    t0 = (lz - o.z) * inv.z; t1 = (hz - o.z) * inv.z;
    tn = fmaxf(tn, fminf(t0, t1)); tf = fminf(tf, fmaxf(t0, t1));
    *tenter = tn;
    return tf >= fmaxf(tn, 0.f) && tn <= tmax;
}

__device__ __forceinline__ float safe_inv(float d) {
    return 1.f / (fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d));
}

__global__ void __launch_bounds__(128) ray_query_kernel(const float4* __restrict__ nodes,
                                                        const float4* __restrict__ tris, int64_t n,
                                                        const float* __restrict__ origins,
                                                        const float* __restrict__ dirs, int64_t rows, int64_t cols,
                                                        float tmin, float tmax, float4* __restrict__ out,
                                                        int32_t* __restrict__ status) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows * cols) return;
    const int64_t row = r / cols;
    const V3<float> o = load3(origins, row);
    V3<float> d = load3(dirs, r);
    d = rsqrtf(dot(d, d)) * d;
    const V3<float> inv = v3<float>(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    float best = tmax;
    int32_t hit = -1;
    int32_t stack[kRayStack];
    int sp = 0;
    stack[sp++] = (n == 1) ? (int32_t)kLeafBit : 0;
    // A tree visits each of its 2n - 1 nodes at most once per ray; the cap only guards
    // against a buffer that does not hold a tree of n faces.
    for (int64_t visits = 0; sp > 0; ++visits) {
        if (visits > 2 * n) {
            atomicOr(status, 2);
            break;
        }
        const int32_t node = stack[--sp];
        if (node & kLeafBit) {
            const int64_t li = node & ~kLeafBit;
            const float4 t0 = __ldg(tris + 3 * li), t1 = __ldg(tris + 3 * li + 1), t2 = __ldg(tris + 3 * li + 2);
            const V3<float> v0 = v3<float>(t0.x, t0.y, t0.z), e1 = v3<float>(t1.x, t1.y, t1.z),
                            e2 = v3<float>(t2.x, t2.y, t2.z);
            const int32_t f = __float_as_int(t0.w);
            const V3<float> p = cross(d, e2);
            const float det = dot(e1, p);
            if (fabsf(det) < 1e-30f) continue;
            const float idet = 1.f / det;
            const V3<float> s = o - v0;
            const float u = dot(s, p) * idet;
            if (u < 0.f || u > 1.f) continue;
            const V3<float> q = cross(s, e1);
            const float v = dot(d, q) * idet;
            if (v < 0.f || u + v > 1.f) continue;
            const float t = dot(e2, q) * idet;
            if (t >= tmin && (t < best || (t == best && (hit < 0 || f < hit)))) {
                best = t;
                hit = f;
            }
            continue;
        }
        const float4 a = __ldg(nodes + 4 * (int64_t)node), b = __ldg(nodes + 4 * (int64_t)node + 1),
                     c = __ldg(nodes + 4 * (int64_t)node + 2), k = __ldg(nodes + 4 * (int64_t)node + 3);
        const int32_t lc = __float_as_int(k.x), rc = __float_as_int(k.y);
        float tl, tr;
        const bool hl = slab(a.x, a.y, a.z, a.w, b.x, b.y, o, inv, best, &tl);
        const bool hr = slab(b.z, b.w, c.x, c.y, c.z, c.w, o, inv, best, &tr);
        if (sp + 2 > kRayStack) {
            atomicOr(status, 1);
            break;
        }
        if (hl && hr) {
            if (tl <= tr) { stack[sp++] = rc; stack[sp++] = lc; }
            else { stack[sp++] = lc; stack[sp++] = rc; }
        } else if (hl) {
            stack[sp++] = lc;
        } else if (hr) {
            stack[sp++] = rc;
        }
    }
    out[r] = hit >= 0 ? make_float4((float)hit, 0.f, 0.f, best) : make_float4(-1.f, 0.f, 0.f, -1.f);
}

int bvh_build(const float* verts, const int32_t* faces, int64_t n, void* ws, size_t ws_bytes, cudaStream_t s) {
    if (n <= 0) return set_error(MB_ERR_ARG, "mesh has no faces");
    if (n >= (1LL << 30)) return set_error(MB_ERR_SIZE, "too many faces for the BVH (limit 2^30)");
    const size_t need = bvh_bytes(n);
    if (ws_bytes < need) return set_error(MB_ERR_ARG, "BVH buffer too small (need %zu bytes)", need);
    if (reinterpret_cast<uintptr_t>(ws) % 256) return set_error(MB_ERR_ARG, "BVH buffer not 256-byte aligned");
    BvhLayout L;
    carve_bvh(ws, n, &L);
    const int tb = 256;
    const unsigned blocks = (unsigned)((n + tb - 1) / tb);
    bvh_init_kernel<<<1, 32, 0, s>>>(L.bounds, L.status);
    bvh_bounds_kernel<<<blocks, tb, 0, s>>>(verts, faces, n, L.bounds);
    bvh_morton_kernel<<<blocks, tb, 0, s>>>(verts, faces, n, L.bounds, L.keys_in, L.ids_in);
    size_t tmp = L.sort_bytes;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(L.sort_tmp, tmp, L.keys_in, L.keys_out, L.ids_in, L.ids_out,
                                                    (int)n, 0, 30, s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "radix sort: %s", cudaGetErrorString(e));
    if (n > 1) {
        bvh_internal_kernel<<<(unsigned)((n - 1 + tb - 1) / tb), tb, 0, s>>>(L.keys_out, n, L.left, L.right,
                                                                              L.parent, L.flags);
    }
    bvh_boxes_kernel<<<blocks, tb, 0, s>>>(verts, faces, L.ids_out, n, L.left, L.right, L.parent, L.flags, L.ibox,
                                           L.lbox, L.tris);
    if (n > 1) {
        bvh_pack_kernel<<<(unsigned)((n - 1 + tb - 1) / tb), tb, 0, s>>>(n, L.left, L.right, L.ibox, L.lbox,
                                                                          L.nodes);
    }
    return check_launch("bvh_build");
}

int ray_query(const void* ws, int64_t n, const float* origins, const float* dirs, int64_t rows, int64_t cols,
              double tmin, double tmax, float* out, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return MB_OK;
    if (reinterpret_cast<uintptr_t>(out) % 16) return set_error(MB_ERR_ARG, "output not 16-byte aligned");
    BvhLayout L;
    carve_bvh(const_cast<void*>(ws), n, &L);
    const int64_t total = rows * cols;
    const unsigned blocks = (unsigned)((total + 127) / 128);
    ray_query_kernel<<<blocks, 128, 0, s>>>(L.nodes, L.tris, n, origins, dirs, rows, cols, (float)tmin,
                                            (float)tmax, reinterpret_cast<float4*>(out), L.status);
    return check_launch("ray_query");
}

int ray_status(const void* ws, int64_t n, int32_t* host_status, cudaStream_t s) {
    BvhLayout L;
    carve_bvh(const_cast<void*>(ws), n, &L);
    cudaError_t e = cudaMemcpyAsync(host_status, L.status, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "ray status: %s", cudaGetErrorString(e));
    return MB_OK;
}

}  // namespace mb
