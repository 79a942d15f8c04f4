// capi.cu -- the C ABI of libmeshbem_gb300.so (declared in include/mesh_bem_gb300.h).
//
// Every entry point takes device pointers, element counts and a cudaStream_t (as void*;
// NULL = the legacy default stream), validates its arguments, launches asynchronously on
// that stream and returns MB_OK or an error code; mb_last_error() returns the message of
// the calling thread's last failure.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/mesh_bem_gb300.h"
#include "common.cuh"

namespace mb {

static thread_local char g_err[512] = "";

int set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(MB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return MB_OK;
}

struct PlaneWave;
template <typename T>
int launch_mom_ref_zmat(const T*, int64_t, const int32_t*, int64_t, const T*, const T*, const T*,
                        const T*, int, const T*, const T*, int, double, const int32_t*, int64_t, int64_t,
                        int64_t, int64_t, T*, T*, cudaStream_t);
template <typename T>
int launch_mom_ref_rhs(const T*, const int32_t*, int64_t, const T*, const T*, const T*, const T*, int,
                       const PlaneWave*, double, int, int, int64_t, const int32_t*, T*, T*, cudaStream_t);
int launch_mom_ref_zmat_batched(const float*, const int32_t*, const float*, const float*, const int32_t*,
                                const int64_t*, const int64_t*, int64_t, const double*, int, const float*, const float*,
                                int, const float*, const float*, int, float*, cudaStream_t, int);
template <typename T>
int launch_mom_ref_rhs_batched(const T*, const int32_t*, const T*, const T*, const int32_t*, const int64_t*, int,
                               int64_t, const T*, const T*, int, const PlaneWave*, int, int64_t, T*, cudaStream_t);
template <typename T>
int launch_mom_interp(const T*, const int32_t*, const int32_t*, const T*, const T*, const T*, int64_t,
                      int64_t, int64_t, int64_t, int, T*, T*, cudaStream_t);
template <typename T>
int launch_laplace_panels(const T*, const int32_t*, int64_t, const T*, const T*, const T*, const int*,
                          const uint8_t*, int, int, int, double, int64_t, int64_t, T*, T*, cudaStream_t);
template <typename T>
int launch_pack_tight(const T*, const T*, const int32_t*, int64_t, int64_t, int, T*, cudaStream_t);
template <typename T>
int launch_hypersingular(const T*, const int32_t*, int64_t, const T*, T*, cudaStream_t);
int64_t near_pairs_workspace_bytes(int64_t nf, int64_t nv);
int near_pairs_count(const int32_t* faces, int64_t nf, int64_t nv, void* ws, int64_t ws_bytes, int64_t* n_pairs,
                     cudaStream_t s);
int near_pairs_fill(const int32_t* faces, int64_t nf, int64_t nv, void* ws, int32_t* pairs, cudaStream_t s);
template <typename T>
int launch_hypersingular_tight(const T*, const int32_t*, int64_t, int64_t, const T*, T*, cudaStream_t);
template <typename T>
int launch_laplace_sym(const T*, const int32_t*, int64_t, int, int, const int32_t*, int64_t, int64_t, int64_t, T*,
                       cudaStream_t);
template <typename T>
int launch_laplace_sym_tight(const T*, const int32_t*, int64_t, int64_t, int, const int32_t*, int64_t, int64_t,
                             int64_t, T*, cudaStream_t);
template <typename T>
int launch_laplace_colloc_sl(const T*, const int32_t*, int64_t, const int32_t*, int64_t, int64_t, int64_t, T*,
                             cudaStream_t);
int launch_panel_relation(const int32_t*, int64_t, uint8_t*, cudaStream_t);
size_t gmres_workspace_bytes(int64_t n, int m);
size_t gmres_real_workspace_bytes(int64_t n, int m);
int tc_selftest(double* max_rel_err, cudaStream_t s);
size_t cgemm_workspace_bytes(int64_t n, int64_t m);
int split_tf32(const float* src, int64_t count, float* hi, float* lo, cudaStream_t s);
int cgemm_tf32x3(const float* z_hi, const float* z_lo, int64_t n, const float* x, int64_t m, float* y, void* ws,
                 size_t ws_bytes, cudaStream_t s);
int cgemm_status(void* ws, int64_t n, int64_t m, int* out, cudaStream_t s);
size_t gmres_multi_workspace_bytes(int64_t n, int64_t m, int r);
int gnn_gemm(const void* X, int x_bf16, const void* W, int w_bf16, int trans_w, const float* bias, int64_t N, int K,
             int M, int relu, void* Y, int y_bf16, cudaStream_t s);
int gnn_gemm_tn(const void* X, int x_bf16, const float* dY, int64_t N, int K, int M, float* dW, cudaStream_t s);
int gnn_colsum(const float* dY, int64_t N, int M, float* db, cudaStream_t s);
int gnn_aggregate(const void* h, const int32_t* nbr, int64_t N, int F, void* out, cudaStream_t s);
int gnn_aggregate_bwd(const float* dcat, const int32_t* nbr, int64_t N, int F, float* dh, cudaStream_t s);
int gnn_relu_bwd(const void* y, const float* dy, int64_t count, float* dz, cudaStream_t s);
int gnn_adam(float* w, float* m1, float* m2, const float* g, int64_t count, float lr, float b1, float b2, float eps,
             int step, void* w16, cudaStream_t s);
int launch_edge_rows(const int32_t* fei, int64_t nf, int64_t n_edges, int32_t* er, cudaStream_t s);
bool launch_fast_zmat_edges(const float* verts, const int32_t* faces, const float* areas, const float* normals,
                            const int32_t* fei, const int32_t* edge_rows, int64_t n_edges, const float* gpx,
                            const float* gwx, int nx, const float* gpy, const float* gwy, int ny, double k,
                            int64_t nf, int64_t m_begin, int64_t m_end, float* z, cudaStream_t stream);
bool launch_fast_zmat_gather(const float* verts, const int32_t* faces, const float* areas, const float* normals,
                             const int32_t* edge_rows, int64_t n_edges, const float* gpx, const float* gwx, int nx,
                             const float* gpy, const float* gwy, int ny, double k, int64_t m_begin, int64_t m_end,
                             float* z, cudaStream_t stream);
int zmat_edges_to_host(const float* verts, const int32_t* faces, const float* areas, const float* normals,
                       const int32_t* fei, const int32_t* edge_rows, int64_t n_edges, const float* gpx,
                       const float* gwx, int nx, const float* gpy, const float* gwy, int ny, double k, int64_t nf,
                       float* z_dev, float* z_host, int chunks, cudaStream_t s);
size_t gmres_blockdiag_workspace_bytes(int64_t n, int64_t m, int r);
int gmres_multi_column_steps(const void* ws, int64_t n, int64_t m, int r, int32_t* out, cudaStream_t s);
int gmres_blockdiag_column_steps(const void* ws, int64_t n, int64_t m, int r, int32_t* out, cudaStream_t s);
int blockdiag_matvec(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                     const float* x, int64_t ld, int nc, int rows, float* y, cudaStream_t s, const int* cact);
int gmres_blockdiag(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                    int rows_per_warp, int nc, int64_t n_rows, const double* b, double* x, int r, int max_iters,
                    double tol, bool use_graph, void* workspace, size_t ws_bytes, int64_t* iters_out,
                    int64_t* cycles_out, double* max_relres_out, int* status_out, cudaStream_t s);
template <typename T>
int launch_mom_sym_batched(const T*, const int32_t*, const int32_t*, const int64_t*, const double*, int, int64_t,
                           const int32_t*, int64_t, T*, cudaStream_t);
template <typename T>
int launch_mom_sym_rhs_batched(const T*, const int32_t*, const int32_t*, const int64_t*, int, int64_t, const double*,
                               int, int64_t, T*, cudaStream_t);
int gmres_multi(const float* z_hi, const float* z_lo, int64_t n, const double* b, double* x, int64_t m, int r,
                int max_iters, double tol, void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out,
                double* max_relres_out, int* status_out, cudaStream_t s);
int gmres_real(int kind, const void* a, int64_t n, const double* b, double* x, int m, int max_iters, double tol,
               void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out, double* relres_out,
               int* status_out, cudaStream_t s);
size_t bvh_bytes(int64_t n);
int bvh_build(const float*, const int32_t*, int64_t, void*, size_t, cudaStream_t);
int ray_query(const void*, int64_t, const float*, const float*, int64_t, int64_t, double, double, float*,
              cudaStream_t);
int ray_status(const void*, int64_t, int32_t*, cudaStream_t);
template <typename T>
int launch_mom_sym_regular(const T*, const int32_t*, const int32_t*, int64_t, double, int64_t, int64_t, int64_t,
                           T*, cudaStream_t);
template <typename T>
int launch_mom_sym_near(const T*, const int32_t*, const int32_t*, int64_t, const int32_t*, int64_t, double, T*,
                        cudaStream_t);
template <typename T>
int launch_mom_sym_rhs(const T*, const int32_t*, const int32_t*, const double*, int, int64_t, T*, cudaStream_t);
int sym_zmat_to_host(const float* verts, const int32_t* faces, const int32_t* fei, int64_t nf, int64_t n_edges,
                     double k, const int32_t* pairs, int64_t n_pairs, float* z_dev, float* z_host, int chunks,
                     cudaStream_t s);
template <typename T>
int launch_radiate_h(const T*, int64_t, const T*, const T*, const T*, int64_t, double, T*, cudaStream_t);
int gmres_c64(const float*, int64_t, const double*, double*, int, int, double, void*, size_t, int64_t*,
              int64_t*, double*, int*, cudaStream_t);
size_t spai_workspace_bytes(int64_t total_edges);
int spai_build(const float* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc, int n_mesh,
               int64_t total_faces, int64_t total_edges, const int32_t* pairs, int64_t n_pairs, const float* z,
               int32_t* m_cols, float* m_vals, void* ws, size_t ws_bytes, cudaStream_t s);
int spai_status(const void* ws, int64_t total_edges, int32_t* out, cudaStream_t s);
int spai_apply_c64(const int32_t* m_cols, const float* m_vals, int64_t n, const float* v, float* y, cudaStream_t s);
size_t pgmres_workspace_bytes(int64_t n, int m);
int pgmres(int kind, const void* z, const void* z_half, const float* half_scale, double inner_rtol, int64_t n,
           const int32_t* m_cols, const float* m_vals, const double* b, double* x, int m, int max_iters, double tol,
           bool use_graph, void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out,
           double* relres_out, int* status_out, cudaStream_t s);
int half_copy_c64(const float* z, int64_t count, void* zh, float* scale, cudaStream_t s);
int launch_mom_sym_rows_batched(const float* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc,
                                const double* ks, int n_mesh, const int32_t* sched, const int64_t* boff,
                                int64_t total_blocks, int rows_per_block, const int32_t* pairs, int64_t n_pairs,
                                float* z, cudaStream_t s);
int gmres_blockdiag_pc(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                       int rows_per_warp, int nc, int64_t n_rows, const int32_t* m_cols, const float* m_vals,
                       const int64_t* eoff, const double* b, double* x, int r, int max_iters, double tol,
                       bool use_graph, void* workspace, size_t ws_bytes, int64_t* iters_out, int64_t* cycles_out,
                       double* max_relres_out, int* status_out, cudaStream_t s);
int gmres_blockdiag_aug(const float*, const int64_t*, const int64_t*, int, int64_t, int, int, int64_t, const int32_t*,
                        const float*, const int64_t*, const float*, const float*, int, const double*, double*, int, int,
                        double, bool, void*, size_t, int64_t*, int64_t*, double*, int*, cudaStream_t);
int gmres_c64_noalloc(const float*, int64_t, const double*, double*, int, int, double, int64_t*, int64_t*,
                      double*, int*, cudaStream_t);
int launch_matvec_c64(const float*, const float*, int64_t, double*, cudaStream_t);
int launch_residual_c128(const float*, const double*, const double*, int64_t, double*, cudaStream_t);

}  // namespace mb

using namespace mb;

#define MB_REQUIRE(cond, ...)                              \
    do {                                                   \
        if (!(cond)) return set_error(MB_ERR_ARG, __VA_ARGS__); \
    } while (0)

static inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

template <typename T>
static int zmat_fe(const T* verts, int64_t nv, const int32_t* faces, int64_t nf, const T* areas,
                   const T* normals, const T* gpx, const T* gwx, int nx, const T* gpy, const T* gwy,
                   int ny, double k, int64_t batch, T* zr, T* zi, void* stream) {
    MB_REQUIRE(nf >= 0 && nv >= 0 && batch >= 1, "bad sizes (n_faces=%lld, batch=%lld)", (long long)nf,
               (long long)batch);
    if (nf == 0) return MB_OK;
    MB_REQUIRE(verts && faces && areas && normals && gpx && gwx && gpy && gwy && zr && zi,
               "null pointer argument");
    return launch_mom_ref_zmat<T>(verts, nv, faces, nf, areas, normals, gpx, gwx, nx, gpy, gwy, ny, k,
                                  nullptr, 0, 0, 3 * nf, batch, zr, zi, as_stream(stream));
}

template <typename T>
static int zmat_rwg(const T* verts, int64_t nv, const int32_t* faces, int64_t nf, const T* areas,
                    const T* normals, const int32_t* fei, int64_t ne, const T* gpx, const T* gwx, int nx,
                    const T* gpy, const T* gwy, int ny, double k, int64_t row_begin, int64_t row_end,
                    T* z, void* stream) {
    MB_REQUIRE(nf >= 0 && ne >= 0, "bad sizes");
    if (nf == 0) return MB_OK;
    MB_REQUIRE(verts && faces && areas && normals && fei && gpx && gwx && gpy && gwy && z,
               "null pointer argument");
    MB_REQUIRE(0 <= row_begin && row_begin <= row_end && row_end <= 3 * nf,
               "row range [%lld, %lld) outside [0, 3F)", (long long)row_begin, (long long)row_end);
    return launch_mom_ref_zmat<T>(verts, nv, faces, nf, areas, normals, gpx, gwx, nx, gpy, gwy, ny, k,
                                  fei, ne, row_begin, row_end, 1, z, nullptr, as_stream(stream));
}

extern "C" {

const char* mb_last_error(void) { return g_err; }

int mb_abi_version(void) { return MB_ABI_VERSION; }

int mb_mom_zmat_fe_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                       const float* face_areas, const float* face_normals, const float* gp_x,
                       const float* gw_x, int n_x, const float* gp_y, const float* gw_y, int n_y,
                       double wavenumber, int64_t batch, float* z_real, float* z_imag, void* stream) {
    return zmat_fe<float>(verts, n_verts, faces, n_faces, face_areas, face_normals, gp_x, gw_x, n_x,
                          gp_y, gw_y, n_y, wavenumber, batch, z_real, z_imag, stream);
}

int mb_mom_zmat_fe_f64(const double* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                       const double* face_areas, const double* face_normals, const double* gp_x,
                       const double* gw_x, int n_x, const double* gp_y, const double* gw_y, int n_y,
                       double wavenumber, int64_t batch, double* z_real, double* z_imag, void* stream) {
    return zmat_fe<double>(verts, n_verts, faces, n_faces, face_areas, face_normals, gp_x, gw_x, n_x,
                           gp_y, gw_y, n_y, wavenumber, batch, z_real, z_imag, stream);
}

int mb_mom_zmat_rwg_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                        const float* face_areas, const float* face_normals,
                        const int32_t* face_edge_indices, int64_t n_edges, const float* gp_x,
                        const float* gw_x, int n_x, const float* gp_y, const float* gw_y, int n_y,
                        double wavenumber, int64_t row_begin, int64_t row_end, float* z, void* stream) {
    return zmat_rwg<float>(verts, n_verts, faces, n_faces, face_areas, face_normals, face_edge_indices,
                           n_edges, gp_x, gw_x, n_x, gp_y, gw_y, n_y, wavenumber, row_begin, row_end, z,
                           stream);
}

int mb_mom_zmat_rwg_c128(const double* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                         const double* face_areas, const double* face_normals,
                         const int32_t* face_edge_indices, int64_t n_edges, const double* gp_x,
                         const double* gw_x, int n_x, const double* gp_y, const double* gw_y, int n_y,
                         double wavenumber, int64_t row_begin, int64_t row_end, double* z, void* stream) {
    return zmat_rwg<double>(verts, n_verts, faces, n_faces, face_areas, face_normals, face_edge_indices,
                            n_edges, gp_x, gw_x, n_x, gp_y, gw_y, n_y, wavenumber, row_begin, row_end, z,
                            stream);
}

int mb_mom_edge_rows(const int32_t* face_edge_indices, int64_t n_faces, int64_t n_edges, int32_t* edge_rows,
                     void* stream) {
    MB_REQUIRE(n_faces >= 0 && n_edges >= 0 && n_edges < (1ll << 30) && 3 * n_faces < (1ll << 31), "bad sizes");
    MB_REQUIRE(face_edge_indices && edge_rows, "null pointer argument");
    return launch_edge_rows(face_edge_indices, n_faces, n_edges, edge_rows, as_stream(stream));
}

int mb_mom_zmat_rwg_edges_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                              const float* face_areas, const float* face_normals,
                              const int32_t* face_edge_indices, const int32_t* edge_rows, int64_t n_edges,
                              const float* gp_x, const float* gw_x, int n_x, const float* gp_y,
                              const float* gw_y, int n_y, double wavenumber, int64_t m_begin, int64_t m_end,
                              float* z, void* stream) {
    (void)n_verts;
    MB_REQUIRE(n_faces >= 0 && n_edges >= 0, "bad sizes");
    MB_REQUIRE(0 <= m_begin && m_begin <= m_end && m_end <= n_edges, "row range outside [0, n_edges)");
    MB_REQUIRE(verts && faces && face_areas && face_normals && face_edge_indices && edge_rows && gp_x && gw_x &&
                   gp_y && gw_y && z,
               "null pointer argument");
    MB_REQUIRE(wavenumber > 0, "wavenumber must be > 0");
    MB_REQUIRE((m_end - m_begin) * ((3 * n_faces + 127) / 128) < 0x7fffffffLL, "mesh too large for one launch");
    if (!launch_fast_zmat_edges(verts, faces, face_areas, face_normals, face_edge_indices, edge_rows, n_edges,
                                gp_x, gw_x, n_x, gp_y, gw_y, n_y, wavenumber, n_faces, m_begin, m_end, z,
                                as_stream(stream)))
        return set_error(MB_ERR_UNSUPPORTED, "edge-row assembly: no instance for rule sizes (%d, %d)", n_x, n_y);
    return check_launch("mom_ref_zmat_edges");
}

int mb_mom_zmat_rwg_gather_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                               const float* face_areas, const float* face_normals, const int32_t* edge_rows,
                               int64_t n_edges, const float* gp_x, const float* gw_x, int n_x, const float* gp_y,
                               const float* gw_y, int n_y, double wavenumber, int64_t m_begin, int64_t m_end,
                               float* z, void* stream) {
    (void)n_verts;
    MB_REQUIRE(n_faces >= 0 && n_edges >= 0, "bad sizes");
    MB_REQUIRE(0 <= m_begin && m_begin <= m_end && m_end <= n_edges, "row range outside [0, n_edges)");
    MB_REQUIRE(verts && faces && face_areas && face_normals && edge_rows && gp_x && gw_x && gp_y && gw_y && z,
               "null pointer argument");
    MB_REQUIRE(wavenumber > 0, "wavenumber must be > 0");
    MB_REQUIRE((m_end - m_begin) * ((n_edges + 127) / 128) < 0x7fffffffLL, "mesh too large for one launch");
    if (!launch_fast_zmat_gather(verts, faces, face_areas, face_normals, edge_rows, n_edges, gp_x, gw_x, n_x, gp_y,
                                 gw_y, n_y, wavenumber, m_begin, m_end, z, as_stream(stream)))
        return set_error(MB_ERR_UNSUPPORTED, "gather assembly: no instance for rule sizes (%d, %d)", n_x, n_y);
    return check_launch("mom_ref_zmat_gather");
}

int mb_mom_zmat_rwg_to_host_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                                const float* face_areas, const float* face_normals,
                                const int32_t* face_edge_indices, int64_t n_edges, const float* gp_x,
                                const float* gw_x, int n_x, const float* gp_y, const float* gw_y, int n_y,
                                double wavenumber, int32_t* edge_rows, float* z_dev, float* z_host, int chunks,
                                void* stream) {
    MB_REQUIRE(n_faces >= 0 && n_edges >= 0 && n_edges < (1ll << 30), "bad sizes");
    MB_REQUIRE(verts && faces && face_areas && face_normals && face_edge_indices && edge_rows && gp_x && gw_x &&
                   gp_y && gw_y && z_dev && z_host,
               "null pointer argument");
    MB_REQUIRE(wavenumber > 0, "wavenumber must be > 0");
    if (n_faces == 0 || n_edges == 0) return MB_OK;
    cudaStream_t s = as_stream(stream);
    int rc = launch_edge_rows(face_edge_indices, n_faces, n_edges, edge_rows, s);
    if (rc) return rc;
    int32_t many = 0;
    cudaMemcpyAsync(&many, edge_rows + 2 * n_edges, 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return check_launch("zmat to host: edge rows");
    const bool fast = (n_x == 4 && n_y == 3) || (n_x == 3 && n_y == 2) || (n_x == 2 && n_y == 1) ||
                      (n_x == 5 && n_y == 4);
    MB_REQUIRE((n_edges / std::max(chunks, 1) + 1) * ((3 * n_faces + 127) / 128) < 0x7fffffffLL,
               "mesh too large for one launch per chunk");
    if (!many && fast)
        return zmat_edges_to_host(verts, faces, face_areas, face_normals, face_edge_indices, edge_rows, n_edges,
                                  gp_x, gw_x, n_x, gp_y, gw_y, n_y, wavenumber, n_faces, z_dev, z_host, chunks, s);
    cudaMemsetAsync(z_dev, 0, (size_t)n_edges * n_edges * 8, s);
    rc = zmat_rwg<float>(verts, n_verts, faces, n_faces, face_areas, face_normals, face_edge_indices, n_edges,
                         gp_x, gw_x, n_x, gp_y, gw_y, n_y, wavenumber, 0, 3 * n_faces, z_dev, stream);
    if (rc) return rc;
    if (cudaMemcpyAsync(z_host, z_dev, (size_t)n_edges * n_edges * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return check_launch("zmat to host: copy");
    return MB_OK;
}

int mb_gmres_multi_column_steps(const void* workspace, int64_t n, int64_t m, int restart, int32_t* out,
                                void* stream) {
    MB_REQUIRE(workspace && out && n > 0 && m > 0 && restart >= 1, "bad arguments");
    return gmres_multi_column_steps(workspace, n, m, restart, out, as_stream(stream));
}

int mb_gmres_blockdiag_column_steps(const void* workspace, int64_t n_rows, int64_t m, int restart, int32_t* out,
                                    void* stream) {
    MB_REQUIRE(workspace && out && n_rows > 0 && m > 0 && restart >= 1, "bad arguments");
    return gmres_blockdiag_column_steps(workspace, n_rows, m, restart, out, as_stream(stream));
}

#define MB_RHS_FE(SFX, T)                                                                             \
    int mb_mom_rhs_fe_##SFX(const T* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,     \
                            const T* face_areas, const T* face_normals, const T* gp, const T* gw, int n, \
                            double wavenumber, int64_t batch, T* rhs_real, T* rhs_imag, void* stream) { \
        (void)n_verts;                                                                                \
        MB_REQUIRE(n_faces >= 0 && batch >= 1, "bad sizes");                                          \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && face_areas && face_normals && gp && gw && rhs_real && rhs_imag,    \
                   "null pointer argument");                                                          \
        return launch_mom_ref_rhs<T>(verts, faces, n_faces, face_areas, face_normals, gp, gw, n,       \
                                     nullptr, wavenumber, 1, 0, batch, nullptr, rhs_real, rhs_imag,    \
                                     as_stream(stream));                                              \
    }
MB_RHS_FE(f32, float)
MB_RHS_FE(f64, double)
#undef MB_RHS_FE

#define MB_RHS_RWG(SFX, T)                                                                            \
    int mb_mom_rhs_rwg_##SFX(const T* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,    \
                             const T* face_areas, const T* face_normals,                              \
                             const int32_t* face_edge_indices, int64_t n_edges, const T* gp,          \
                             const T* gw, int n, const double* waves, int n_rhs, T* rhs,              \
                             void* stream) {                                                          \
        (void)n_verts; (void)n_edges;                                                                 \
        MB_REQUIRE(n_faces >= 0 && n_rhs >= 1, "bad sizes");                                          \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && face_areas && face_normals && face_edge_indices && gp && gw &&     \
                       waves && rhs,                                                                  \
                   "null pointer argument");                                                          \
        return launch_mom_ref_rhs<T>(verts, faces, n_faces, face_areas, face_normals, gp, gw, n,       \
                                     reinterpret_cast<const PlaneWave*>(waves), 0.0, n_rhs, 1, 1,      \
                                     face_edge_indices, rhs, nullptr, as_stream(stream));              \
    }
MB_RHS_RWG(c64, float)
MB_RHS_RWG(c128, double)
#undef MB_RHS_RWG

#define MB_INTERP_FE(SFX, T)                                                                          \
    int mb_mom_interp_js_##SFX(const T* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,  \
                               const int32_t* face_edge_indices, const T* face_areas,                  \
                               const T* i_real, const T* i_imag, int64_t n_edges, int64_t batch,       \
                               T* js_real, T* js_imag, void* stream) {                                 \
        MB_REQUIRE(n_faces >= 0 && batch >= 0 && n_edges >= 0, "bad sizes");                          \
        if (n_faces == 0 || batch == 0) return MB_OK;                                                 \
        MB_REQUIRE(verts && faces && face_edge_indices && face_areas && i_real && i_imag && js_real && \
                       js_imag,                                                                       \
                   "null pointer argument");                                                          \
        return launch_mom_interp<T>(verts, faces, face_edge_indices, face_areas, i_real, i_imag,      \
                                    n_edges, n_faces, n_verts, batch, 0, js_real, js_imag,             \
                                    as_stream(stream));                                               \
    }
MB_INTERP_FE(f32, float)
MB_INTERP_FE(f64, double)
#undef MB_INTERP_FE

#define MB_INTERP_V(SFX, T)                                                                           \
    int mb_mom_interp_vert_##SFX(const T* verts, int64_t n_verts, const int32_t* faces,                \
                                 int64_t n_faces, const int32_t* face_edge_indices,                   \
                                 const T* face_areas, const T* i_coeff, int64_t n_edges,               \
                                 int64_t batch, T* vert_js, void* stream) {                            \
        MB_REQUIRE(n_faces >= 0 && batch >= 0 && n_edges >= 0, "bad sizes");                          \
        if (n_faces == 0 || batch == 0) return MB_OK;                                                 \
        MB_REQUIRE(verts && faces && face_edge_indices && face_areas && i_coeff && vert_js,            \
                   "null pointer argument");                                                          \
        return launch_mom_interp<T>(verts, faces, face_edge_indices, face_areas, i_coeff, nullptr,    \
                                    n_edges, n_faces, n_verts, batch, 1, vert_js, nullptr,             \
                                    as_stream(stream));                                               \
    }
MB_INTERP_V(c64, float)
MB_INTERP_V(c128, double)
#undef MB_INTERP_V

#define MB_LAP(SFX, T)                                                                                \
    int mb_laplace_panels_##SFX(const T* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces, \
                                const T* face_areas, const T* face_normals, const T* table,           \
                                const int32_t* segments, const uint8_t* relations, int layer,          \
                                int order, int kind, double wavenumber, int64_t row_begin,             \
                                int64_t row_end, T* out_real, T* out_imag, void* stream) {             \
        (void)n_verts;                                                                                \
        MB_REQUIRE(n_faces >= 0, "bad sizes");                                                        \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && face_areas && face_normals && table && segments && out_real,     \
                   "null pointer argument");                                                          \
        MB_REQUIRE(0 <= row_begin && row_begin <= row_end && row_end <= n_faces, "bad row range");    \
        for (int s = 0; s < 4; ++s)                                                                   \
            MB_REQUIRE(segments[s] >= 0 && segments[s] <= segments[s + 1], "bad rule segments");      \
        return launch_laplace_panels<T>(verts, faces, n_faces, face_areas, face_normals, table,       \
                                        segments, relations, layer, order, kind, wavenumber,           \
                                        row_begin, row_end, out_real, out_imag, as_stream(stream));    \
    }
MB_LAP(f32, float)
MB_LAP(f64, double)
#undef MB_LAP

#define MB_PACK(SFX, T)                                                                               \
    int mb_pack_tight_##SFX(const T* m_real, const T* m_imag, const int32_t* faces, int64_t n_faces,   \
                            int64_t n_verts, int order, T* packed, void* stream) {                    \
        MB_REQUIRE(n_faces >= 0 && n_verts >= 0, "bad sizes");                                        \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(m_real && faces && packed, "null pointer argument");                               \
        MB_REQUIRE(order == 0 || order == 1, "order must be 0 or 1");                                 \
        return launch_pack_tight<T>(m_real, m_imag, faces, n_faces, n_verts, order, packed,           \
                                    as_stream(stream));                                               \
    }
MB_PACK(f32, float)
MB_PACK(f64, double)
#undef MB_PACK

#define MB_HYP(SFX, T)                                                                                \
    int mb_laplace_hypersingular_##SFX(const T* verts, int64_t n_verts, const int32_t* faces,           \
                                       int64_t n_faces, const T* v0, T* out, void* stream) {           \
        (void)n_verts;                                                                                \
        MB_REQUIRE(n_faces >= 0, "bad sizes");                                                        \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && v0 && out, "null pointer argument");                             \
        return launch_hypersingular<T>(verts, faces, n_faces, v0, out, as_stream(stream));            \
    }
MB_HYP(f32, float)
MB_HYP(f64, double)
#undef MB_HYP

int64_t mb_shared_vertex_pairs_workspace_bytes(int64_t n_faces, int64_t n_verts) {
    if (n_faces < 0 || n_verts < 0) return 0;
    return near_pairs_workspace_bytes(n_faces, n_verts);
}

int mb_shared_vertex_pairs_count(const int32_t* faces, int64_t n_faces, int64_t n_verts, void* workspace,
                                 int64_t workspace_bytes, int64_t* n_pairs, void* stream) {
    MB_REQUIRE(n_faces >= 0 && n_verts >= 0, "bad sizes");
    MB_REQUIRE(n_pairs, "null pointer argument");
    *n_pairs = 0;
    if (n_faces == 0) return MB_OK;
    MB_REQUIRE(faces && workspace, "null pointer argument");
    return near_pairs_count(faces, n_faces, n_verts, workspace, workspace_bytes, n_pairs, as_stream(stream));
}

int mb_shared_vertex_pairs_fill(const int32_t* faces, int64_t n_faces, int64_t n_verts, void* workspace,
                                int32_t* pairs, void* stream) {
    MB_REQUIRE(n_faces >= 0 && n_verts >= 0, "bad sizes");
    if (n_faces == 0) return MB_OK;
    MB_REQUIRE(faces && workspace && pairs, "null pointer argument");
    return near_pairs_fill(faces, n_faces, n_verts, workspace, pairs, as_stream(stream));
}

#define MB_HYPT(SFX, T)                                                                               \
    int mb_laplace_hypersingular_tight_##SFX(const T* verts, int64_t n_verts, const int32_t* faces,     \
                                             int64_t n_faces, const T* v0, T* packed, void* stream) {  \
        MB_REQUIRE(n_faces >= 0 && n_verts >= 0, "bad sizes");                                        \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && v0 && packed, "null pointer argument");                          \
        return launch_hypersingular_tight<T>(verts, faces, n_faces, n_verts, v0, packed,              \
                                             as_stream(stream));                                      \
    }
MB_HYPT(f32, float)
MB_HYPT(f64, double)
#undef MB_HYPT

#define MB_LSYM(SFX, T)                                                                               \
    int mb_laplace_sym_##SFX(const T* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,    \
                             int layer, int order, const int32_t* near_pairs, int64_t n_near,          \
                             int64_t row_begin, int64_t row_end, T* out, void* stream) {               \
        (void)n_verts;                                                                                \
        MB_REQUIRE(n_faces >= 0 && n_near >= 0, "bad sizes");                                         \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && out && (near_pairs || n_near == 0), "null pointer argument");    \
        MB_REQUIRE(0 <= row_begin && row_begin <= row_end && row_end <= n_faces, "bad row range");    \
        return launch_laplace_sym<T>(verts, faces, n_faces, layer, order, near_pairs, n_near,         \
                                     row_begin, row_end, out, as_stream(stream));                     \
    }                                                                                                 \
    int mb_laplace_colloc_sl_##SFX(const T* verts, int64_t n_verts, const int32_t* faces,               \
                                   int64_t n_faces, const int32_t* near_pairs, int64_t n_near,         \
                                   int64_t row_begin, int64_t row_end, T* out, void* stream) {         \
        (void)n_verts;                                                                                \
        MB_REQUIRE(n_faces >= 0 && n_near >= 0, "bad sizes");                                         \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && out && (near_pairs || n_near == 0), "null pointer argument");    \
        MB_REQUIRE(0 <= row_begin && row_begin <= row_end && row_end <= n_faces, "bad row range");    \
        return launch_laplace_colloc_sl<T>(verts, faces, n_faces, near_pairs, n_near, row_begin,      \
                                           row_end, out, as_stream(stream));                          \
    }
MB_LSYM(f32, float)
MB_LSYM(f64, double)
#undef MB_LSYM

#define MB_LSYMT(SFX, T)                                                                              \
    int mb_laplace_sym_tight_##SFX(const T* verts, int64_t n_verts, const int32_t* faces,               \
                                   int64_t n_faces, int op, const int32_t* near_pairs, int64_t n_near,  \
                                   int64_t row_begin, int64_t row_end, T* packed, void* stream) {      \
        MB_REQUIRE(n_faces >= 0 && n_verts >= 0 && n_near >= 0, "bad sizes");                          \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && packed && (near_pairs || n_near == 0), "null pointer argument"); \
        MB_REQUIRE(0 <= row_begin && row_begin <= row_end && row_end <= n_faces, "bad row range");    \
        return launch_laplace_sym_tight<T>(verts, faces, n_faces, n_verts, op, near_pairs, n_near,    \
                                           row_begin, row_end, packed, as_stream(stream));            \
    }
MB_LSYMT(f32, float)
MB_LSYMT(f64, double)
#undef MB_LSYMT

#define MB_SYM(SFX, T)                                                                                \
    int mb_mom_sym_zmat_rwg_##SFX(const T* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,   \
                                  const int32_t* fei, int64_t n_edges, double wavenumber,               \
                                  int64_t face_begin, int64_t face_end, T* z, void* stream) {           \
        (void)n_verts;                                                                                \
        MB_REQUIRE(n_faces >= 0 && n_edges >= 0, "bad sizes");                                        \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && fei && z, "null pointer argument");                              \
        MB_REQUIRE(0 <= face_begin && face_begin <= face_end && face_end <= n_faces, "bad face range");  \
        return launch_mom_sym_regular<T>(verts, faces, fei, n_edges, wavenumber, n_faces, face_begin,    \
                                         face_end, z, as_stream(stream));                              \
    }                                                                                                 \
    int mb_mom_sym_near_##SFX(const T* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,       \
                              const int32_t* fei, int64_t n_edges, const int32_t* pairs, int64_t n_pairs, \
                              double wavenumber, T* z, void* stream) {                                \
        (void)n_verts; (void)n_faces;                                                                 \
        MB_REQUIRE(n_pairs >= 0 && n_edges >= 0, "bad sizes");                                        \
        if (n_pairs == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && fei && pairs && z, "null pointer argument");                     \
        return launch_mom_sym_near<T>(verts, faces, fei, n_edges, pairs, n_pairs, wavenumber, z,       \
                                      as_stream(stream));                                             \
    }                                                                                                 \
    int mb_mom_sym_rhs_rwg_##SFX(const T* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,    \
                                 const int32_t* fei, int64_t n_edges, const double* waves, int n_rhs,   \
                                 T* rhs, void* stream) {                                              \
        (void)n_verts; (void)n_edges;                                                                 \
        MB_REQUIRE(n_faces >= 0 && n_rhs >= 1, "bad sizes");                                          \
        if (n_faces == 0) return MB_OK;                                                               \
        MB_REQUIRE(verts && faces && fei && waves && rhs, "null pointer argument");                   \
        return launch_mom_sym_rhs<T>(verts, faces, fei, waves, n_rhs, n_faces, rhs, as_stream(stream)); \
    }
MB_SYM(c64, float)
MB_SYM(c128, double)
#undef MB_SYM

int mb_mom_sym_zmat_rwg_to_host_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                                    const int32_t* fei, int64_t n_edges, double wavenumber, const int32_t* pairs,
                                    int64_t n_pairs, float* z_dev, float* z_host, int chunks, void* stream) {
    (void)n_verts;
    MB_REQUIRE(n_faces >= 0 && n_edges >= 0 && n_pairs >= 0 && n_edges < (1ll << 31), "bad sizes");
    if (n_faces == 0 || n_edges == 0) return MB_OK;
    MB_REQUIRE(verts && faces && fei && z_dev && z_host && (pairs || n_pairs == 0), "null pointer argument");
    MB_REQUIRE(wavenumber > 0, "wavenumber must be > 0");
    return sym_zmat_to_host(verts, faces, fei, n_faces, n_edges, wavenumber, pairs, n_pairs, z_dev, z_host, chunks,
                            as_stream(stream));
}

size_t mb_ray_bvh_bytes(int64_t n_faces) { return n_faces > 0 ? bvh_bytes(n_faces) : 0; }

int mb_ray_bvh_build_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces, void* bvh,
                         size_t bvh_nbytes, void* stream) {
    (void)n_verts;
    MB_REQUIRE(n_faces > 0, "mesh has no faces");
    MB_REQUIRE(verts && faces && bvh, "null pointer argument");
    return bvh_build(verts, faces, n_faces, bvh, bvh_nbytes, as_stream(stream));
}

int mb_ray_query_f32(const void* bvh, int64_t n_faces, const float* origins, const float* dirs, int64_t n_rows,
                     int64_t n_cols, double tmin, double tmax, float* out, void* stream) {
    MB_REQUIRE(n_faces > 0 && n_rows >= 0 && n_cols >= 0, "bad sizes");
    if (n_rows == 0 || n_cols == 0) return MB_OK;
    MB_REQUIRE(bvh && origins && dirs && out, "null pointer argument");
    MB_REQUIRE(tmin <= tmax, "tmin > tmax");
    return ray_query(bvh, n_faces, origins, dirs, n_rows, n_cols, tmin, tmax, out, as_stream(stream));
}

int mb_ray_status(const void* bvh, int64_t n_faces, int32_t* overflow, void* stream) {
    MB_REQUIRE(bvh && overflow && n_faces > 0, "bad arguments");
    return ray_status(bvh, n_faces, overflow, as_stream(stream));
}

#define MB_RAD(SFX, T)                                                                                \
    int mb_radiate_h_##SFX(const T* points, int64_t n_points, const T* verts, const T* vert_areas,       \
                           const T* js, int64_t n_verts, double wavenumber, T* h, void* stream) {       \
        MB_REQUIRE(n_points >= 0 && n_verts >= 0, "bad sizes");                                       \
        if (n_points == 0) return MB_OK;                                                              \
        MB_REQUIRE(points && h && (n_verts == 0 || (verts && vert_areas && js)),                       \
                   "null pointer argument");                                                          \
        return launch_radiate_h<T>(points, n_points, verts, vert_areas, js, n_verts, wavenumber, h,    \
                                   as_stream(stream));                                                \
    }
MB_RAD(c64, float)
MB_RAD(c128, double)
#undef MB_RAD

size_t mb_gmres_workspace_bytes(int64_t n, int restart) {
    if (n <= 0 || restart < 1) return 0;
    return gmres_workspace_bytes(n, restart);
}

int mb_tc_selftest(double* max_rel_err, void* stream) {
    MB_REQUIRE(max_rel_err, "null pointer argument");
    return tc_selftest(max_rel_err, as_stream(stream));
}

int mb_split_tf32(const float* src, int64_t count, float* hi, float* lo, void* stream) {
    MB_REQUIRE(count >= 0, "bad sizes");
    if (count == 0) return MB_OK;
    MB_REQUIRE(src && hi && lo, "null pointer argument");
    return split_tf32(src, count, hi, lo, as_stream(stream));
}

size_t mb_cgemm_workspace_bytes(int64_t n, int64_t m) { return n > 0 && m > 0 ? cgemm_workspace_bytes(n, m) : 0; }

int mb_cgemm_tf32x3(const float* z_hi, const float* z_lo, int64_t n, const float* x, int64_t m, float* y,
                    void* workspace, size_t workspace_bytes, void* stream) {
    MB_REQUIRE(n >= 0 && m >= 0, "bad sizes");
    if (n == 0 || m == 0) return MB_OK;
    MB_REQUIRE(z_hi && z_lo && x && y && workspace, "null pointer argument");
    return cgemm_tf32x3(z_hi, z_lo, n, x, m, y, workspace, workspace_bytes, as_stream(stream));
}

int mb_cgemm_status(void* workspace, int64_t n, int64_t m, int32_t* status, void* stream) {
    MB_REQUIRE(workspace && status && n > 0 && m > 0, "bad arguments");
    return cgemm_status(workspace, n, m, status, as_stream(stream));
}

size_t mb_gmres_multi_workspace_bytes(int64_t n, int64_t m, int restart) {
    if (n <= 0 || m <= 0 || restart < 1) return 0;
    return gmres_multi_workspace_bytes(n, m, restart);
}

int mb_gmres_multi_c64(const float* z_hi, const float* z_lo, int64_t n, const double* b, double* x, int64_t m,
                       int restart, int max_iters, double tol, void* workspace, size_t workspace_bytes,
                       mb_gmres_info* info, void* stream) {
    MB_REQUIRE(n > 0 && m > 0, "n and m must be > 0");
    MB_REQUIRE(z_hi && z_lo && b && x && workspace, "null pointer argument");
    int64_t it = 0, cyc = 0;
    double rr = 0.0;
    int st = 1;
    const int rc = gmres_multi(z_hi, z_lo, n, b, x, m, restart, max_iters, tol, workspace, workspace_bytes, &it,
                               &cyc, &rr, &st, as_stream(stream));
    if (rc == MB_OK && info) {
        info->iterations = it;
        info->restarts = cyc;
        info->rel_residual = rr;
        info->status = st;
        info->reserved = 0;
    }
    return rc;
}

#define MB_BATCH(SFX, T)                                                                              \
    int mb_mom_sym_zmat_batched_##SFX(const T* verts, const int32_t* faces, const int32_t* fei,         \
                                      const int64_t* desc, const double* ks, int n_mesh,               \
                                      int64_t total_blocks, const int32_t* near_pairs, int64_t n_near, \
                                      T* z, void* stream) {                                            \
        MB_REQUIRE(n_mesh >= 0 && total_blocks >= 0 && n_near >= 0, "bad sizes");                     \
        if (n_mesh == 0) return MB_OK;                                                                \
        MB_REQUIRE(verts && faces && fei && desc && ks && z && (near_pairs || n_near == 0),           \
                   "null pointer argument");                                                          \
        return launch_mom_sym_batched<T>(verts, faces, fei, desc, ks, n_mesh, total_blocks, near_pairs, \
                                         n_near, z, as_stream(stream));                              \
    }                                                                                                 \
    int mb_mom_sym_rhs_batched_##SFX(const T* verts, const int32_t* faces, const int32_t* fei,          \
                                     const int64_t* desc, int n_mesh, int64_t total_faces,              \
                                     const double* waves, int nrhs, int64_t ld, T* rhs, void* stream) { \
        MB_REQUIRE(n_mesh >= 0 && total_faces >= 0 && nrhs >= 0 && ld >= 0, "bad sizes");             \
        if (n_mesh == 0 || total_faces == 0 || nrhs == 0) return MB_OK;                               \
        MB_REQUIRE(verts && faces && fei && desc && waves && rhs, "null pointer argument");           \
        return launch_mom_sym_rhs_batched<T>(verts, faces, fei, desc, n_mesh, total_faces, waves, nrhs, \
                                             ld, rhs, as_stream(stream));                            \
    }
MB_BATCH(c64, float)
MB_BATCH(c128, double)
#undef MB_BATCH

int mb_mom_ref_zmat_batched_c64(const float* verts, const int32_t* faces, const float* face_areas,
                                const float* face_normals, const int32_t* fei, const int64_t* desc,
                                const int64_t* block_offsets, int64_t total_blocks, const double* ks, int n_mesh,
                                const float* gpx, const float* gwx, int nx, const float* gpy, const float* gwy,
                                int ny, float* z, void* stream) {
    MB_REQUIRE(n_mesh >= 0 && total_blocks >= 0, "bad sizes");
    if (n_mesh == 0) return MB_OK;
    MB_REQUIRE(verts && faces && face_areas && face_normals && fei && desc && block_offsets && ks && gpx && gwx &&
                   gpy && gwy && z,
               "null pointer argument");
    return launch_mom_ref_zmat_batched(verts, faces, face_areas, face_normals, fei, desc, block_offsets,
                                       total_blocks, ks, n_mesh, gpx, gwx, nx, gpy, gwy, ny, z, as_stream(stream), 0);
}

int mb_mom_ref_zmat_batched_persistent_c64(const float* verts, const int32_t* faces, const float* face_areas,
                                           const float* face_normals, const int32_t* fei, const int64_t* desc,
                                           const int64_t* block_offsets, int64_t total_blocks, const double* ks,
                                           int n_mesh, const float* gpx, const float* gwx, int nx, const float* gpy,
                                           const float* gwy, int ny, float* z, void* stream) {
    MB_REQUIRE(n_mesh >= 0 && total_blocks >= 0, "bad sizes");
    if (n_mesh == 0) return MB_OK;
    MB_REQUIRE(verts && faces && face_areas && face_normals && fei && desc && block_offsets && ks && gpx && gwx &&
                   gpy && gwy && z,
               "null pointer argument");
    return launch_mom_ref_zmat_batched(verts, faces, face_areas, face_normals, fei, desc, block_offsets,
                                       total_blocks, ks, n_mesh, gpx, gwx, nx, gpy, gwy, ny, z, as_stream(stream), 1);
}

int mb_mom_ref_rhs_batched_c64(const float* verts, const int32_t* faces, const float* face_areas,
                               const float* face_normals, const int32_t* fei, const int64_t* desc, int n_mesh,
                               int64_t total_faces, const float* gp, const float* gw, int n, const double* waves,
                               int nrhs, int64_t ld, float* rhs, void* stream) {
    MB_REQUIRE(n_mesh >= 0 && total_faces >= 0 && nrhs >= 0, "bad sizes");
    if (n_mesh == 0 || total_faces == 0 || nrhs == 0) return MB_OK;
    MB_REQUIRE(verts && faces && face_areas && face_normals && fei && desc && gp && gw && waves && rhs,
               "null pointer argument");
    return launch_mom_ref_rhs_batched<float>(verts, faces, face_areas, face_normals, fei, desc, n_mesh, total_faces,
                                             gp, gw, n, reinterpret_cast<const PlaneWave*>(waves), nrhs, ld, rhs,
                                             as_stream(stream));
}

int mb_blockdiag_matvec_c64(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh,
                            int64_t total_warps, const float* x, int64_t ld, int nc, int rows_per_warp, float* y,
                            void* stream) {
    MB_REQUIRE(n_mesh >= 0 && total_warps >= 0, "bad sizes");
    if (n_mesh == 0) return MB_OK;
    MB_REQUIRE(z && desc && goff && x && y, "null pointer argument");
    return blockdiag_matvec(z, desc, goff, n_mesh, total_warps, x, ld, nc, rows_per_warp, y, as_stream(stream),
                            nullptr);
}

size_t mb_gmres_blockdiag_workspace_bytes(int64_t n_rows, int64_t m, int restart) {
    if (n_rows <= 0 || m <= 0 || restart < 1) return 0;
    return gmres_blockdiag_workspace_bytes(n_rows, m, restart);
}

int mb_gmres_blockdiag_c64(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh, int64_t total_warps,
                           int rows_per_warp, int nc, int64_t n_rows, const double* b, double* x, int restart,
                           int max_iters, double tol, int use_graph, void* workspace, size_t workspace_bytes,
                           mb_gmres_info* info, void* stream) {
    MB_REQUIRE(n_mesh > 0 && nc > 0 && n_rows > 0, "bad sizes");
    MB_REQUIRE(z && desc && goff && b && x && workspace, "null pointer argument");
    int64_t it = 0, cyc = 0;
    double rr = 0.0;
    int st = 1;
    const int rc = gmres_blockdiag(z, desc, goff, n_mesh, total_warps, rows_per_warp, nc, n_rows, b, x, restart,
                                   max_iters, tol, use_graph != 0, workspace, workspace_bytes, &it, &cyc, &rr, &st,
                                   as_stream(stream));
    if (rc == MB_OK && info) {
        info->iterations = it;
        info->restarts = cyc;
        info->rel_residual = rr;
        info->status = st;
        info->reserved = 0;
    }
    return rc;
}

int mb_gnn_gemm(const void* x, int x_bf16, const void* w, int w_bf16, int trans_w, const float* bias, int64_t n,
                int k, int m, int relu, void* y, int y_bf16, void* stream) {
    MB_REQUIRE(n >= 0 && k >= 0 && m >= 0, "bad sizes");
    if (n == 0 || k == 0 || m == 0) return MB_OK;
    MB_REQUIRE(x && w && y, "null pointer argument");
    return gnn_gemm(x, x_bf16, w, w_bf16, trans_w, bias, n, k, m, relu, y, y_bf16, as_stream(stream));
}
int mb_gnn_gemm_tn(const void* x, int x_bf16, const float* dy, int64_t n, int k, int m, float* dw, void* stream) {
    MB_REQUIRE(n >= 0 && k >= 0 && m >= 0, "bad sizes");
    if (n == 0 || k == 0 || m == 0) return MB_OK;
    MB_REQUIRE(x && dy && dw, "null pointer argument");
    return gnn_gemm_tn(x, x_bf16, dy, n, k, m, dw, as_stream(stream));
}
int mb_gnn_colsum(const float* dy, int64_t n, int m, float* db, void* stream) {
    MB_REQUIRE(n >= 0 && m >= 0 && (n == 0 || (dy && db)), "bad arguments");
    return gnn_colsum(dy, n, m, db, as_stream(stream));
}
int mb_gnn_aggregate(const void* h, const int32_t* nbr, int64_t n, int f, void* out, void* stream) {
    MB_REQUIRE(n >= 0 && f > 0 && (n == 0 || (h && nbr && out)), "bad arguments");
    return gnn_aggregate(h, nbr, n, f, out, as_stream(stream));
}
int mb_gnn_aggregate_bwd(const float* dcat, const int32_t* nbr, int64_t n, int f, float* dh, void* stream) {
    MB_REQUIRE(n >= 0 && f > 0 && (n == 0 || (dcat && nbr && dh)), "bad arguments");
    return gnn_aggregate_bwd(dcat, nbr, n, f, dh, as_stream(stream));
}
int mb_gnn_relu_bwd(const void* y, const float* dy, int64_t count, float* dz, void* stream) {
    MB_REQUIRE(count >= 0 && (count == 0 || (y && dy && dz)), "bad arguments");
    return gnn_relu_bwd(y, dy, count, dz, as_stream(stream));
}
int mb_gnn_adam(float* w, float* m1, float* m2, const float* g, int64_t count, double lr, double beta1, double beta2,
                double eps, int step, void* w_bf16, void* stream) {
    MB_REQUIRE(count >= 0 && step >= 1 && (count == 0 || (w && m1 && m2 && g)), "bad arguments");
    return gnn_adam(w, m1, m2, g, count, (float)lr, (float)beta1, (float)beta2, (float)eps, step, w_bf16,
                    as_stream(stream));
}

size_t mb_gmres_real_workspace_bytes(int64_t n, int restart) {
    if (n <= 0 || restart < 1) return 0;
    return gmres_real_workspace_bytes(n, restart);
}

static int gmres_real_entry(int kind, const void* a, int64_t n, const double* b, double* x, int restart,
                            int max_iters, double tol, void* workspace, size_t workspace_bytes,
                            mb_gmres_info* info, void* stream) {
    MB_REQUIRE(n > 0, "n must be > 0");
    MB_REQUIRE(a && b && x && workspace, "null pointer argument");
    int64_t it = 0, cyc = 0;
    double rr = 0.0;
    int st = 1;
    const int rc = gmres_real(kind, a, n, b, x, restart, max_iters, tol, workspace, workspace_bytes, &it, &cyc,
                              &rr, &st, as_stream(stream));
    if (rc == MB_OK && info) {
        info->iterations = it;
        info->restarts = cyc;
        info->rel_residual = rr;
        info->status = st;
        info->reserved = 0;
    }
    return rc;
}

int mb_gmres_f32(const float* a, int64_t n, const double* b, double* x, int restart, int max_iters, double tol,
                 void* workspace, size_t workspace_bytes, mb_gmres_info* info, void* stream) {
    return gmres_real_entry(1, a, n, b, x, restart, max_iters, tol, workspace, workspace_bytes, info, stream);
}

int mb_gmres_f64(const double* a, int64_t n, const double* b, double* x, int restart, int max_iters, double tol,
                 void* workspace, size_t workspace_bytes, mb_gmres_info* info, void* stream) {
    return gmres_real_entry(2, a, n, b, x, restart, max_iters, tol, workspace, workspace_bytes, info, stream);
}

int mb_gmres_c64(const float* z, int64_t n, const double* b, double* x, int restart, int max_iters,
                 double tol, void* workspace, size_t workspace_bytes, mb_gmres_info* info, void* stream) {
    MB_REQUIRE(n > 0, "n must be > 0");
    MB_REQUIRE(z && b && x && workspace, "null pointer argument");
    int64_t it = 0, cyc = 0;
    double rr = 0.0;
    int st = 1;
    const int rc = gmres_c64(z, n, b, x, restart, max_iters, tol, workspace, workspace_bytes, &it, &cyc, &rr,
                             &st, as_stream(stream));
    if (rc == MB_OK && info) {
        info->iterations = it;
        info->restarts = cyc;
        info->rel_residual = rr;
        info->status = st;
        info->reserved = 0;
    }
    return rc;
}

int mb_gmres_c64_noalloc(const float* z, int64_t n, const double* b, double* x, int restart, int max_iters,
                         double tol, mb_gmres_info* info, void* stream) {
    MB_REQUIRE(n > 0, "n must be > 0");
    MB_REQUIRE(z && b && x, "null pointer argument");
    int64_t it = 0, cyc = 0;
    double rr = 0.0;
    int st = 1;
    const int rc = gmres_c64_noalloc(z, n, b, x, restart, max_iters, tol, &it, &cyc, &rr, &st, as_stream(stream));
    if (rc == MB_OK && info) {
        info->iterations = it;
        info->restarts = cyc;
        info->rel_residual = rr;
        info->status = st;
        info->reserved = 0;
    }
    return rc;
}

int mb_matvec_c64(const float* z, const float* v, int64_t n, double* y, void* stream) {
    MB_REQUIRE(n >= 0, "bad sizes");
    if (n == 0) return MB_OK;
    MB_REQUIRE(z && v && y, "null pointer argument");
    return launch_matvec_c64(z, v, n, y, as_stream(stream));
}

int mb_residual_c128(const float* z, const double* x, const double* b, int64_t n, double* r, void* stream) {
    MB_REQUIRE(n >= 0, "bad sizes");
    if (n == 0) return MB_OK;
    MB_REQUIRE(z && x && b && r, "null pointer argument");
    return launch_residual_c128(z, x, b, n, r, as_stream(stream));
}

size_t mb_spai_workspace_bytes(int64_t total_edges) { return total_edges > 0 ? spai_workspace_bytes(total_edges) : 0; }

int mb_spai_build_c64(const float* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc, int n_mesh,
                      int64_t total_faces, int64_t total_edges, const int32_t* near_pairs, int64_t n_near,
                      const float* z, int32_t* m_cols, float* m_vals, void* workspace, size_t workspace_bytes,
                      void* stream) {
    return spai_build(verts, faces, fei, desc, n_mesh, total_faces, total_edges, near_pairs, n_near, z, m_cols,
                      m_vals, workspace, workspace_bytes, as_stream(stream));
}

int mb_spai_status(const void* workspace, int64_t total_edges, int32_t* status, void* stream) {
    MB_REQUIRE(workspace && status && total_edges > 0, "bad arguments");
    return spai_status(workspace, total_edges, status, as_stream(stream));
}

int mb_spai_apply_c64(const int32_t* m_cols, const float* m_vals, int64_t n, const float* v, float* y,
                      void* stream) {
    MB_REQUIRE(n >= 0, "bad sizes");
    if (n == 0) return MB_OK;
    MB_REQUIRE(m_cols && m_vals && v && y, "null pointer argument");
    return spai_apply_c64(m_cols, m_vals, n, v, y, as_stream(stream));
}

size_t mb_pgmres_workspace_bytes(int64_t n, int restart) {
    return (n > 0 && restart > 0) ? pgmres_workspace_bytes(n, restart) : 0;
}

static int pgmres_entry(int kind, const void* z, const void* z_half, const float* half_scale, double inner_rtol,
                        int64_t n, const int32_t* m_cols, const float* m_vals, const double* b, double* x,
                        int restart, int max_iters, double tol, int use_graph, void* workspace,
                        size_t workspace_bytes, mb_gmres_info* info, void* stream) {
    int64_t it = 0, cyc = 0;
    double rr = 0.0;
    int st = 1;
    const int rc = pgmres(kind, z, z_half, half_scale, inner_rtol, n, m_cols, m_vals, b, x, restart, max_iters, tol,
                          use_graph != 0, workspace, workspace_bytes, &it, &cyc, &rr, &st, as_stream(stream));
    if (rc == MB_OK && info) {
        info->iterations = it;
        info->restarts = cyc;
        info->rel_residual = rr;
        info->status = st;
        info->reserved = 0;
    }
    return rc;
}

int mb_pgmres_c64(const float* z, int64_t n, const void* z_half, const float* half_scale, double inner_rtol,
                  const int32_t* m_cols, const float* m_vals, const double* b, double* x, int restart, int max_iters,
                  double tol, int use_graph, void* workspace, size_t workspace_bytes, mb_gmres_info* info,
                  void* stream) {
    return pgmres_entry(0, z, z_half, half_scale, inner_rtol, n, m_cols, m_vals, b, x, restart, max_iters, tol,
                        use_graph, workspace, workspace_bytes, info, stream);
}

int mb_pgmres_c128(const double* z, int64_t n, const int32_t* m_cols, const float* m_vals, const double* b,
                   double* x, int restart, int max_iters, double tol, int use_graph, void* workspace,
                   size_t workspace_bytes, mb_gmres_info* info, void* stream) {
    return pgmres_entry(1, z, nullptr, nullptr, 0.0, n, m_cols, m_vals, b, x, restart, max_iters, tol, use_graph,
                        workspace, workspace_bytes, info, stream);
}

int mb_gmres_blockdiag_pc_c64(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh,
                              int64_t total_warps, int rows_per_warp, int nc, int64_t n_rows, const int32_t* m_cols,
                              const float* m_vals, const int64_t* edge_offsets, const double* b, double* x,
                              int restart, int max_iters, double tol, int use_graph, void* workspace,
                              size_t workspace_bytes, mb_gmres_info* info, void* stream) {
    MB_REQUIRE(n_mesh > 0 && nc > 0 && n_rows > 0, "bad sizes");
    MB_REQUIRE(z && desc && goff && b && x && workspace && m_cols && m_vals && edge_offsets, "null pointer argument");
    int64_t it = 0, cyc = 0;
    double rr = 0.0;
    int st = 1;
    const int rc = gmres_blockdiag_pc(z, desc, goff, n_mesh, total_warps, rows_per_warp, nc, n_rows, m_cols, m_vals,
                                      edge_offsets, b, x, restart, max_iters, tol, use_graph != 0, workspace,
                                      workspace_bytes, &it, &cyc, &rr, &st, as_stream(stream));
    if (rc == MB_OK && info) {
        info->iterations = it;
        info->restarts = cyc;
        info->rel_residual = rr;
        info->status = st;
        info->reserved = 0;
    }
    return rc;
}

int mb_gmres_blockdiag_aug_c64(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh,
                               int64_t total_warps, int rows_per_warp, int nc, int64_t n_rows, const int32_t* m_cols,
                               const float* m_vals, const int64_t* edge_offsets, const float* aug_q,
                               const float* aug_ut, int aug_k, const double* b, double* x, int restart, int max_iters,
                               double tol, int use_graph, void* workspace, size_t workspace_bytes, mb_gmres_info* info,
                               void* stream) {
    MB_REQUIRE(n_mesh > 0 && nc > 0 && n_rows > 0, "bad sizes");
    MB_REQUIRE(z && desc && goff && b && x && workspace && aug_q && aug_ut, "null pointer argument");
    int64_t it = 0, cyc = 0;
    double rr = 0.0;
    int st = 1;
    const int rc = gmres_blockdiag_aug(z, desc, goff, n_mesh, total_warps, rows_per_warp, nc, n_rows, m_cols, m_vals,
                                       edge_offsets, aug_q, aug_ut, aug_k, b, x, restart, max_iters, tol,
                                       use_graph != 0, workspace, workspace_bytes, &it, &cyc, &rr, &st,
                                       as_stream(stream));
    if (rc == MB_OK && info) {
        info->iterations = it;
        info->restarts = cyc;
        info->rel_residual = rr;
        info->status = st;
        info->reserved = 0;
    }
    return rc;
}

int mb_mom_sym_zmat_batched_rows_c64(const float* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc,
                                     const double* ks, int n_mesh, const int32_t* schedule,
                                     const int64_t* block_offsets, int64_t total_blocks, int rows_per_block,
                                     const int32_t* near_pairs, int64_t n_near, float* z, void* stream) {
    MB_REQUIRE(n_mesh >= 0 && total_blocks >= 0 && n_near >= 0, "bad sizes");
    if (n_mesh == 0) return MB_OK;
    MB_REQUIRE(verts && faces && fei && desc && ks && schedule && block_offsets && z, "null pointer argument");
    MB_REQUIRE(n_near == 0 || near_pairs, "null near-pair list");
    return launch_mom_sym_rows_batched(verts, faces, fei, desc, ks, n_mesh, schedule, block_offsets, total_blocks,
                                       rows_per_block, near_pairs, n_near, z, as_stream(stream));
}

int mb_half_copy_c64(const float* z, int64_t count, void* z_half, float* scale, void* stream) {
    return half_copy_c64(z, count, z_half, scale, as_stream(stream));
}

int mb_panel_relation(const int32_t* faces, int64_t n_faces, uint8_t* relations, void* stream) {
    MB_REQUIRE(n_faces >= 0, "bad sizes");
    if (n_faces == 0) return MB_OK;
    MB_REQUIRE(faces && relations, "null pointer argument");
    return launch_panel_relation(faces, n_faces, relations, as_stream(stream));
}

}  // extern "C"
