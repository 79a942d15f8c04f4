/*
 * mesh_bem_gb300.h -- C ABI of libmeshbem_gb300.so, the sm_103a (GB300) implementation of
 * the GeCao/Mesh-Ferrofluid boundary-element hot path (RWG method of moments and 3D
 * Laplace single/double-layer assembly).
 *
 * Conventions (all entry points):
 *   - Array arguments are DEVICE pointers to contiguous row-major data; sizes are element
 *     counts.  Faces and face-edge indices are int32, everything else float (f32 / c64
 *     variants) or double (f64 / c128 variants).  "Interleaved complex" arrays store
 *     (re, im) pairs.
 *   - `stream` is a cudaStream_t passed as void*; NULL means the legacy default stream.
 *     Every call is asynchronous with respect to the host.
 *   - Return value: MB_OK (0) or an MB_ERR_* code; mb_last_error() returns the message of
 *     the calling thread's last failure.  Invalid arguments are rejected before any launch.
 *   - Outputs written with "=" are overwritten; outputs documented as "accumulated (+=)"
 *     must be zeroed by the caller (as the reference's Python wrappers do with torch.zeros).
 * The reference interface each entry point replaces is cited as file:line within the
 * reference project.
 */
#ifndef MESH_BEM_GB300_H
#define MESH_BEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MB_ABI_VERSION 1

#define MB_OK 0
#define MB_ERR_ARG 1         /* invalid argument: null pointer, bad size or range */
#define MB_ERR_CUDA 2        /* CUDA launch / runtime error */
#define MB_ERR_UNSUPPORTED 3 /* unsupported rule order, layer or kernel kind */
#define MB_ERR_SIZE 4        /* problem too large for one launch */

/* Message of the calling thread's last failure ("" if none). */
const char* mb_last_error(void);
/* MB_ABI_VERSION of the loaded library. */
int mb_abi_version(void);

/* ---- Reference-op drop-ins (src/mesh_BEM/cuda/mesh_MOM_3d.cpp:111-121) -------------- */

/* Replaces create_MOM_Zmat_3d_forward (mesh_MOM_3d.cpp:52-77; kernel mesh_MOM_3d.cu:332-496).
 * EFIE + MFIE face-edge matrix with the collapsed Gauss rule: test rule gp_x/gw_x (n_x
 * nodes on [0,1]), source rule gp_y/gw_y (n_y nodes), n_x, n_y <= 16.
 * z_real, z_imag: [batch, 3F, 3F] (row = test face*3 + local edge), overwritten; every
 * batch slice receives the same matrix, as in the reference. */
int mb_mom_zmat_fe_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                       const float* face_areas, const float* face_normals, const float* gp_x,
                       const float* gw_x, int n_x, const float* gp_y, const float* gw_y, int n_y,
                       double wavenumber, int64_t batch, float* z_real, float* z_imag, void* stream);
int mb_mom_zmat_fe_f64(const double* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                       const double* face_areas, const double* face_normals, const double* gp_x,
                       const double* gw_x, int n_x, const double* gp_y, const double* gw_y, int n_y,
                       double wavenumber, int64_t batch, double* z_real, double* z_imag, void* stream);

/* Replaces create_MOM_rhs_3d_forward (mesh_MOM_3d.cpp:15-36; kernel mesh_MOM_3d.cu:244-330)
 * with the reference's hard-coded plane wave (mesh_MOM_3d.cu:24-70).
 * rhs_real, rhs_imag: [batch, F, 3], overwritten. */
int mb_mom_rhs_fe_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                      const float* face_areas, const float* face_normals, const float* gp,
                      const float* gw, int n, double wavenumber, int64_t batch, float* rhs_real,
                      float* rhs_imag, void* stream);
int mb_mom_rhs_fe_f64(const double* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                      const double* face_areas, const double* face_normals, const double* gp,
                      const double* gw, int n, double wavenumber, int64_t batch, double* rhs_real,
                      double* rhs_imag, void* stream);

/* Replaces interpolate_Icoeff_to_Js_3d_forward (mesh_MOM_3d.cpp:90-109; kernel
 * mesh_MOM_3d.cu:498-565).  i_real, i_imag: [batch, n_edges]; js_real, js_imag:
 * [batch, 3F, 3], accumulated (+=). */
int mb_mom_interp_js_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                         const int32_t* face_edge_indices, const float* face_areas,
                         const float* i_real, const float* i_imag, int64_t n_edges, int64_t batch,
                         float* js_real, float* js_imag, void* stream);
int mb_mom_interp_js_f64(const double* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                         const int32_t* face_edge_indices, const double* face_areas,
                         const double* i_real, const double* i_imag, int64_t n_edges, int64_t batch,
                         double* js_real, double* js_imag, void* stream);

/* ---- RWG-space operators (fuse the reference's scatter_add_ steps) ------------------- */

/* Replaces MeshMOMZmatKernel.apply + Zmn.scatter_add_ (src/mesh_BEM/kernel_functions.py:39-74,
 * src/mesh_BEM/mesh_BEM_solver_3d.py:128-147): assembles face-edge rows [row_begin, row_end)
 * of the same matrix as mb_mom_zmat_fe_* straight into the RWG matrix
 * z[fei[row], fei[col]], interleaved complex [n_edges, n_edges], accumulated (+=). */
int mb_mom_zmat_rwg_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                        const float* face_areas, const float* face_normals,
                        const int32_t* face_edge_indices, int64_t n_edges, const float* gp_x,
                        const float* gw_x, int n_x, const float* gp_y, const float* gw_y, int n_y,
                        double wavenumber, int64_t row_begin, int64_t row_end, float* z, void* stream);
int mb_mom_zmat_rwg_c128(const double* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                         const double* face_areas, const double* face_normals,
                         const int32_t* face_edge_indices, int64_t n_edges, const double* gp_x,
                         const double* gw_x, int n_x, const double* gp_y, const double* gw_y, int n_y,
                         double wavenumber, int64_t row_begin, int64_t row_end, double* z,
                         void* stream);

/* Ordered face pairs sharing at least one vertex (each face with itself), sorted by first
 * face then second: the nonzeros of compute_panel_relation (src/utils/mesh_utils.py:700-725)
 * in row-major order -- the near-pair list of the symmetric-rule operators -- in O(F) memory.
 * Two calls on one workspace of mb_shared_vertex_pairs_workspace_bytes bytes: _count builds
 * the vertex-face incidences and per-face offsets and returns the list length in *n_pairs
 * (host memory; the stream is synchronised), _fill writes pairs [n_pairs, 2] int32.  Vertex
 * ids outside [0, n_verts) fail with MB_ERR_ARG. */
int64_t mb_shared_vertex_pairs_workspace_bytes(int64_t n_faces, int64_t n_verts);
int mb_shared_vertex_pairs_count(const int32_t* faces, int64_t n_faces, int64_t n_verts, void* workspace,
                                 int64_t workspace_bytes, int64_t* n_pairs, void* stream);
int mb_shared_vertex_pairs_fill(const int32_t* faces, int64_t n_faces, int64_t n_verts, void* workspace,
                                int32_t* pairs, void* stream);

/* No counterpart in the reference (its scatter_add_ runs after the whole face-edge matrix
 * exists).  edge_rows [2 n_edges + 1] int32: for Z row m (edge m) the face-edge rows 3f + e
 * of its faces (smaller first; -1 for a missing second face); edge_rows[2 n_edges] = 1 when
 * some edge has more than two faces (the edge-row operators below then do not apply). */
int mb_mom_edge_rows(const int32_t* face_edge_indices, int64_t n_faces, int64_t n_edges, int32_t* edge_rows,
                     void* stream);
/* The same matrix as mb_mom_zmat_rwg_c64, built Z row by Z row: rows [m_begin, m_end) of z
 * (accumulated), each entry's (up to two) face-edge contributions summed before one atomic;
 * float32 meshes with the gaussQR 2-5 rules (n_x = gaussQR, n_y = gaussQR - 1). */
int mb_mom_zmat_rwg_edges_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                              const float* face_areas, const float* face_normals,
                              const int32_t* face_edge_indices, const int32_t* edge_rows, int64_t n_edges,
                              const float* gp_x, const float* gw_x, int n_x, const float* gp_y,
                              const float* gw_y, int n_y, double wavenumber, int64_t m_begin, int64_t m_end,
                              float* z, void* stream);
/* The same matrix in gather form: thread (m, n) sums the (up to 2 x 2) face-edge entries of
 * Z[m, n] and writes the entry once (no atomics): rows [m_begin, m_end) of z are OVERWRITTEN
 * (no zeroing needed; half the DRAM traffic of the edge order, ~3 % slower at 20480 faces).
 * edge_rows from mb_mom_edge_rows; float32 meshes, gaussQR 2-5. */
int mb_mom_zmat_rwg_gather_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                               const float* face_areas, const float* face_normals, const int32_t* edge_rows,
                               int64_t n_edges, const float* gp_x, const float* gw_x, int n_x, const float* gp_y,
                               const float* gw_y, int n_y, double wavenumber, int64_t m_begin, int64_t m_end,
                               float* z, void* stream);
/* Z into host memory z_host [n_edges, n_edges] complex64 (pinned for overlap): the rows are
 * assembled in `chunks` ranges into the device scratch z_dev [n_edges, n_edges]
 * and each range is copied to z_host on a second stream while the next one is assembled; edge_rows device
 * scratch [2 n_edges + 1].  Meshes with an edge of more than two faces, or rules without an
 * edge-row instance, are assembled face row by face row and copied once.  Returns when the
 * work is queued; the calling stream waits for the last copy. */
int mb_mom_zmat_rwg_to_host_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                                const float* face_areas, const float* face_normals,
                                const int32_t* face_edge_indices, int64_t n_edges, const float* gp_x,
                                const float* gw_x, int n_x, const float* gp_y, const float* gw_y, int n_y,
                                double wavenumber, int32_t* edge_rows, float* z_dev, float* z_host, int chunks,
                                void* stream);

/* Replaces MeshMOMRhsKernel.apply + rhs.scatter_add_ (kernel_functions.py:90-121,
 * mesh_BEM_solver_3d.py:149-164) for n_rhs plane waves at once.  waves: device array of
 * n_rhs records of 9 doubles (k*khat[3], E polarisation[3], H = khat x E / eta [3]);
 * rhs: interleaved complex [n_edges, n_rhs], accumulated (+=). */
int mb_mom_rhs_rwg_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                       const float* face_areas, const float* face_normals,
                       const int32_t* face_edge_indices, int64_t n_edges, const float* gp,
                       const float* gw, int n, const double* waves, int n_rhs, float* rhs,
                       void* stream);
int mb_mom_rhs_rwg_c128(const double* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                        const double* face_areas, const double* face_normals,
                        const int32_t* face_edge_indices, int64_t n_edges, const double* gp,
                        const double* gw, int n, const double* waves, int n_rhs, double* rhs,
                        void* stream);

/* Replaces MeshMOMInterpolateJsKernel.apply + vert_Js.scatter_add_ (kernel_functions.py:137-171,
 * mesh_BEM_solver_3d.py:177-192).  i_coeff: interleaved complex [batch, n_edges];
 * vert_js: interleaved complex [batch, n_verts, 3], accumulated (+=). */
int mb_mom_interp_vert_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                           const int32_t* face_edge_indices, const float* face_areas,
                           const float* i_coeff, int64_t n_edges, int64_t batch, float* vert_js,
                           void* stream);
int mb_mom_interp_vert_c128(const double* verts, int64_t n_verts, const int32_t* faces,
                            int64_t n_faces, const int32_t* face_edge_indices,
                            const double* face_areas, const double* i_coeff, int64_t n_edges,
                            int64_t batch, double* vert_js, void* stream);

/* ---- EFIE with a symmetric rule and singularity extraction (new capability) ---------- */

/* No single reference counterpart: the reference's only rule is the per-edge collapsed
 * Gauss rule above.  These build the EFIE part of the reference's operator (its terms
 * jk G f_m.f_n - (j/k) G div f_m div f_n, mesh_MOM_3d.cu:474-480, RWG convention :154-242)
 * with the 7-point degree-5 rule on both triangles.
 * mb_mom_sym_zmat_rwg_*: every pair (test face in [face_begin, face_end), any source face)
 *   that shares no vertex, in the working precision, accumulated (+=) into z
 *   (interleaved complex [n_edges, n_edges]).
 * mb_mom_sym_near_*: the pairs listed in `pairs` ([n_pairs, 2] int32 (test, source); give
 *   every pair that shares a vertex, including each face with itself), in FP64 with the
 *   1/R part integrated in closed form, accumulated (+=) into z.
 * mb_mom_sym_rhs_rwg_*: EFIE excitation of n_rhs plane waves (records as for
 *   mb_mom_rhs_rwg_*), accumulated (+=) into rhs [n_edges, n_rhs]. */
int mb_mom_sym_zmat_rwg_c64(const float* verts, int64_t n_verts, const int32_t* faces,
                            int64_t n_faces, const int32_t* face_edge_indices, int64_t n_edges,
                            double wavenumber, int64_t face_begin, int64_t face_end, float* z,
                            void* stream);
int mb_mom_sym_zmat_rwg_c128(const double* verts, int64_t n_verts, const int32_t* faces,
                             int64_t n_faces, const int32_t* face_edge_indices, int64_t n_edges,
                             double wavenumber, int64_t face_begin, int64_t face_end, double* z,
                             void* stream);
int mb_mom_sym_near_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                        const int32_t* face_edge_indices, int64_t n_edges, const int32_t* pairs,
                        int64_t n_pairs, double wavenumber, float* z, void* stream);
int mb_mom_sym_near_c128(const double* verts, int64_t n_verts, const int32_t* faces,
                         int64_t n_faces, const int32_t* face_edge_indices, int64_t n_edges,
                         const int32_t* pairs, int64_t n_pairs, double wavenumber, double* z,
                         void* stream);
/* The whole symmetric-rule Z (complex64: separated pairs + the near pairs, sorted by test
 * face as mb_near_pairs / near_pairs give them) into pinned host memory z_host [E, E] with the
 * copy overlapped: test faces are assembled in `chunks` ranges into the device scratch z_dev
 * [E, E], and after each range the Z rows whose faces are all done are written to z_host by a
 * drain kernel on a second stream.  The calling stream waits for the last row. */
int mb_mom_sym_zmat_rwg_to_host_c64(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                                    const int32_t* face_edge_indices, int64_t n_edges, double wavenumber,
                                    const int32_t* pairs, int64_t n_pairs, float* z_dev, float* z_host,
                                    int chunks, void* stream);
int mb_mom_sym_rhs_rwg_c64(const float* verts, int64_t n_verts, const int32_t* faces,
                           int64_t n_faces, const int32_t* face_edge_indices, int64_t n_edges,
                           const double* waves, int n_rhs, float* rhs, void* stream);
int mb_mom_sym_rhs_rwg_c128(const double* verts, int64_t n_verts, const int32_t* faces,
                            int64_t n_faces, const int32_t* face_edge_indices, int64_t n_edges,
                            const double* waves, int n_rhs, double* rhs, void* stream);

/* ---- Radiated field (post-solve) ---------------------------------------------------- */

/* Replaces the scattered-field sum after solve_MOM (demo/demo_Helmholtz_MOM_3d.py:246-257,
 * gradG_y / G of src/utils/functions.py:807-868):
 *   h[p] = sum_v vert_areas[v] * ( js[v] x gradG_y(k, points[p], verts[v]) ),
 * gradG_y = e^{+jkR} (1 + jkR) / (4 pi R^2) * (p - v)/R, vertices closer than 1e-6 skipped.
 * points [n_points, 3], verts [n_verts, 3], vert_areas [n_verts]; js: interleaved complex
 * [n_verts, 3]; h: interleaved complex [n_points, 3], overwritten. */
int mb_radiate_h_c64(const float* points, int64_t n_points, const float* verts,
                     const float* vert_areas, const float* js, int64_t n_verts, double wavenumber,
                     float* h, void* stream);
int mb_radiate_h_c128(const double* points, int64_t n_points, const double* verts,
                      const double* vert_areas, const double* js, int64_t n_verts,
                      double wavenumber, double* h, void* stream);

/* ---- Closest-hit ray queries (replaces the Vulkan ray-query plugin) ------------------ */

/* Replaces VulkanRayTracing.RayQueryApp (src/vulkan_ray_tracing/pybind.cpp:14-28;
 * QueryForLOS / QueryForNLOS at ray_query_App.hpp:881-1000; shaders raygen.rgen:23-64,
 * closesthit.rchit, miss.rmiss).  mb_ray_bvh_build_f32 builds a linear BVH of the mesh in a
 * caller-owned, 256-byte aligned device buffer of mb_ray_bvh_bytes(n_faces) bytes; the
 * finished buffer is self-contained (the mesh arrays are not read by queries).
 * mb_ray_query_f32 casts n_rows x n_cols rays: ray (r, c) starts at origins[r] and runs
 * along dirs[r * n_cols + c] (normalised inside); opaque, no culling, hits with t in
 * [tmin, tmax].  out (16-byte aligned): [n_rows * n_cols, 4] float (face index, 0, 0,
 * distance) or (-1, 0, 0, -1) on a miss, as the plugin returns.  Equal distances keep the
 * lower face index.  mb_ray_status reports (synchronously) whether any traversal since the
 * build stopped early (bit 0: 64-entry stack full; bit 1: more visits than the tree has
 * nodes, i.e. the buffer does not hold a BVH of n_faces faces). */
size_t mb_ray_bvh_bytes(int64_t n_faces);
int mb_ray_bvh_build_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                         void* bvh, size_t bvh_bytes, void* stream);
int mb_ray_query_f32(const void* bvh, int64_t n_faces, const float* origins, const float* dirs,
                     int64_t n_rows, int64_t n_cols, double tmin, double tmax, float* out, void* stream);
int mb_ray_status(const void* bvh, int64_t n_faces, int32_t* overflow, void* stream);

/* ---- Tensor-core (tcgen05) multi-right-hand-side product ------------------------------ */

/* Self-test of the tcgen05 path: one 128 x 256 x 32 kind::tf32 tile with the operands in
 * the 128-byte-swizzled K-major shared-memory layout, accumulated in TMEM and read back;
 * *max_rel_err receives the largest |D - A B^T| / sum |a b| against a double product
 * (expected ~1e-7: TF32-exact inputs, FP32 accumulation).  Allocates and frees a few
 * hundred KB of device memory; synchronous. */
int mb_tc_selftest(double* max_rel_err, void* stream);

/* Split of an fp32 array into TF32 parts: hi = x rounded to TF32, lo = TF32(x - hi).
 * Applied once to the impedance matrix (viewed as fp32 [n, 2n]) before mb_cgemm_tf32x3. */
int mb_split_tf32(const float* src, int64_t count, float* hi, float* lo, void* stream);

/* Multi-right-hand-side product for the block / many-incidence solves (no counterpart in
 * the reference, which solves one right-hand side with torch.linalg.solve,
 * mesh_BEM_solver_3d.py:174): Y = Z X with Z complex64 [n, n] given by its TF32 split
 * (z_hi, z_lo from mb_split_tf32 of Z viewed as fp32 [n, 2n]), X, Y complex64 [n, m]
 * interleaved.  tcgen05 kind::tf32 products A_hi B_hi + A_hi B_lo + A_lo B_hi with FP32
 * accumulation in TMEM (FP32-class accuracy); TMA-fed, one 128 x 256 tile per CTA.
 * n even; operands 16-byte aligned.  workspace: mb_cgemm_workspace_bytes(n, m) bytes
 * (the split, reordered right-hand sides and a status word); mb_cgemm_status reads that
 * status (synchronous; nonzero = a pipeline wait ran out and Y is incomplete). */
size_t mb_cgemm_workspace_bytes(int64_t n, int64_t m);
int mb_cgemm_tf32x3(const float* z_hi, const float* z_lo, int64_t n, const float* x, int64_t m, float* y,
                    void* workspace, size_t workspace_bytes, void* stream);
int mb_cgemm_status(void* workspace, int64_t n, int64_t m, int32_t* status, void* stream);


/* ---- Learned initial guess: kernels of the message-passing network ----------------------
 * (no counterpart in the reference).  Row-major matrices; dtype flags 1 = bf16, 0 = fp32.
 * mb_gnn_gemm: y[n, m] = act(x[n, k] w[k, m] + bias) (w [m, k] used transposed when
 * trans_w); FP32 accumulation; relu 0/1; bias may be NULL.  Supported: bf16 x bf16 ->
 * bf16 or fp32; fp32 x bf16^T -> fp32; fp32 x fp32 (either orientation) -> fp32.
 * mb_gnn_gemm_tn: dw[k, m] += x[n, k]^T dy[n, m] (FP32 atomics).  mb_gnn_colsum:
 * db[m] += sum_n dy[n, m].  mb_gnn_aggregate: out[n] = [h[n], mean of h over nbr[n, 0..3]
 * (-1 = none)] (bf16, out [n, 2f]).  mb_gnn_aggregate_bwd: its adjoint into dh (fp32,
 * accumulated).  mb_gnn_relu_bwd: dz = dy where y > 0.  mb_gnn_adam: one Adam step on fp32
 * master weights (step counts from 1), refreshing the bf16 copy when w_bf16 != NULL. */
int mb_gnn_gemm(const void* x, int x_bf16, const void* w, int w_bf16, int trans_w, const float* bias,
                int64_t n, int k, int m, int relu, void* y, int y_bf16, void* stream);
int mb_gnn_gemm_tn(const void* x, int x_bf16, const float* dy, int64_t n, int k, int m, float* dw,
                   void* stream);
int mb_gnn_colsum(const float* dy, int64_t n, int m, float* db, void* stream);
int mb_gnn_aggregate(const void* h, const int32_t* nbr, int64_t n, int f, void* out, void* stream);
int mb_gnn_aggregate_bwd(const float* dcat, const int32_t* nbr, int64_t n, int f, float* dh, void* stream);
int mb_gnn_relu_bwd(const void* y, const float* dy, int64_t count, float* dz, void* stream);
int mb_gnn_adam(float* w, float* m1, float* m2, const float* g, int64_t count, double lr, double beta1,
                double beta2, double eps, int step, void* w_bf16, void* stream);

/* ---- Dense iterative solve (replaces torch.linalg.solve, mesh_BEM_solver_3d.py:174) -- */

/* Outcome of mb_gmres_c64. status: 0 converged to tol, 1 stopped at max_iters. */
typedef struct mb_gmres_info {
    int64_t iterations;  /* Arnoldi steps (matrix-vector products with Z) */
    int64_t restarts;    /* restart cycles, each started from an FP64 residual */
    double rel_residual; /* ||b - Z x|| / ||b|| in FP64 at return */
    int32_t status;
    int32_t reserved;
} mb_gmres_info;

/* Device workspace (bytes) mb_gmres_c64 needs for n unknowns and restart length m. */
size_t mb_gmres_workspace_bytes(int64_t n, int restart);

/* Replaces torch.linalg.solve(Zmn, rhs) (src/mesh_BEM/mesh_BEM_solver_3d.py:174).
 * GMRES(restart) on Z x = b with Z interleaved complex64 [n, n]: FP32 matrix-vector
 * products, FP64 Arnoldi (CGS2) and Givens rotations, and an FP64 residual b - Z x at the
 * start of every restart cycle (iterative refinement).  b, x: interleaved complex128 [n];
 * x holds the initial guess on entry and the solution on return.  restart in [1, 128].
 * Runs on `stream` and returns after synchronising it (the host drives the Arnoldi loop).
 * workspace: >= mb_gmres_workspace_bytes(n, restart) bytes of device memory owned by the
 * caller.  info (host pointer, may be NULL) receives the outcome. */
int mb_gmres_c64(const float* z, int64_t n, const double* b, double* x, int restart, int max_iters,
                 double tol, void* workspace, size_t workspace_bytes, mb_gmres_info* info,
                 void* stream);

/* The same solver for a real system A x = b (the Laplace single-layer collocation system;
 * the reference solves its Laplace systems with torch.linalg.solve,
 * mesh_BEM_solver_3d.py:345): A float32 (FP32 products) or float64 (FP64 products)
 * [n, n] row-major; b, x float64 [n] (x: initial guess in, solution out).  Workspace:
 * mb_gmres_real_workspace_bytes(n, restart) bytes. */
size_t mb_gmres_real_workspace_bytes(int64_t n, int restart);
int mb_gmres_f32(const float* a, int64_t n, const double* b, double* x, int restart, int max_iters,
                 double tol, void* workspace, size_t workspace_bytes, mb_gmres_info* info,
                 void* stream);
int mb_gmres_f64(const double* a, int64_t n, const double* b, double* x, int restart, int max_iters,
                 double tol, void* workspace, size_t workspace_bytes, mb_gmres_info* info,
                 void* stream);

/* GMRES(restart) for m right-hand sides in lockstep (many incidences on one mesh; the
 * reference solves one right-hand side per dense LU, mesh_BEM_solver_3d.py:174): Z X = B
 * with Z given by its TF32 split (as for mb_cgemm_tf32x3), B, X complex128 [n, m]
 * interleaved (X: initial guess in, solution out).  Every Arnoldi step multiplies all m
 * basis vectors with one tensor-core product; the basis is complex64 and CGS2 runs in FP32
 * with FP64 sums across rows (TMA-streamed kernels), the Hessenberg matrix, the Givens
 * rotations and X are FP64 per column; each restart cycle starts from B - Z X through the
 * same product (attainable relative residual ~1e-6).  info: total Arnoldi steps, restart
 * cycles, the largest per-column relative residual, status 0 when every column reached
 * tol.  Workspace: mb_gmres_multi_workspace_bytes(n, m, restart) bytes (the basis
 * dominates: 8 n m' (restart + 1), m' = m rounded up to even). */
size_t mb_gmres_multi_workspace_bytes(int64_t n, int64_t m, int restart);
int mb_gmres_multi_c64(const float* z_hi, const float* z_lo, int64_t n, const double* b, double* x,
                       int64_t m, int restart, int max_iters, double tol, void* workspace,
                       size_t workspace_bytes, mb_gmres_info* info, void* stream);

/* ---- Many meshes at once (batched assembly and solve; no counterpart in the reference,
 * which handles one mesh per solver call) ---------------------------------------------------
 * The meshes are packed into one vertex array and one face array (vertex ids global);
 * fei [sum F_i, 3] holds each mesh's local RWG edge ids; desc [n_mesh, 6] int64 =
 * (first face, faces F_i, edges E_i, offset of Z_i in the flat block-diagonal array in
 * complex entries, first block of the mesh in the regular launch = sum over earlier meshes
 * of F_j ceil(F_j / 128), first right-hand-side column); ks [n_mesh] the wavenumbers.
 * Z_i is row-major with the even row pitch P_i = E_i + (E_i & 1) (the offsets are sums of
 * E_j P_j); a padding entry is never written.
 * mb_mom_sym_zmat_batched_*: the symmetric-rule EFIE (as mb_mom_sym_zmat_rwg_* +
 * mb_mom_sym_near_*) of every mesh in one launch of each kernel, accumulated into the flat
 * array (caller zeroes); total_blocks = the block count above; near_pairs [n_near, 2]
 * global face ids of all pairs sharing a vertex.
 * mb_mom_sym_rhs_batched_*: nrhs plane waves per mesh (waves [n_mesh * nrhs, 9]) into the
 * padded block rhs [max E_i, ld] (row = local edge, column desc[i][5] + r; accumulated). */
int mb_mom_sym_zmat_batched_c64(const float* verts, const int32_t* faces, const int32_t* fei,
                                const int64_t* desc, const double* ks, int n_mesh, int64_t total_blocks,
                                const int32_t* near_pairs, int64_t n_near, float* z, void* stream);
int mb_mom_sym_zmat_batched_c128(const double* verts, const int32_t* faces, const int32_t* fei,
                                 const int64_t* desc, const double* ks, int n_mesh, int64_t total_blocks,
                                 const int32_t* near_pairs, int64_t n_near, double* z, void* stream);
int mb_mom_sym_rhs_batched_c64(const float* verts, const int32_t* faces, const int32_t* fei,
                               const int64_t* desc, int n_mesh, int64_t total_faces, const double* waves,
                               int nrhs, int64_t ld, float* rhs, void* stream);
int mb_mom_sym_rhs_batched_c128(const double* verts, const int32_t* faces, const int32_t* fei,
                                const int64_t* desc, int n_mesh, int64_t total_faces, const double* waves,
                                int nrhs, int64_t ld, double* rhs, void* stream);

/* The same float matrices as mb_mom_sym_zmat_batched_c64 with the separated pairs in the rows
 * layout: a block owns rows_per_block (8, 16 or 32) test faces of one mesh, staged in shared
 * memory, and 128 of its source faces.  schedule [n_mesh] int32 is the order in which the
 * meshes' blocks are laid out and block_offsets [n_mesh + 1] int64 the first block of the j-th
 * scheduled mesh (mesh schedule[j], of F faces, takes ceil(F / rows_per_block) * ceil(F / 128)
 * blocks; the last entry = total_blocks).  Chosen by MeshBatch.autotune_assembly.
 * Accumulated into z (caller zeroes). */
int mb_mom_sym_zmat_batched_rows_c64(const float* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc,
                                     const double* ks, int n_mesh, const int32_t* schedule,
                                     const int64_t* block_offsets, int64_t total_blocks, int rows_per_block,
                                     const int32_t* near_pairs, int64_t n_near, float* z, void* stream);

/* The reference's operator and rule (as mb_mom_zmat_rwg_c64 / mb_mom_rhs_rwg_c64) for every
 * mesh of the batch in one launch each: face_areas, face_normals per packed face;
 * block_offsets [n_mesh + 1] = first block of each mesh with 3 F_i rows of
 * ceil(3 F_i / 128) blocks (total_blocks = the last entry); gaussQR (nx = gaussQR, ny =
 * gaussQR - 1) in {2, 3, 4, 5}.  Excitation <f, E + n x H> of nrhs waves per mesh (waves
 * [n_mesh * nrhs, 9]) into the padded block rhs [max E_i, ld]. */
int mb_mom_ref_zmat_batched_c64(const float* verts, const int32_t* faces, const float* face_areas,
                                const float* face_normals, const int32_t* fei, const int64_t* desc,
                                const int64_t* block_offsets, int64_t total_blocks, const double* ks,
                                int n_mesh, const float* gpx, const float* gwx, int nx, const float* gpy,
                                const float* gwy, int ny, float* z, void* stream);
/* The same matrices from one resident grid (SMs x blocks per SM) whose blocks take the
 * (mesh, row, 128-column tile) work items of block_offsets from a device counter until they
 * run out (a counter of 8 bytes allocated stream-ordered per call).  Chosen against the grid
 * form by MeshBatch.autotune_assembly. */
int mb_mom_ref_zmat_batched_persistent_c64(const float* verts, const int32_t* faces, const float* face_areas,
                                           const float* face_normals, const int32_t* fei, const int64_t* desc,
                                           const int64_t* block_offsets, int64_t total_blocks, const double* ks,
                                           int n_mesh, const float* gpx, const float* gwx, int nx, const float* gpy,
                                           const float* gwy, int ny, float* z, void* stream);
int mb_mom_ref_rhs_batched_c64(const float* verts, const int32_t* faces, const float* face_areas,
                               const float* face_normals, const int32_t* fei, const int64_t* desc,
                               int n_mesh, int64_t total_faces, const float* gp, const float* gw, int n,
                               const double* waves, int nrhs, int64_t ld, float* rhs, void* stream);

/* Block-diagonal product over the batch: y[r, c] = sum_l Z_i[r, l] x[l, c] for the nc
 * columns of mesh i (x, y complex64 [max E_i, ld], ld >= n_mesh * nc); goff [n_mesh + 1] =
 * first work unit of each mesh with rows_per_warp rows per unit, goff[n_mesh] =
 * total_warps: 1, 2, 4 or 8 (8 for nc <= 4) rows per warp reading Z directly, or 32 rows
 * per block with Z streamed through shared memory by bulk copies (z 16-byte aligned).
 * nc in {1, 2, 4, 8}.  Rows beyond E_i are not written. */
int mb_blockdiag_matvec_c64(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh,
                            int64_t total_warps, const float* x, int64_t ld, int nc, int rows_per_warp,
                            float* y, void* stream);

/* GMRES(restart) on every mesh and right-hand side of the batch in lockstep (the algorithm
 * of mb_gmres_multi_c64 with the block-diagonal product): b, x complex128 [n_rows, n_mesh *
 * nc] padded (rows beyond E_i zero).  use_graph: capture the restart cycle's Arnoldi steps
 * once as a CUDA graph and replay it (no host synchronisation inside a cycle; iterations
 * are counted in whole cycles).  Workspace: mb_gmres_blockdiag_workspace_bytes. */
size_t mb_gmres_blockdiag_workspace_bytes(int64_t n_rows, int64_t m, int restart);
/* Arnoldi steps each column took (while it was active, over all restart cycles) in the last
 * mb_gmres_blockdiag_c64 / mb_gmres_multi_c64 call on `workspace`: int32 [m] into out
 * (device or host memory; stream-ordered). */
int mb_gmres_blockdiag_column_steps(const void* workspace, int64_t n_rows, int64_t m, int restart, int32_t* out,
                                    void* stream);
int mb_gmres_multi_column_steps(const void* workspace, int64_t n, int64_t m, int restart, int32_t* out,
                                void* stream);
int mb_gmres_blockdiag_c64(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh,
                           int64_t total_warps, int rows_per_warp, int nc, int64_t n_rows, const double* b,
                           double* x, int restart, int max_iters, double tol, int use_graph, void* workspace,
                           size_t workspace_bytes, mb_gmres_info* info, void* stream);

/* mb_gmres_blockdiag_c64 with the near-field right preconditioner of every mesh: m_cols /
 * m_vals from mb_spai_build_c64 run on the whole batch (desc rows (first face, F_i, first
 * edge, E_i, offset of Z_i, row pitch)), edge_offsets [n_mesh] int64 the first global edge of
 * each mesh (device); nc in {1, 2, 4, 8}.  Each Arnoldi step multiplies Z_i by M_i V_j; each
 * cycle's update goes through M_i before it is added to X, and each cycle starts from the
 * residual B - Z X by compensated FP32 dot products (FP64-class accuracy, so tolerances below
 * the FP32 product's ~1e-6 are reachable).  Same workspace as mb_gmres_blockdiag_c64 (its size
 * includes the preconditioned vectors). */
int mb_gmres_blockdiag_pc_c64(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh,
                              int64_t total_warps, int rows_per_warp, int nc, int64_t n_rows, const int32_t* m_cols,
                              const float* m_vals, const int64_t* edge_offsets, const double* b, double* x,
                              int restart, int max_iters, double tol, int use_graph, void* workspace,
                              size_t workspace_bytes, mb_gmres_info* info, void* stream);

/* mb_gmres_blockdiag_c64 / _pc_c64 with a fixed augmentation (deflation) subspace per mesh:
 * aug_k (4, 8 or 16) vectors U_i of x-space per mesh, given through the thin QR of their
 * products, Z_i U_i = Q_i R_i: aug_q = Q_i and aug_ut = U_i R_i^{-1}, complex64 [n_rows,
 * n_mesh * aug_k] with mesh i's vectors at columns i * aug_k (rows beyond E_i zero).  Every
 * Arnoldi step removes the Q_i components of the product and keeps them; every cycle starts by
 * adding the residual-minimising combination of U_i to X (at the first cycle this is the
 * least-squares initial guess from U_i); the cycle's update subtracts U_i R_i^{-1} times the
 * kept components (GCRO with a fixed recycled space), so the reported residual is the true
 * one.  m_cols, m_vals and edge_offsets: all null (no preconditioner) or all given (as
 * mb_gmres_blockdiag_pc_c64).  Buffers of (64 + restart + 1) * n_mesh * nc * aug_k * 16 bytes
 * are allocated stream-ordered per call; the workspace is mb_gmres_blockdiag_c64's.
 * New capability beside the dense LU the reference solves with (torch.linalg.solve,
 * mesh_BEM_solver_3d.py:174). */
int mb_gmres_blockdiag_aug_c64(const float* z, const int64_t* desc, const int64_t* goff, int n_mesh,
                               int64_t total_warps, int rows_per_warp, int nc, int64_t n_rows, const int32_t* m_cols,
                               const float* m_vals, const int64_t* edge_offsets, const float* aug_q,
                               const float* aug_ut, int aug_k, const double* b, double* x, int restart, int max_iters,
                               double tol, int use_graph, void* workspace, size_t workspace_bytes, mb_gmres_info* info,
                               void* stream);

/* No counterpart in the reference.  The same solver as mb_gmres_c64 for callers that
 * cannot allocate device memory -- for example a host application or plugin that must
 * budget all GPU memory at start-up, or a foreign-language caller (Go, Java, ...) that has
 * no access to a CUDA allocator.  It takes no workspace and allocates nothing: the device
 * scratch is a fixed array inside this library (about 7 MB, held on every GPU that loads
 * the library until the process exits), sized for at most MB_GMRES_NOALLOC_MAX_N unknowns
 * and restart <= MB_GMRES_NOALLOC_MAX_RESTART; larger requests fail with MB_ERR_SIZE.
 * The first call on each device looks up that array's device address (a one-time set-up
 * with that device current) and keeps it for the life of the process; make that first call
 * before any stream capture.  Calls after cudaDeviceReset() on that device are not supported
 * (the kept address would be stale).  All calls share the array, which keeps the previous
 * call's contents (the solver writes every scratch value before reading it); calls that
 * overlap on the GPU race on it. */
#define MB_GMRES_NOALLOC_MAX_N 8192
#define MB_GMRES_NOALLOC_MAX_RESTART 50
int mb_gmres_c64_noalloc(const float* z, int64_t n, const double* b, double* x, int restart,
                         int max_iters, double tol, mb_gmres_info* info, void* stream);

/* y = Z v: Z interleaved complex64 [n, n], v complex64 [n], y complex128 [n] (FP32 products,
 * FP64 row reduction).  The HBM-bound kernel inside mb_gmres_c64.  Alignment: z, v and y
 * need only the natural alignment of their element type (8 bytes); rows and a v that start
 * on a 16-byte boundary are read 16 bytes at a time, others one complex number at a time
 * (slower), so a view such as X[1:n+1] of a complex64 array is accepted. */
int mb_matvec_c64(const float* z, const float* v, int64_t n, double* y, void* stream);

/* r = b - Z x in FP64: Z complex64 [n, n], x, b, r complex128 [n]. */
int mb_residual_c128(const float* z, const double* x, const double* b, int64_t n, double* r,
                     void* stream);

/* ---- Near-field preconditioner and preconditioned solve (no counterpart in the reference,
 * which factors Z densely with torch.linalg.solve, mesh_BEM_solver_3d.py:174) ------------
 * Sparse approximate inverse M of the RWG matrix, the right preconditioner of
 * mb_pgmres_*: column j of M minimises ||Z[I_j, J_j] m - e_j|| with J_j the edges of the
 * faces sharing a vertex with a face of edge j and I_j the edges of the faces sharing a
 * vertex with those (least squares by Householder QR in FP32, one block per edge).  M is
 * stored as rows of MB_SPAI_WIDTH (local column, complex64 value) pairs, m_cols [E,
 * MB_SPAI_WIDTH] int32 (a row ends at its first -1) and m_vals [E, MB_SPAI_WIDTH]
 * interleaved complex64.  Several meshes at once: desc [n_mesh, 6] int64 = (first face,
 * faces, first edge, edges, offset of Z_i in complex entries, row pitch of Z_i); faces
 * [total_faces, 3] (global vertex ids), fei [total_faces, 3] local edge ids, near_pairs
 * [n_near, 2] (global face ids, sorted by first face; mb_shared_vertex_pairs_*), z the
 * complex64 matrix (blocks).  For one mesh: desc = {0, F, 0, E, 0, E}.  Patterns above
 * MB_SPAI_WIDTH columns or 128 rows keep the edges nearest to edge j.  Workspace:
 * mb_spai_workspace_bytes(total_edges) bytes.  mb_spai_status copies the build's status word
 * into *status (host or device memory; synchronises the stream): bit 0 a pattern was cut
 * to its cap, bit 1 a least-squares block without full column rank, bit 2 a face-edge map
 * with an out-of-range id or an edge without faces or with more than two. */
#define MB_SPAI_WIDTH 48
size_t mb_spai_workspace_bytes(int64_t total_edges);
int mb_spai_build_c64(const float* verts, const int32_t* faces, const int32_t* fei, const int64_t* desc, int n_mesh,
                      int64_t total_faces, int64_t total_edges, const int32_t* near_pairs, int64_t n_near,
                      const float* z, int32_t* m_cols, float* m_vals, void* workspace, size_t workspace_bytes,
                      void* stream);
int mb_spai_status(const void* workspace, int64_t total_edges, int32_t* status, void* stream);
/* y = M v for one mesh (complex64 v, y [n]). */
int mb_spai_apply_c64(const int32_t* m_cols, const float* m_vals, int64_t n, const float* v, float* y,
                      void* stream);

/* GMRES(restart) on Z x = b with the right preconditioner M (m_cols / m_vals from
 * mb_spai_build_c64, or both NULL for none): each restart cycle starts from the refinement
 * residual b - Z x, solves (Z M) u = r and adds M u to x.  The whole cycle runs on the device
 * (CGS2 Arnoldi, Givens rotations, the residual estimate and the back substitution in
 * kernels; Hessenberg matrix, rotations and x in FP64; deterministic block reductions);
 * use_graph = 1 captures it once as a CUDA graph and replays it.  The host reads the solver
 * state once per cycle.
 * mb_pgmres_c64: Z interleaved complex64 [n, n]; FP32 products, complex64 Krylov basis with
 * FP32 Gram-Schmidt products and FP64 sums; the refinement residual by compensated FP32 dot
 * products (exact products and sums, ~1e-13 of sum |Z_ij x_j|).  With z_half (from
 * mb_half_copy_c64) and half_scale, the Arnoldi products read the half-precision copy instead,
 * each cycle ends once its residual estimate has dropped by inner_rtol (e.g. 3e-3; the copy's
 * ~2e-4 relative error bounds what one cycle can gain) and the next cycle restarts from the
 * complex64 residual; pass NULL, NULL, 0 to use Z itself.
 * mb_pgmres_c128: Z interleaved complex128; FP64 products, basis and residual.  z, b, x (and
 * z_half) 16-byte aligned; b, x complex128 [n] (x: initial guess in, solution out).  info as
 * for mb_gmres_c64.  Workspace: mb_pgmres_workspace_bytes(n, restart) bytes. */
size_t mb_pgmres_workspace_bytes(int64_t n, int restart);
int mb_pgmres_c64(const float* z, int64_t n, const void* z_half, const float* half_scale, double inner_rtol,
                  const int32_t* m_cols, const float* m_vals, const double* b, double* x, int restart, int max_iters,
                  double tol, int use_graph, void* workspace, size_t workspace_bytes, mb_gmres_info* info,
                  void* stream);
int mb_pgmres_c128(const double* z, int64_t n, const int32_t* m_cols, const float* m_vals, const double* b,
                   double* x, int restart, int max_iters, double tol, int use_graph, void* workspace,
                   size_t workspace_bytes, mb_gmres_info* info, void* stream);
/* Half-precision copy for mb_pgmres_c64: *scale (device float) = max |Re|, |Im| over the
 * complex64 array z (count complex entries, count even, z 16-byte aligned), and z_half
 * (count pairs of IEEE binary16, interleaved like z, 8-byte aligned) = z / *scale rounded to
 * nearest (magnitudes below 2^-24 of the scale, the smallest binary16 subnormal, become 0). */
int mb_half_copy_c64(const float* z, int64_t count, void* z_half, float* scale, void* stream);

/* ---- Laplace / Helmholtz-BEM layers ------------------------------------------------- */

/* Replaces double_integration_on_panels_3d (src/mesh_BEM/utils/integrations_3d.py:252-452).
 * table: [rows, 5] of (r1x, r2x, r1y, r2y, w*jacobian) -- the sub-domain maps of
 * get_rands_and_jacobian_3d (integrations_3d.py:18-249) flattened; segments (HOST array of
 * 5): the rows of relation r are [segments[r], segments[r+1]) for r = 0 separate,
 * 1 shared vertex, 2 shared edge, 3 same face.  relations: [F, F] uint8
 * (compute_panel_relation, src/utils/mesh_utils.py:700-725) or NULL to derive it from
 * `faces`.  layer: 1 single (G_3d), 2 double (grad_G_y_3d . n of the first panel).
 * order: 0 planar (P0), 1 linear (P1).  kind: 0 Laplace, 1 Helmholtz e^{+jkR}
 * (src/utils/BEM_utils.py:72-172).  Rows [row_begin, row_end) of the first ("y") face.
 * out_real (and out_imag for kind 1): [row_end-row_begin, F, nphi, nphi], overwritten. */
int mb_laplace_panels_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                          const float* face_areas, const float* face_normals, const float* table,
                          const int32_t* segments, const uint8_t* relations, int layer, int order,
                          int kind, double wavenumber, int64_t row_begin, int64_t row_end,
                          float* out_real, float* out_imag, void* stream);
int mb_laplace_panels_f64(const double* verts, int64_t n_verts, const int32_t* faces,
                          int64_t n_faces, const double* face_areas, const double* face_normals,
                          const double* table, const int32_t* segments, const uint8_t* relations,
                          int layer, int order, int kind, double wavenumber, int64_t row_begin,
                          int64_t row_end, double* out_real, double* out_imag, void* stream);

/* Replaces pack_matrix_tight (src/utils/BEM_utils.py:314-357): packed[faces[fy,a], faces[fx,b]]
 * += m[fy, fx, a, b] (P1) or m[fy, fx]/9 (P0).  packed: [n_verts, n_verts] real, or interleaved
 * complex when m_imag != NULL; accumulated (+=). */
int mb_pack_tight_f32(const float* m_real, const float* m_imag, const int32_t* faces, int64_t n_faces,
                      int64_t n_verts, int order, float* packed, void* stream);
int mb_pack_tight_f64(const double* m_real, const double* m_imag, const int32_t* faces,
                      int64_t n_faces, int64_t n_verts, int order, double* packed, void* stream);

/* Hypersingular operator, P1 Galerkin, for the Neumann and mixed branches of
 * MeshBEMSolver3d.solve (src/mesh_BEM/mesh_BEM_solver_3d.py:268-281, 306-341), which the
 * reference declares (hypersingular_layer/hypersingular_layer_3d.py) but never computes
 * (integrations_3d.py:440-442).  Maue's formula: out[fy, fx, a, b] = curl phi_a(fy) .
 * curl phi_b(fx) * v0[fy, fx], with v0 [F, F] the P0 single-layer panel integrals
 * (mb_laplace_panels_* with layer 1, order 0) and curl phi_a = (p_{a+1} - p_{a+2}) / (2 A).
 * out: [F, F, 3, 3], overwritten. */
int mb_laplace_hypersingular_f32(const float* verts, int64_t n_verts, const int32_t* faces,
                                 int64_t n_faces, const float* v0, float* out, void* stream);
int mb_laplace_hypersingular_f64(const double* verts, int64_t n_verts, const int32_t* faces,
                                 int64_t n_faces, const double* v0, double* out, void* stream);

/* The same operator packed like mb_pack_tight_* with order 1, straight from v0 [F, F]:
 * packed[faces[fy,a], faces[fx,b]] += curl phi_a(fy) . curl phi_b(fx) * v0[fy, fx], without
 * storing the [F, F, 3, 3] panels (the matrix MeshBEMSolver3d.solve uses,
 * src/mesh_BEM/mesh_BEM_solver_3d.py:268-281).  packed: [n_verts, n_verts], accumulated (+=);
 * needs 3 * n_verts * sizeof(T) <= 160 KiB of shared memory (MB_ERR_SIZE otherwise). */
int mb_laplace_hypersingular_tight_f32(const float* verts, int64_t n_verts, const int32_t* faces,
                                       int64_t n_faces, const float* v0, float* packed, void* stream);
int mb_laplace_hypersingular_tight_f64(const double* verts, int64_t n_verts, const int32_t* faces,
                                       int64_t n_faces, const double* v0, double* packed, void* stream);

/* Symmetric-rule Laplace operators (an accurate mode next to the reference's rule of
 * double_integration_on_panels_3d, integrations_3d.py:252-452; same output layout):
 * out[fy, fx, a, b] = int_fy int_fx phi_a(y) phi_b(x) k(x, y) for rows fy in
 * [row_begin, row_end), k = 1/(4 pi R) (layer 1) or n_fy.(x - y)/(4 pi R^3) (layer 2),
 * order 0 (P0, nphi 1) or 1 (P1, nphi 3).  7 x 7 points per separated pair; near_pairs
 * [n_near, 2] lists every ordered pair (fy, fx) sharing a vertex (compute_panel_relation
 * > 0), integrated with the inner integral in closed form in FP64.  out:
 * [row_end - row_begin, F, nphi, nphi], overwritten. */
int mb_laplace_sym_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                       int layer, int order, const int32_t* near_pairs, int64_t n_near,
                       int64_t row_begin, int64_t row_end, float* out, void* stream);
int mb_laplace_sym_f64(const double* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                       int layer, int order, const int32_t* near_pairs, int64_t n_near,
                       int64_t row_begin, int64_t row_end, double* out, void* stream);

/* Packed symmetric-rule operators [n_verts, n_verts] (+=) without the [F, F, 3, 3] panels:
 * op 1 single layer and 2 double layer, P1 x P1, equal to mb_pack_tight_* (order 1) of the
 * mb_laplace_sym_* panels; op 3 the hypersingular operator, equal to
 * mb_laplace_hypersingular_tight_* of the P0 single-layer panels.  These are the matrices
 * MeshBEMSolver3d.solve works with (src/mesh_BEM/mesh_BEM_solver_3d.py:197-373, get_Vmat_tight /
 * get_Kmat_tight, single_layer_3d.py and double_layer_3d.py).  Test rows [row_begin, row_end)
 * contribute; near_pairs as for mb_laplace_sym_*.  Needs 3 * n_verts * sizeof(T) <= 160 KiB of
 * shared memory (MB_ERR_SIZE otherwise). */
int mb_laplace_sym_tight_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                             int op, const int32_t* near_pairs, int64_t n_near, int64_t row_begin,
                             int64_t row_end, float* packed, void* stream);
int mb_laplace_sym_tight_f64(const double* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                             int op, const int32_t* near_pairs, int64_t n_near, int64_t row_begin,
                             int64_t row_end, double* packed, void* stream);

/* Single-layer collocation system at face centroids (the Laplace form of the large sphere
 * solve; no counterpart in the reference): out[i - row_begin, j] = int_{T_j} 1/(4 pi
 * |c_i - y|) dS_y, the 7-point rule for faces without a shared vertex; the pairs (i, j)
 * listed in near_pairs [n_near, 2] (every pair sharing a vertex, as for mb_laplace_sym_*)
 * in closed form (FP64).  out: [row_end - row_begin, F], overwritten. */
int mb_laplace_colloc_sl_f32(const float* verts, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                             const int32_t* near_pairs, int64_t n_near, int64_t row_begin,
                             int64_t row_end, float* out, void* stream);
int mb_laplace_colloc_sl_f64(const double* verts, int64_t n_verts, const int32_t* faces,
                             int64_t n_faces, const int32_t* near_pairs, int64_t n_near,
                             int64_t row_begin, int64_t row_end, double* out, void* stream);

/* Replaces compute_panel_relation (src/utils/mesh_utils.py:700-725): relations [F, F] uint8,
 * overwritten. */
int mb_panel_relation(const int32_t* faces, int64_t n_faces, uint8_t* relations, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MESH_BEM_GB300_H */
