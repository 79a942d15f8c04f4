/*
 * mesh_bem_oracle.c -- CPU restatement of the reference's boundary-element hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the smoke
 * check and the CPU-baseline leg of bench.py call it to check the CUDA path.  The
 * product (the CUDA library and its Python host layer) never links, loads or calls it.
 *
 * It restates, loop for loop, what the reference computes (GeCao/Mesh-Ferrofluid):
 *   - kernel_create_MOM_Zmat_3d_forward   src/mesh_BEM/cuda/mesh_MOM_3d.cu:332-496
 *   - kernel_create_MOM_rhs_3d_forward    src/mesh_BEM/cuda/mesh_MOM_3d.cu:244-330
 *   - kernel_interpolate_Icoeff_to_Js_3d_forward  src/mesh_BEM/cuda/mesh_MOM_3d.cu:498-565
 *     with the helpers G :72-95, gradG_y :97-126, gradG_x :128-152, is_Tn_plus :154-165,
 *     RWG :167-206, div_RWG :208-242, calculate_Einc :24-38, calculate_Hinc :40-70
 *   - the scattered-field sum after the solve  demo/demo_Helmholtz_MOM_3d.py:246-257 with
 *     G / gradG_y                           src/utils/functions.py:807-868
 *   - get_rands_and_jacobian_3d           src/mesh_BEM/utils/integrations_3d.py:18-249
 *   - double_integration_on_panels_3d     src/mesh_BEM/utils/integrations_3d.py:252-452
 *     with G_3d / grad_G_y_3d / shape_function  src/utils/BEM_utils.py:72-104,141-207
 *
 * Compiled twice by oracle/build_oracle.py: REAL=double (symbols orc_*_f64) and
 * REAL=float (orc_*_f32).  OpenMP parallelises the outer loops; every output element is
 * written by exactly one thread so results do not depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL double
#endif
#ifndef SFX
#define SFX f64
#endif
/* Math in the working precision: the reference's float build calls the float overloads
   (CUDA's sqrt/cos/sin on float arguments). */
#ifdef ORC_FLOAT
#define R_SQRT(x) sqrtf(x)
#define R_COS(x) cosf(x)
#define R_SIN(x) sinf(x)
#else
#define R_SQRT(x) sqrt(x)
#define R_COS(x) cos(x)
#define R_SIN(x) sin(x)
#endif
#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define ORC(name) CAT(orc_##name, SFX)

static const double ORC_PI = 3.14159265358979323846;

/* ------------------------------------------------------------------------------------ */
/* MoM helpers (mesh_MOM_3d.cu:12-242)                                                  */
/* ------------------------------------------------------------------------------------ */

/* n = t x b  (mesh_MOM_3d.cu:12-22) */
static void ORC(cross3)(const REAL* t, const REAL* b, REAL* n) {
    n[0] = t[1] * b[2] - t[2] * b[1];
    n[1] = t[2] * b[0] - t[0] * b[2];
    n[2] = t[0] * b[1] - t[1] * b[0];
}

/* e^{-jkR}/(4 pi R)  (mesh_MOM_3d.cu:72-95) */
static void ORC(green)(REAL k, const REAL* p1, const REAL* p2, REAL* gr, REAL* gi) {
    REAL d0 = p1[0] - p2[0], d1 = p1[1] - p2[1], d2 = p1[2] - p2[2];
    REAL dist = R_SQRT((d0 * d0 + d1 * d1 + d2 * d2));
    REAL inv = (REAL)1 / dist;
    REAL th = -k * dist;
    *gr = (REAL)(R_COS(th) / (4 * ORC_PI)) * inv;
    *gi = (REAL)(R_SIN(th) / (4 * ORC_PI)) * inv;
}

/* grad_x G = -grad_y G  (mesh_MOM_3d.cu:97-152) */
static void ORC(grad_green_x)(REAL k, const REAL* p1, const REAL* p2, REAL* gr, REAL* gi) {
    REAL r[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
    REAL dist = R_SQRT((r[0] * r[0] + r[1] * r[1] + r[2] * r[2]));
    REAL inv = (REAL)1 / dist;
    REAL th = -k * dist;
    REAL c = R_COS(th), s = R_SIN(th);
    REAL fr = (REAL)((c + th * s) / (4 * ORC_PI)) * inv * inv * inv;
    REAL fi = (REAL)((s - th * c) / (4 * ORC_PI)) * inv * inv * inv;
    for (int a = 0; a < 3; ++a) {
        gr[a] = -(fr * r[a]);
        gi[a] = -(fi * r[a]);
    }
}

/* RWG basis on the triangle (v0 opposite the edge v1->v2); sign + iff v1 < v2
   (mesh_MOM_3d.cu:154-206) */
static void ORC(rwg)(const REAL* x, const REAL* verts, REAL area, int32_t i0, int32_t i1, int32_t i2,
                     REAL* out) {
    const REAL* v0 = verts + 3 * (int64_t)i0;
    const REAL* v1 = verts + 3 * (int64_t)i1;
    const REAL* v2 = verts + 3 * (int64_t)i2;
    REAL e0 = v2[0] - v1[0], e1 = v2[1] - v1[1], e2 = v2[2] - v1[2];
    REAL len = R_SQRT((e0 * e0 + e1 * e1 + e2 * e2));
    REAL sc = len / (2 * area);
    int plus = i1 < i2;
    for (int a = 0; a < 3; ++a) out[a] = (plus ? x[a] - v0[a] : v0[a] - x[a]) * sc;
}

/* divergence of the RWG basis  (mesh_MOM_3d.cu:208-242) */
static REAL ORC(div_rwg)(const REAL* verts, REAL area, int32_t i1, int32_t i2) {
    const REAL* v1 = verts + 3 * (int64_t)i1;
    const REAL* v2 = verts + 3 * (int64_t)i2;
    REAL e0 = v2[0] - v1[0], e1 = v2[1] - v1[1], e2 = v2[2] - v1[2];
    REAL len = R_SQRT((e0 * e0 + e1 * e1 + e2 * e2));
    REAL sc = len / (2 * area);
    return (i1 < i2) ? sc * 2 : -sc * 2;
}

/* ------------------------------------------------------------------------------------ */
/* Face-edge impedance matrix (mesh_MOM_3d.cu:332-496)                                  */
/* Rows [row_begin, row_end) of the [3F, 3F] face-edge matrix, row = f1*3 + e1.          */
/* ------------------------------------------------------------------------------------ */
void ORC(mom_zmat_fe)(const REAL* verts, const int32_t* faces, int64_t nf, const REAL* areas,
                      const REAL* normals, const REAL* gpx, const REAL* gwx, int nx,
                      const REAL* gpy, const REAL* gwy, int ny, double wavenumber,
                      int64_t row_begin, int64_t row_end, REAL* zr, REAL* zi) {
    const REAL k = (REAL)wavenumber;
    const int64_t ncol = 3 * nf;
    const int64_t nrows = row_end - row_begin;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t rr = 0; rr < nrows; ++rr) {
        const int64_t row = row_begin + rr;
        const int64_t f1 = row / 3;
        const int e1 = (int)(row % 3);
        for (int64_t col = 0; col < ncol; ++col) {
            const int64_t f2 = col / 3;
            const int e2 = (int)(col % 3);
            const int same = (f1 == f2);
            const REAL area1 = areas[f1], area2 = areas[f2];
            const REAL* n1 = normals + 3 * f1;
            const int32_t a0 = faces[3 * f1 + e1], a1 = faces[3 * f1 + (e1 + 1) % 3],
                          a2 = faces[3 * f1 + (e1 + 2) % 3];
            const int32_t b0 = faces[3 * f2 + e2], b1 = faces[3 * f2 + (e2 + 1) % 3],
                          b2 = faces[3 * f2 + (e2 + 2) % 3];
            const REAL* A0 = verts + 3 * (int64_t)a0;
            const REAL* A1 = verts + 3 * (int64_t)a1;
            const REAL* A2 = verts + 3 * (int64_t)a2;
            const REAL* B0 = verts + 3 * (int64_t)b0;
            const REAL* B1 = verts + 3 * (int64_t)b1;
            const REAL* B2 = verts + 3 * (int64_t)b2;
            const REAL div1 = ORC(div_rwg)(verts, area1, a1, a2);
            const REAL div2 = ORC(div_rwg)(verts, area2, b1, b2);
            REAL acc_r = 0, acc_i = 0;
            for (int i = 0; i < nx * nx; ++i) {
                REAL r1 = gpx[i / nx];
                REAL r2 = gpx[i % nx] * r1;
                REAL w1 = gwx[i / nx] * gwx[i % nx] * (2 * area1);
                REAL j1 = r1;
                REAL x[3];
                for (int a = 0; a < 3; ++a) x[a] = (1 - r1) * A0[a] + (r1 - r2) * A1[a] + r2 * A2[a];
                REAL f1v[3];
                ORC(rwg)(x, verts, area1, a0, a1, a2, f1v);
                if (same) {
                    REAL f2v[3];
                    ORC(rwg)(x, verts, area2, b0, b1, b2, f2v);
                    for (int a = 0; a < 3; ++a) acc_r += w1 * j1 * (REAL)0.5 * f1v[a] * f2v[a];
                }
                REAL Kr[3] = {0, 0, 0}, Ki[3] = {0, 0, 0}, L1r[3] = {0, 0, 0}, L1i[3] = {0, 0, 0};
                REAL L2r = 0, L2i = 0;
                for (int j = 0; j < ny * ny; ++j) {
                    REAL r3 = gpy[j / ny];
                    REAL r4 = gpy[j % ny] * r3;
                    REAL w2 = gwy[j / ny] * gwy[j % ny] * (2 * area2);
                    REAL j2 = r3;
                    REAL y[3];
                    for (int a = 0; a < 3; ++a) y[a] = (1 - r3) * B0[a] + (r3 - r4) * B1[a] + r4 * B2[a];
                    REAL f2v[3];
                    ORC(rwg)(y, verts, area2, b0, b1, b2, f2v);
                    REAL gr, gi;
                    ORC(green)(k, x, y, &gr, &gi);
                    REAL ggr[3], ggi[3];
                    ORC(grad_green_x)(k, x, y, ggr, ggi);
                    REAL cr[3], ci[3];
                    ORC(cross3)(f2v, ggr, cr);
                    ORC(cross3)(f2v, ggi, ci);
                    for (int a = 0; a < 3; ++a) {
                        Kr[a] += w2 * j2 * cr[a];
                        Ki[a] += w2 * j2 * ci[a];
                        L1i[a] += k * w2 * j2 * (f2v[a] * gr);
                        L1r[a] += -k * w2 * j2 * (f2v[a] * gi);
                    }
                    L2i += -(REAL)1 / k * w2 * j2 * (div2 * gr);
                    L2r += (REAL)1 / k * w2 * j2 * (div2 * gi);
                }
                REAL nKr[3], nKi[3];
                ORC(cross3)(n1, Kr, nKr);
                ORC(cross3)(n1, Ki, nKi);
                for (int a = 0; a < 3; ++a) {
                    acc_r += w1 * j1 * f1v[a] * (nKr[a] + L1r[a]);
                    acc_i += w1 * j1 * f1v[a] * (nKi[a] + L1i[a]);
                }
                acc_r += w1 * j1 * div1 * L2r;
                acc_i += w1 * j1 * div1 * L2i;
            }
            zr[rr * ncol + col] = acc_r;
            zi[rr * ncol + col] = acc_i;
        }
    }
}

/* ------------------------------------------------------------------------------------ */
/* Face-edge excitation (mesh_MOM_3d.cu:244-330) for a plane wave.                       */
/* khat: unit propagation direction, e0: real polarisation, eta: wave impedance.         */
/* ref_incidence != 0 evaluates the reference's hard-coded wave exactly as written at    */
/* mesh_MOM_3d.cu:24-70 (k along azimuth 30 deg, E along z, H at azimuth -60 deg).       */
/* ------------------------------------------------------------------------------------ */
void ORC(mom_rhs_fe)(const REAL* verts, const int32_t* faces, int64_t nf, const REAL* areas,
                     const REAL* normals, const REAL* gp, const REAL* gw, int n, double wavenumber,
                     int ref_incidence, const double* khat, const double* e0, double eta,
                     REAL* rr_out, REAL* ri_out) {
    const REAL k = (REAL)wavenumber;
    REAL kv[3], E0[3], H0[3];
    if (ref_incidence) {
        REAL az = (REAL)(30 / 180.0 * ORC_PI);
        kv[0] = k * R_COS(az);
        kv[1] = k * R_SIN(az);
        kv[2] = 0;
        REAL hdir = (REAL)(az - 0.5 * ORC_PI);
        E0[0] = 0; E0[1] = 0; E0[2] = 1;
        REAL inv_eta = (REAL)1 / (REAL)sqrt(1.0);
        H0[0] = inv_eta * R_COS(hdir);
        H0[1] = inv_eta * R_SIN(hdir);
        H0[2] = 0;
    } else {
        for (int a = 0; a < 3; ++a) {
            kv[a] = (REAL)(wavenumber * khat[a]);
            E0[a] = (REAL)e0[a];
        }
        H0[0] = (REAL)((khat[1] * e0[2] - khat[2] * e0[1]) / eta);
        H0[1] = (REAL)((khat[2] * e0[0] - khat[0] * e0[2]) / eta);
        H0[2] = (REAL)((khat[0] * e0[1] - khat[1] * e0[0]) / eta);
    }
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < 3 * nf; ++idx) {
        const int64_t f = idx / 3;
        const int e = (int)(idx % 3);
        const REAL area = areas[f];
        const REAL* nrm = normals + 3 * f;
        const int32_t i0 = faces[3 * f + e], i1 = faces[3 * f + (e + 1) % 3], i2 = faces[3 * f + (e + 2) % 3];
        const REAL* v0 = verts + 3 * (int64_t)i0;
        const REAL* v1 = verts + 3 * (int64_t)i1;
        const REAL* v2 = verts + 3 * (int64_t)i2;
        REAL acc_r = 0, acc_i = 0;
        for (int i = 0; i < n * n; ++i) {
            REAL r1 = gp[i / n];
            REAL r2 = gp[i % n] * r1;
            REAL w = gw[i / n] * gw[i % n] * (2 * area);
            REAL jac = r1;
            REAL x[3];
            for (int a = 0; a < 3; ++a) x[a] = (1 - r1) * v0[a] + (r1 - r2) * v1[a] + r2 * v2[a];
            REAL fv[3];
            ORC(rwg)(x, verts, area, i0, i1, i2, fv);
            REAL kx = kv[0] * x[0] + kv[1] * x[1] + kv[2] * x[2];
            REAL ph_r = R_COS(-kx), ph_i = R_SIN(-kx);
            REAL Er[3], Ei[3], Hr[3], Hi[3];
            for (int a = 0; a < 3; ++a) {
                Er[a] = E0[a] * ph_r; Ei[a] = E0[a] * ph_i;
                Hr[a] = H0[a] * ph_r; Hi[a] = H0[a] * ph_i;
            }
            for (int a = 0; a < 3; ++a) {
                int b = (a + 1) % 3, c = (a + 2) % 3;
                acc_r += w * jac * fv[a] * Er[a];
                acc_i += w * jac * fv[a] * Ei[a];
                acc_r += w * jac * fv[a] * (nrm[b] * Hr[c] - Hr[b] * nrm[c]);
                acc_i += w * jac * fv[a] * (nrm[b] * Hi[c] - Hi[b] * nrm[c]);
            }
        }
        rr_out[idx] = acc_r;
        ri_out[idx] = acc_i;
    }
}

/* ------------------------------------------------------------------------------------ */
/* Edge coefficients -> per-face vertex currents (mesh_MOM_3d.cu:498-565)                */
/* I: [B, E] split real/imag.  out: [B, 3F, 3] split real/imag, accumulated (+=).        */
/* ------------------------------------------------------------------------------------ */
void ORC(mom_interp_js)(const REAL* verts, const int32_t* faces, const int32_t* fei, int64_t nf,
                        const REAL* areas, const REAL* ir, const REAL* ii, int64_t n_edges,
                        int64_t batch, REAL* jr, REAL* ji) {
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < batch * nf; ++idx) {
        const int64_t b = idx / nf;
        const int64_t f = idx % nf;
        for (int e = 0; e < 3; ++e) {
            const int64_t edge = fei[3 * f + e];
            const int32_t i0 = faces[3 * f + e], i1 = faces[3 * f + (e + 1) % 3], i2 = faces[3 * f + (e + 2) % 3];
            const REAL area = areas[f];
            REAL p1[3], p2[3], g1[3], g2[3];
            for (int a = 0; a < 3; ++a) {
                p1[a] = verts[3 * (int64_t)i1 + a];
                p2[a] = verts[3 * (int64_t)i2 + a];
            }
            ORC(rwg)(p1, verts, area, i0, i1, i2, g1);
            ORC(rwg)(p2, verts, area, i0, i1, i2, g2);
            const int64_t base = b * nf * 9 + f * 9;
            for (int a = 0; a < 3; ++a) {
                jr[base + ((e + 1) % 3) * 3 + a] += g1[a] * ir[b * n_edges + edge];
                ji[base + ((e + 1) % 3) * 3 + a] += g1[a] * ii[b * n_edges + edge];
                jr[base + ((e + 2) % 3) * 3 + a] += g2[a] * ir[b * n_edges + edge];
                ji[base + ((e + 2) % 3) * 3 + a] += g2[a] * ii[b * n_edges + edge];
            }
        }
    }
}

/* ------------------------------------------------------------------------------------ */
/* Laplace / Helmholtz panel double integrals (integrations_3d.py:18-452).              */
/* ------------------------------------------------------------------------------------ */

/* Sub-domain maps of one 4-D point for one panel relation.  Writes nd entries of
   (r1x, r2x, r1y, r2y, jac) and returns nd.  Follows get_rands_and_jacobian_3d
   (integrations_3d.py:18-249) term by term. */
static int ORC(ss_maps)(int rel, REAL xsi, REAL e1, REAL e2, REAL e3, REAL out[5][5]) {
    if (rel == 0) { /* SEPARATE :49-56 */
        out[0][0] = xsi; out[0][1] = e1 * xsi; out[0][2] = e2; out[0][3] = e2 * e3;
        out[0][4] = xsi * e2;
        return 1;
    }
    if (rel == 1) { /* SAME_VERTEX :58-79 */
        REAL jac = xsi * xsi * xsi * e2;
        out[0][0] = xsi; out[0][1] = xsi * e1; out[0][2] = xsi * e2; out[0][3] = xsi * e2 * e3; out[0][4] = jac;
        out[1][0] = xsi * e2; out[1][1] = xsi * e2 * e3; out[1][2] = xsi; out[1][3] = xsi * e1; out[1][4] = jac;
        return 2;
    }
    if (rel == 2) { /* SAME_EDGE :81-201 */
        REAL w[5][4];
        w[0][0] = xsi; w[0][1] = -xsi * e1 * e2; w[0][2] = xsi * e1 * (1 - e2); w[0][3] = xsi * e1 * e3;
        w[1][0] = xsi; w[1][1] = -xsi * e1 * e2 * e3; w[1][2] = xsi * e1 * e2 * (1 - e3); w[1][3] = xsi * e1;
        w[2][0] = xsi * (1 - e1 * e2); w[2][1] = xsi * e1 * e2; w[2][2] = xsi * e1 * e2 * e3;
        w[2][3] = xsi * e1 * (1 - e2);
        w[3][0] = xsi * (1 - e1 * e2 * e3); w[3][1] = xsi * e1 * e2 * e3; w[3][2] = xsi * e1;
        w[3][3] = xsi * e1 * e2 * (1 - e3);
        w[4][0] = xsi * (1 - e1 * e2 * e3); w[4][1] = xsi * e1 * e2 * e3; w[4][2] = xsi * e1 * e2;
        w[4][3] = xsi * e1 * (1 - e2 * e3);
        REAL j0 = xsi * xsi * xsi * e1 * e1;
        REAL j1 = xsi * xsi * xsi * e1 * e1 * e2;
        for (int d = 0; d < 5; ++d) {
            out[d][0] = w[d][0];
            out[d][1] = w[d][3];
            out[d][2] = w[d][0] + w[d][1];
            out[d][3] = w[d][2];
            out[d][4] = d == 0 ? j0 : j1;
        }
        return 5;
    }
    /* SAME_FACE :203-247 */
    REAL w0 = xsi, w1 = xsi * e1, w2 = xsi * e1 * e2, w3 = xsi * e1 * e2 * e3;
    REAL xz[3][4] = {
        {w0, w0 - w1 + w2, w3, w2},
        {w0, w1 - w2 + w3, w2, w3},
        {w0 - w3, w1 - w3, -w3, w2 - w3},
    };
    REAL jac = xsi * xsi * xsi * e1 * e1 * e2;
    for (int d = 0; d < 3; ++d) {
        out[d][0] = xz[d][0];
        out[d][1] = xz[d][1];
        out[d][2] = xz[d][0] - xz[d][2];
        out[d][3] = xz[d][1] - xz[d][3];
        out[d][4] = jac;
    }
    return 3;
}

/*
 * out[fy, fx, a, b] = sum_{g,d} f(x, y) * 4 A_fy A_fx * phi_a(y) * phi_b(x) * w_g * jac
 * for every ordered face pair (fy = first index, the "y" panel; fx = second, the "x" panel),
 * with the relation taken from rel[fy*nf + fx] (0 separate, 1 vertex, 2 edge, 3 face).
 * layer: 1 single layer G, 2 double layer grad_y G . n_fy.  order: 0 planar (1 shape
 * function), 1 linear (3).  kind: 0 Laplace 1/(4 pi R); 1 Helmholtz e^{+jkR}/(4 pi R)
 * (BEM_utils.py:95-102, :161-170), in which case out_i receives the imaginary part.
 * rands: [q, 2] (r1, r2) of the collapsed 2-D rule, w: [q] its weights.
 * Rows [fy_begin, fy_end) only; out is [(fy_end-fy_begin), nf, nphi, nphi].
 */
void ORC(laplace_panels)(const REAL* verts, const int32_t* faces, int64_t nf, const REAL* areas,
                         const REAL* normals, const REAL* rands, const REAL* w, int q,
                         const uint8_t* rel, int layer, int order, int kind, double wavenumber,
                         int64_t fy_begin, int64_t fy_end, REAL* out_r, REAL* out_i) {
    const int nphi = order == 1 ? 3 : 1;
    const int ng = q * q;
    const REAL k = (REAL)wavenumber;
    const REAL inv4pi = (REAL)(1.0 / 4.0 / ORC_PI);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t fy = fy_begin; fy < fy_end; ++fy) {
        for (int64_t fx = 0; fx < nf; ++fx) {
            const int r = rel[fy * nf + fx];
            const REAL afix = 4 * (areas[fy] * areas[fx]);
            const REAL* Y0 = verts + 3 * (int64_t)faces[3 * fy + 0];
            const REAL* Y1 = verts + 3 * (int64_t)faces[3 * fy + 1];
            const REAL* Y2 = verts + 3 * (int64_t)faces[3 * fy + 2];
            const REAL* X0 = verts + 3 * (int64_t)faces[3 * fx + 0];
            const REAL* X1 = verts + 3 * (int64_t)faces[3 * fx + 1];
            const REAL* X2 = verts + 3 * (int64_t)faces[3 * fx + 2];
            const REAL* ny = normals + 3 * fy;
            REAL accr[9] = {0}, acci[9] = {0};
            for (int g = 0; g < ng; ++g) {
                const int s = g / q, t = g % q;
                const REAL xsi = rands[2 * t], e1 = rands[2 * t + 1];
                const REAL e2 = rands[2 * s], e3 = rands[2 * s + 1];
                const REAL wyx = w[s] * w[t];
                REAL m[5][5];
                const int nd = ORC(ss_maps)(r, xsi, e1, e2, e3, m);
                for (int d = 0; d < nd; ++d) {
                    const REAL r1x = m[d][0], r2x = m[d][1], r1y = m[d][2], r2y = m[d][3], jac = m[d][4];
                    REAL x[3], y[3];
                    for (int a = 0; a < 3; ++a) {
                        x[a] = (1 - r1x) * X0[a] + (r1x - r2x) * X1[a] + r2x * X2[a];
                        y[a] = (1 - r1y) * Y0[a] + (r1y - r2y) * Y1[a] + r2y * Y2[a];
                    }
                    REAL dv[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
                    REAL dist = R_SQRT((dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]));
                    REAL fr, fi = 0;
                    if (layer == 1) {
                        if (kind == 0) {
                            fr = inv4pi / dist;
                        } else {
                            REAL b = inv4pi / dist;
                            fr = b * R_COS((k * dist));
                            fi = b * R_SIN((k * dist));
                        }
                    } else {
                        REAL dsq = dist * dist;
                        REAL dn = (dv[0] * ny[0] + dv[1] * ny[1] + dv[2] * ny[2]) / dist;
                        if (kind == 0) {
                            fr = inv4pi * dn / dsq;
                        } else {
                            REAL b = inv4pi * dn / dsq;
                            REAL c = R_COS((k * dist)), sn = R_SIN((k * dist));
                            /* (1 - jkd)(c + j s) */
                            fr = b * (c + k * dist * sn);
                            fi = b * (sn - k * dist * c);
                        }
                    }
                    REAL py[3], px[3];
                    if (nphi == 3) {
                        py[0] = 1 - r1y; py[1] = r1y - r2y; py[2] = r2y;
                        px[0] = 1 - r1x; px[1] = r1x - r2x; px[2] = r2x;
                    } else {
                        py[0] = 1; px[0] = 1;
                    }
                    const REAL sc = wyx * jac;
                    for (int a = 0; a < nphi; ++a)
                        for (int b = 0; b < nphi; ++b) {
                            accr[a * nphi + b] += fr * afix * (py[a] * px[b] * sc);
                            acci[a * nphi + b] += fi * afix * (py[a] * px[b] * sc);
                        }
                }
            }
            const int64_t base = ((fy - fy_begin) * nf + fx) * nphi * nphi;
            for (int c = 0; c < nphi * nphi; ++c) {
                out_r[base + c] = accr[c];
                if (out_i) out_i[base + c] = acci[c];
            }
        }
    }
}

/* Panel relation by shared-vertex count (mesh_utils.py:700-725). */
void ORC(panel_relation)(const int32_t* faces, int64_t nf, uint8_t* rel) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nf; ++i)
        for (int64_t j = 0; j < nf; ++j) {
            int cnt = 0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) cnt += faces[3 * i + a] == faces[3 * j + b];
            rel[i * nf + j] = (uint8_t)(cnt <= 3 ? cnt : 0);
        }
}

/* ------------------------------------------------------------------------------------ */
/* Scattered magnetic field radiated from vertex currents                               */
/* (demo/demo_Helmholtz_MOM_3d.py:246-257 with gradG_y / G, src/utils/functions.py:807-868):*/
/*   H(p) = -sum_v A_v ( J_v x (-gradG_y(k, p, v)) ),                                    */
/*   gradG_y = G(+k) / R * (1 + jkR) * (p - v)/R,  G(+k) = e^{+jkR} / (4 pi R),           */
/* with the reference's mask: a vertex closer than 1e-6 contributes nothing.             */
/* js: [V, 3] split real/imag; h: [P, 3] split real/imag (overwritten).                  */
/* ------------------------------------------------------------------------------------ */
void ORC(radiate_h)(const REAL* points, int64_t np, const REAL* verts, const REAL* vert_areas,
                    const REAL* jr, const REAL* ji, int64_t nv, double wavenumber, REAL* hr,
                    REAL* hi) {
    const REAL k = (REAL)wavenumber;
#pragma omp parallel for schedule(static)
    for (int64_t m = 0; m < np; ++m) {
        REAL ar[3] = {0, 0, 0}, ai[3] = {0, 0, 0};
        for (int64_t v = 0; v < nv; ++v) {
            REAL d[3];
            for (int a = 0; a < 3; ++a) d[a] = points[3 * m + a] - verts[3 * v + a];
            REAL dist = R_SQRT((d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
            if (dist < (REAL)1e-6) continue;
            REAL inv = (REAL)1 / dist;
            REAL kr = k * dist;
            REAL gr = (REAL)(R_COS(kr) / (4 * ORC_PI)) * inv;
            REAL gi = (REAL)(R_SIN(kr) / (4 * ORC_PI)) * inv;
            /* G * inv * (1 + j k R) */
            REAL fr = (gr - gi * kr) * inv, fi = (gi + gr * kr) * inv;
            REAL rd[3] = {d[0] * inv, d[1] * inv, d[2] * inv};
            REAL Jr[3], Ji[3];
            for (int a = 0; a < 3; ++a) {
                Jr[a] = jr[3 * v + a];
                Ji[a] = ji[3 * v + a];
            }
            REAL cr[3], ci[3];
            ORC(cross3)(Jr, rd, cr);
            ORC(cross3)(Ji, rd, ci);
            for (int a = 0; a < 3; ++a) {
                ar[a] += vert_areas[v] * (fr * cr[a] - fi * ci[a]);
                ai[a] += vert_areas[v] * (fr * ci[a] + fi * cr[a]);
            }
        }
        for (int a = 0; a < 3; ++a) {
            hr[3 * m + a] = ar[a];
            hi[3 * m + a] = ai[a];
        }
    }
}

/* ==================================================================================== */
/* Symmetric-rule EFIE (a capability the reference does not have; checker for the       */
/* "dunavant7" GPU path).  7-point degree-5 rule (Radon; Dunavant 1985) on both         */
/* triangles; pairs that share a vertex (self, edge- and vertex-adjacent) integrate     */
/* G = 1/(4 pi R) + (e^{-jkR} - 1)/(4 pi R): the smooth part with the source rule, the  */
/* singular part analytically (Wilton, Rao, Glisson, Schaubert, Al-Bundak, Butler 1984, */
/* IEEE Trans. AP-32(3):276-281).  Entries follow the reference's EFIE terms             */
/* jk G f_m . f_n - (j/k) G div f_m div f_n (mesh_MOM_3d.cu:474-480) with its RWG        */
/* convention (mesh_MOM_3d.cu:154-242).  Everything in double.                          */
/* ==================================================================================== */
#ifndef ORC_SYM_DEFINED_ONCE
#define ORC_SYM_DEFINED_ONCE
static void orc_d7(double bary[7][3], double w[7]) {
    const double s15 = sqrt(15.0);
    const double a1 = (6.0 - s15) / 21.0, b1 = 1.0 - 2.0 * a1, w1 = (155.0 - s15) / 1200.0;
    const double a2 = (6.0 + s15) / 21.0, b2 = 1.0 - 2.0 * a2, w2 = (155.0 + s15) / 1200.0;
    const double t[7][4] = {
        {1.0 / 3, 1.0 / 3, 1.0 / 3, 9.0 / 40},
        {a1, a1, b1, w1}, {a1, b1, a1, w1}, {b1, a1, a1, w1},
        {a2, a2, b2, w2}, {a2, b2, a2, w2}, {b2, a2, a2, w2},
    };
    for (int i = 0; i < 7; ++i) {
        bary[i][0] = t[i][0]; bary[i][1] = t[i][1]; bary[i][2] = t[i][2];
        w[i] = t[i][3];
    }
}

/* I1 = int_T 1/|x - y| dS_y and Iv = int_T (y - x)/|x - y| dS_y over triangle P. */
static void orc_pot_integrals(const double* x, const double P[3][3], double* I1, double Iv[3]) {
    double e0[3], e1[3], n[3];
    for (int a = 0; a < 3; ++a) { e0[a] = P[1][a] - P[0][a]; e1[a] = P[2][a] - P[1][a]; }
    n[0] = e0[1] * e1[2] - e0[2] * e1[1];
    n[1] = e0[2] * e1[0] - e0[0] * e1[2];
    n[2] = e0[0] * e1[1] - e0[1] * e1[0];
    double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int a = 0; a < 3; ++a) n[a] /= nn;
    double d = (x[0] - P[0][0]) * n[0] + (x[1] - P[0][1]) * n[1] + (x[2] - P[0][2]) * n[2];
    double rho[3] = {x[0] - d * n[0], x[1] - d * n[1], x[2] - d * n[2]};
    double s1 = 0, sv[3] = {0, 0, 0};
    const double ad = fabs(d);
    for (int i = 0; i < 3; ++i) {
        const double* pm = P[i];
        const double* pp = P[(i + 1) % 3];
        double l[3] = {pp[0] - pm[0], pp[1] - pm[1], pp[2] - pm[2]};
        double ll = sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
        for (int a = 0; a < 3; ++a) l[a] /= ll;
        double u[3] = {l[1] * n[2] - l[2] * n[1], l[2] * n[0] - l[0] * n[2], l[0] * n[1] - l[1] * n[0]};
        double lp = (pp[0] - rho[0]) * l[0] + (pp[1] - rho[1]) * l[1] + (pp[2] - rho[2]) * l[2];
        double lm = (pm[0] - rho[0]) * l[0] + (pm[1] - rho[1]) * l[1] + (pm[2] - rho[2]) * l[2];
        double p0 = (pp[0] - rho[0]) * u[0] + (pp[1] - rho[1]) * u[1] + (pp[2] - rho[2]) * u[2];
        double r0sq = p0 * p0 + d * d;
        double rp = sqrt(r0sq + lp * lp), rm = sqrt(r0sq + lm * lm);
        double lg;
        if ((lm >= 0 || lp >= 0) && rm + lm > 0) lg = log((rp + lp) / (rm + lm));
        else lg = log((rm - lm) / (rp - lp));
        s1 += p0 * lg - ad * (atan2(p0 * lp, r0sq + ad * rp) - atan2(p0 * lm, r0sq + ad * rm));
        double t = 0.5 * (r0sq * lg + lp * rp - lm * rm);
        for (int a = 0; a < 3; ++a) sv[a] += t * u[a];
    }
    *I1 = s1;
    for (int a = 0; a < 3; ++a) Iv[a] = sv[a] - d * n[a] * s1;
}
#endif

/*
 * Z (RWG, [E, E], split real/imag, accumulated) of the EFIE with the symmetric rule.
 * Test faces [f_begin, f_end) only (row window); all source faces.
 */
void ORC(mom_sym_zmat_rwg)(const REAL* verts_r, const int32_t* faces, int64_t nf, const int32_t* fei,
                           int64_t ne, double k, int64_t f_begin, int64_t f_end, double* zr, double* zi) {
    double bary[7][3], w7[7];
    orc_d7(bary, w7);
    const double inv4pi = 1.0 / (4.0 * ORC_PI);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t p = f_begin; p < f_end; ++p) {
        double A[3][3];
        for (int v = 0; v < 3; ++v)
            for (int a = 0; a < 3; ++a) A[v][a] = (double)verts_r[3 * (int64_t)faces[3 * p + v] + a];
        double ap[3] = {A[1][0] - A[0][0], A[1][1] - A[0][1], A[1][2] - A[0][2]};
        double bp[3] = {A[2][0] - A[1][0], A[2][1] - A[1][1], A[2][2] - A[1][2]};
        double cpr[3] = {ap[1] * bp[2] - ap[2] * bp[1], ap[2] * bp[0] - ap[0] * bp[2], ap[0] * bp[1] - ap[1] * bp[0]};
        double areap = 0.5 * sqrt(cpr[0] * cpr[0] + cpr[1] * cpr[1] + cpr[2] * cpr[2]);
        double cm[3];
        for (int e = 0; e < 3; ++e) {
            int i1 = faces[3 * p + (e + 1) % 3], i2 = faces[3 * p + (e + 2) % 3];
            double dl = 0;
            for (int a = 0; a < 3; ++a) dl += (A[(e + 2) % 3][a] - A[(e + 1) % 3][a]) * (A[(e + 2) % 3][a] - A[(e + 1) % 3][a]);
            cm[e] = (i1 < i2 ? 1.0 : -1.0) * sqrt(dl) / (2.0 * areap);
        }
        double X[7][3];
        for (int i = 0; i < 7; ++i)
            for (int a = 0; a < 3; ++a) X[i][a] = bary[i][0] * A[0][a] + bary[i][1] * A[1][a] + bary[i][2] * A[2][a];
        for (int64_t q = 0; q < nf; ++q) {
            double B[3][3];
            for (int v = 0; v < 3; ++v)
                for (int a = 0; a < 3; ++a) B[v][a] = (double)verts_r[3 * (int64_t)faces[3 * q + v] + a];
            int shared = 0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) shared += faces[3 * p + a] == faces[3 * q + b];
            double aq[3] = {B[1][0] - B[0][0], B[1][1] - B[0][1], B[1][2] - B[0][2]};
            double bq[3] = {B[2][0] - B[1][0], B[2][1] - B[1][1], B[2][2] - B[1][2]};
            double cq[3] = {aq[1] * bq[2] - aq[2] * bq[1], aq[2] * bq[0] - aq[0] * bq[2], aq[0] * bq[1] - aq[1] * bq[0]};
            double areaq = 0.5 * sqrt(cq[0] * cq[0] + cq[1] * cq[1] + cq[2] * cq[2]);
            double cn[3];
            for (int e = 0; e < 3; ++e) {
                int i1 = faces[3 * q + (e + 1) % 3], i2 = faces[3 * q + (e + 2) % 3];
                double dl = 0;
                for (int a = 0; a < 3; ++a) dl += (B[(e + 2) % 3][a] - B[(e + 1) % 3][a]) * (B[(e + 2) % 3][a] - B[(e + 1) % 3][a]);
                cn[e] = (i1 < i2 ? 1.0 : -1.0) * sqrt(dl) / (2.0 * areaq);
            }
            double Y[7][3];
            for (int j = 0; j < 7; ++j)
                for (int a = 0; a < 3; ++a) Y[j][a] = bary[j][0] * B[0][a] + bary[j][1] * B[1][a] + bary[j][2] * B[2][a];
            double accr[3][3] = {{0}}, acci[3][3] = {{0}};
            for (int i = 0; i < 7; ++i) {
                /* inner integrals: g0 = int G, gy = int y G (complex) */
                double g0r = 0, g0i = 0, gyr[3] = {0, 0, 0}, gyi[3] = {0, 0, 0};
                for (int j = 0; j < 7; ++j) {
                    double dd[3] = {X[i][0] - Y[j][0], X[i][1] - Y[j][1], X[i][2] - Y[j][2]};
                    double R = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
                    double gr, gi;
                    if (shared == 0) {
                        gr = cos(k * R) / R * inv4pi;
                        gi = -sin(k * R) / R * inv4pi;
                    } else if (R < 1e-300) {
                        gr = 0.0;
                        gi = -k * inv4pi;
                    } else {
                        double sh = sin(0.5 * k * R);
                        gr = -2.0 * sh * sh / R * inv4pi;
                        gi = -sin(k * R) / R * inv4pi;
                    }
                    double wj = w7[j] * areaq;
                    g0r += wj * gr; g0i += wj * gi;
                    for (int a = 0; a < 3; ++a) { gyr[a] += wj * gr * Y[j][a]; gyi[a] += wj * gi * Y[j][a]; }
                }
                if (shared) {
                    double I1, Iv[3];
                    orc_pot_integrals(X[i], B, &I1, Iv);
                    g0r += inv4pi * I1;
                    for (int a = 0; a < 3; ++a) gyr[a] += inv4pi * (Iv[a] + X[i][a] * I1);
                }
                double wi = w7[i] * areap;
                for (int m = 0; m < 3; ++m) {
                    for (int nn = 0; nn < 3; ++nn) {
                        /* int f_n G = c_n (gy - v_n g0);  f_m(x) = c_m (x - v_m) */
                        double fr = 0, fi = 0;
                        for (int a = 0; a < 3; ++a) {
                            double vn = B[nn][a];
                            double tr = gyr[a] - vn * g0r, ti = gyi[a] - vn * g0i;
                            double xm = X[i][a] - A[m][a];
                            fr += xm * tr;
                            fi += xm * ti;
                        }
                        double cc = cm[m] * cn[nn];
                        /* jk cc (fr + j fi) - (4j/k) cc (g0r + j g0i) */
                        accr[m][nn] += wi * cc * (-k * fi + 4.0 / k * g0i);
                        acci[m][nn] += wi * cc * (k * fr - 4.0 / k * g0r);
                    }
                }
            }
            for (int m = 0; m < 3; ++m)
                for (int nn = 0; nn < 3; ++nn) {
                    int64_t row = fei[3 * p + m], col = fei[3 * q + nn];
                    int64_t o = (row * ne + col);
#pragma omp atomic
                    zr[o] += accr[m][nn];
#pragma omp atomic
                    zi[o] += acci[m][nn];
                }
        }
    }
}

/* EFIE excitation with the symmetric rule: rhs[fei, w] += int f_m . E0 e^{-j k khat.x}. */
void ORC(mom_sym_rhs_rwg)(const REAL* verts_r, const int32_t* faces, int64_t nf, const int32_t* fei,
                          int64_t ne, const double* waves, int nrhs, double* rr, double* ri) {
    double bary[7][3], w7[7];
    orc_d7(bary, w7);
    for (int64_t p = 0; p < nf; ++p) {
        double A[3][3];
        for (int v = 0; v < 3; ++v)
            for (int a = 0; a < 3; ++a) A[v][a] = (double)verts_r[3 * (int64_t)faces[3 * p + v] + a];
        double ap[3] = {A[1][0] - A[0][0], A[1][1] - A[0][1], A[1][2] - A[0][2]};
        double bp[3] = {A[2][0] - A[1][0], A[2][1] - A[1][1], A[2][2] - A[1][2]};
        double cpr[3] = {ap[1] * bp[2] - ap[2] * bp[1], ap[2] * bp[0] - ap[0] * bp[2], ap[0] * bp[1] - ap[1] * bp[0]};
        double areap = 0.5 * sqrt(cpr[0] * cpr[0] + cpr[1] * cpr[1] + cpr[2] * cpr[2]);
        for (int m = 0; m < 3; ++m) {
            int i1 = faces[3 * p + (m + 1) % 3], i2 = faces[3 * p + (m + 2) % 3];
            double dl = 0;
            for (int a = 0; a < 3; ++a) dl += (A[(m + 2) % 3][a] - A[(m + 1) % 3][a]) * (A[(m + 2) % 3][a] - A[(m + 1) % 3][a]);
            double c = (i1 < i2 ? 1.0 : -1.0) * sqrt(dl) / (2.0 * areap);
            for (int r = 0; r < nrhs; ++r) {
                const double* wv = waves + 9 * r;
                double sr = 0, si = 0;
                for (int i = 0; i < 7; ++i) {
                    double x[3], proj = 0, ph = 0;
                    for (int a = 0; a < 3; ++a) x[a] = bary[i][0] * A[0][a] + bary[i][1] * A[1][a] + bary[i][2] * A[2][a];
                    for (int a = 0; a < 3; ++a) { proj += (x[a] - A[m][a]) * wv[3 + a]; ph += wv[a] * x[a]; }
                    double wi = w7[i] * areap * c * proj;
                    sr += wi * cos(ph);
                    si -= wi * sin(ph);
                }
                int64_t o = (int64_t)fei[3 * p + m] * nrhs + r;
                rr[o] += sr;
                ri[o] += si;
            }
        }
    }
}

/* Exported for tests: closed-form int_T 1/R and int_T (y - x)/R (see orc_pot_integrals). */
#ifndef ORC_POT_EXPORTED
#define ORC_POT_EXPORTED
#ifdef ORC_FLOAT
#else
void orc_potential_integrals(const double* x, const double* tri, double* I1, double* Iv) {
    double P[3][3];
    for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) P[v][a] = tri[3 * v + a];
    orc_pot_integrals(x, P, I1, Iv);
}
#endif
#endif

/* ------------------------------------------------------------------------------------ */
/* Symmetric-rule Laplace operators (checker for csrc/laplace_sym.cu; the reference has  */
/* no such mode).  Galerkin: out[fy, fx, a, b] = int_fy int_fx phi_a(y) phi_b(x) k(x, y)  */
/* with k = 1/(4 pi R) (layer 1) or n_y.(x - y)/(4 pi R^3) (layer 2), P1 (order 1) or P0; */
/* 7 x 7 points for pairs without a shared vertex, else 7 points on fx and the inner     */
/* integral over fy in closed form (Wilton et al. 1984; van Oosterom & Strackee 1983 for  */
/* the solid angle; int (rho_y - rho)/R^3 = -sum_i u_i ln((R+ + l+)/(R- + l-))).           */
/* Collocation: A[i, j] = int_{T_j} 1/(4 pi |c_i - y|), c_i the centroid of face i.      */
/* Double precision only.                                                               */
/* ------------------------------------------------------------------------------------ */
#ifndef ORC_FLOAT
static double orc_dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void orc_cross3d(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

/* omega = int_T n.(y - x)/R^3 (signed solid angle), J = int_T (rho_y - rho)/R^3, d = n.(x - P0);
 * both 0 when |d| <= dtol (x in the plane of T, where the double-layer kernel vanishes). */
static void orc_dl_integrals(const double* x, const double P[3][3], double dtol, double* omega, double J[3],
                             double* dout) {
    double e0[3], e1[3], n[3];
    for (int a = 0; a < 3; ++a) { e0[a] = P[1][a] - P[0][a]; e1[a] = P[2][a] - P[1][a]; }
    orc_cross3d(e0, e1, n);
    const double nn = sqrt(orc_dot3(n, n));
    for (int a = 0; a < 3; ++a) n[a] /= nn;
    double xp[3] = {x[0] - P[0][0], x[1] - P[0][1], x[2] - P[0][2]};
    const double d = orc_dot3(xp, n);
    *dout = d;
    J[0] = J[1] = J[2] = 0.0;
    if (fabs(d) <= dtol) {
        *omega = 0.0;
        return;
    }
    double r[3][3], l[3];
    for (int v = 0; v < 3; ++v) {
        for (int a = 0; a < 3; ++a) r[v][a] = P[v][a] - x[a];
        l[v] = sqrt(orc_dot3(r[v], r[v]));
    }
    double c12[3];
    orc_cross3d(r[1], r[2], c12);
    const double num = orc_dot3(r[0], c12);
    const double den = l[0] * l[1] * l[2] + orc_dot3(r[0], r[1]) * l[2] + orc_dot3(r[0], r[2]) * l[1] +
                       orc_dot3(r[1], r[2]) * l[0];
    *omega = 2.0 * atan2(num, den);
    double rho[3] = {x[0] - d * n[0], x[1] - d * n[1], x[2] - d * n[2]};
    for (int i = 0; i < 3; ++i) {
        const double* pm = P[i];
        const double* pp = P[(i + 1) % 3];
        double ed[3] = {pp[0] - pm[0], pp[1] - pm[1], pp[2] - pm[2]};
        const double el = sqrt(orc_dot3(ed, ed));
        for (int a = 0; a < 3; ++a) ed[a] /= el;
        double u[3];
        orc_cross3d(ed, n, u);
        double dp[3] = {pp[0] - rho[0], pp[1] - rho[1], pp[2] - rho[2]};
        double dm[3] = {pm[0] - rho[0], pm[1] - rho[1], pm[2] - rho[2]};
        const double lp = orc_dot3(dp, ed), lm = orc_dot3(dm, ed), p0 = orc_dot3(dp, u);
        const double r0sq = p0 * p0 + d * d;
        const double rp = sqrt(r0sq + lp * lp), rm = sqrt(r0sq + lm * lm);
        double lg;
        if ((lm >= 0 || lp >= 0) && rm + lm > 0) lg = log((rp + lp) / (rm + lm));
        else lg = log((rm - lm) / (rp - lp));
        for (int a = 0; a < 3; ++a) J[a] -= lg * u[a];
    }
}

static void orc_face(const double* verts, const int32_t* faces, int64_t f, double P[3][3]) {
    for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) P[v][a] = verts[3 * (int64_t)faces[3 * f + v] + a];
}

static int orc_share_vertex(const int32_t* faces, int64_t p, int64_t q) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (faces[3 * p + i] == faces[3 * q + j]) return 1;
    return 0;
}

void orc_laplace_sym_f64(const double* verts, const int32_t* faces, int64_t nf, int layer, int order,
                         int64_t row_begin, int64_t row_end, double* out) {
    double bary[7][3], w7[7];
    orc_d7(bary, w7);
    const int nphi = order == 1 ? 3 : 1, nn = nphi * nphi;
    const double inv4pi = 1.0 / (4.0 * ORC_PI);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t fy = row_begin; fy < row_end; ++fy) {
        double P[3][3], e0[3], e1[3], ny[3];
        orc_face(verts, faces, fy, P);
        for (int a = 0; a < 3; ++a) { e0[a] = P[1][a] - P[0][a]; e1[a] = P[2][a] - P[1][a]; }
        orc_cross3d(e0, e1, ny);
        const double two_ay = sqrt(orc_dot3(ny, ny));
        for (int a = 0; a < 3; ++a) ny[a] /= two_ay;
        double grad[3][3], cy[3], hmax = 0.0;
        for (int a = 0; a < 3; ++a) {
            double ed[3];
            for (int c = 0; c < 3; ++c) ed[c] = P[(a + 2) % 3][c] - P[(a + 1) % 3][c];
            orc_cross3d(ny, ed, grad[a]);
            for (int c = 0; c < 3; ++c) grad[a][c] /= two_ay;
            cy[a] = (P[0][a] + P[1][a] + P[2][a]) / 3.0;
            double eb[3];
            for (int c = 0; c < 3; ++c) eb[c] = P[(a + 1) % 3][c] - P[a][c];
            hmax = fmax(hmax, sqrt(orc_dot3(eb, eb)));
        }
        double ys[7][3];
        for (int j = 0; j < 7; ++j)
            for (int c = 0; c < 3; ++c) ys[j][c] = bary[j][0] * P[0][c] + bary[j][1] * P[1][c] + bary[j][2] * P[2][c];
        for (int64_t fx = 0; fx < nf; ++fx) {
            double Q[3][3], f0[3], f1[3], nx[3];
            orc_face(verts, faces, fx, Q);
            for (int a = 0; a < 3; ++a) { f0[a] = Q[1][a] - Q[0][a]; f1[a] = Q[2][a] - Q[1][a]; }
            orc_cross3d(f0, f1, nx);
            const double ax = 0.5 * sqrt(orc_dot3(nx, nx));
            const int near = orc_share_vertex(faces, fy, fx);
            double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int i = 0; i < 7; ++i) {
                double x[3];
                for (int c = 0; c < 3; ++c) x[c] = bary[i][0] * Q[0][c] + bary[i][1] * Q[1][c] + bary[i][2] * Q[2][c];
                double sa[3] = {0, 0, 0};
                if (near) {
                    double xc[3] = {x[0] - cy[0], x[1] - cy[1], x[2] - cy[2]};
                    if (layer == 1) {
                        double I0, I1[3];
                        orc_pot_integrals(x, P, &I0, I1);
                        for (int a = 0; a < nphi; ++a)
                            sa[a] = nphi == 3 ? (1.0 / 3.0 + orc_dot3(grad[a], xc)) * I0 + orc_dot3(grad[a], I1) : I0;
                    } else {
                        double om, J[3], d;
                        orc_dl_integrals(x, P, 1e-10 * hmax, &om, J, &d);
                        for (int a = 0; a < nphi; ++a)
                            sa[a] = nphi == 3 ? -(1.0 / 3.0 + orc_dot3(grad[a], xc)) * om + d * orc_dot3(grad[a], J)
                                              : -om;
                    }
                } else {
                    for (int j = 0; j < 7; ++j) {
                        double dd[3] = {x[0] - ys[j][0], x[1] - ys[j][1], x[2] - ys[j][2]};
                        const double R = sqrt(orc_dot3(dd, dd));
                        double g = w7[j] * 0.5 * two_ay / R;
                        if (layer == 2) g *= orc_dot3(ny, dd) / (R * R);
                        for (int a = 0; a < nphi; ++a) sa[a] += g * (nphi == 3 ? bary[j][a] : 1.0);
                    }
                }
                const double wx = w7[i] * ax;
                for (int a = 0; a < nphi; ++a)
                    for (int b = 0; b < nphi; ++b) acc[a * nphi + b] += sa[a] * wx * (nphi == 3 ? bary[i][b] : 1.0);
            }
            double* o = out + ((fy - row_begin) * nf + fx) * nn;
            for (int c = 0; c < nn; ++c) o[c] = acc[c] * inv4pi;
        }
    }
}

void orc_laplace_colloc_sl_f64(const double* verts, const int32_t* faces, int64_t nf, double* out) {
    double bary[7][3], w7[7];
    orc_d7(bary, w7);
    const double inv4pi = 1.0 / (4.0 * ORC_PI);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t i = 0; i < nf; ++i) {
        double A[3][3], c[3];
        orc_face(verts, faces, i, A);
        for (int a = 0; a < 3; ++a) c[a] = (A[0][a] + A[1][a] + A[2][a]) / 3.0;
        for (int64_t j = 0; j < nf; ++j) {
            double P[3][3];
            orc_face(verts, faces, j, P);
            double v;
            if (orc_share_vertex(faces, i, j)) {
                double I1[3];
                orc_pot_integrals(c, P, &v, I1);
            } else {
                double e0[3], e1[3], nr[3];
                for (int a = 0; a < 3; ++a) { e0[a] = P[1][a] - P[0][a]; e1[a] = P[2][a] - P[1][a]; }
                orc_cross3d(e0, e1, nr);
                const double area = 0.5 * sqrt(orc_dot3(nr, nr));
                v = 0.0;
                for (int k = 0; k < 7; ++k) {
                    double y[3];
                    for (int a = 0; a < 3; ++a)
                        y[a] = bary[k][0] * P[0][a] + bary[k][1] * P[1][a] + bary[k][2] * P[2][a] - c[a];
                    v += w7[k] * area / sqrt(orc_dot3(y, y));
                }
            }
            out[i * nf + j] = v * inv4pi;
        }
    }
}
#endif

/* ------------------------------------------------------------------------------------ */
/* Closest-hit ray query (the reference's Vulkan ray-query plugin,                      */
/* src/vulkan_ray_tracing/shaders/raygen.rgen:23-64, closesthit.rchit, miss.rmiss;       */
/* QueryForNLOS / QueryForLOS at ray_query_App.hpp:881-1000): rays from origin[row] along */
/* normalised dir[row*W + col], opaque, no culling, t in [tmin, tmax]; result per ray     */
/* (face index, 0, 0, distance to the hit) or (-1, 0, 0, -1).  Brute force over all       */
/* triangles with the Moller-Trumbore test (Moller & Trumbore 1997), in double.           */
/* ------------------------------------------------------------------------------------ */
void ORC(ray_query)(const REAL* verts, const int32_t* faces, int64_t nf, const REAL* origins,
                    const REAL* dirs, int64_t h, int64_t w, double tmin, double tmax, REAL* out) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < h * w; ++r) {
        const int64_t row = r / w;
        double o[3] = {origins[3 * row], origins[3 * row + 1], origins[3 * row + 2]};
        double d[3] = {dirs[3 * r], dirs[3 * r + 1], dirs[3 * r + 2]};
        double dn = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int a = 0; a < 3; ++a) d[a] /= dn;
        double best = tmax;
        int64_t hit = -1;
        for (int64_t f = 0; f < nf; ++f) {
            const REAL* v0 = verts + 3 * (int64_t)faces[3 * f];
            const REAL* v1 = verts + 3 * (int64_t)faces[3 * f + 1];
            const REAL* v2 = verts + 3 * (int64_t)faces[3 * f + 2];
            double e1[3], e2[3], s[3];
            for (int a = 0; a < 3; ++a) {
                e1[a] = v1[a] - v0[a];
                e2[a] = v2[a] - v0[a];
                s[a] = o[a] - v0[a];
            }
            double p[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
            double det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
            if (fabs(det) < 1e-300) continue;
            double inv = 1.0 / det;
            double u = (s[0] * p[0] + s[1] * p[1] + s[2] * p[2]) * inv;
            if (u < 0.0 || u > 1.0) continue;
            double q[3] = {s[1] * e1[2] - s[2] * e1[1], s[2] * e1[0] - s[0] * e1[2], s[0] * e1[1] - s[1] * e1[0]};
            double v = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * inv;
            if (v < 0.0 || u + v > 1.0) continue;
            double t = (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * inv;
            if (t >= tmin && t <= best) {
                if (t < best || hit < 0 || f < hit) {
                    best = t;
                    hit = f;
                }
            }
        }
        out[4 * r + 0] = (REAL)(hit >= 0 ? (double)hit : -1.0);
        out[4 * r + 1] = 0;
        out[4 * r + 2] = 0;
        out[4 * r + 3] = (REAL)(hit >= 0 ? best : -1.0);
    }
}
