// closed_form.cuh -- the symmetric 7-point triangle rule and closed-form integrals of the
// Laplace kernels over a flat triangle, shared by the symmetric-rule EFIE (mom_sym.cu) and
// the symmetric-rule Laplace operators (laplace_sym.cu).
//
// For an observation point x and a triangle T with unit normal n (orientation of
// (P1 - P0) x (P2 - P1)), d = n.(x - P0), rho = x - d n, and per edge i (from P_i to
// P_{i+1}, unit direction l_i, outward in-plane normal u_i = l_i x n):
//   int_T 1/R dS         = sum_i P0_i ln((R+_i + l+_i)/(R-_i + l-_i)) - |d| sum_i (beta+_i - beta-_i)
//   int_T (y - x)/R dS   = 1/2 sum_i u_i [R0_i^2 ln(...) + l+_i R+_i - l-_i R-_i] - d n int_T 1/R
// (D. R. Wilton, S. M. Rao, A. W. Glisson, D. H. Schaubert, O. M. Al-Bundak, C. M. Butler,
// IEEE Trans. AP-32(3):276-281, 1984), and for the double-layer kernel
//   int_T n.(y - x)/R^3 dS  = 2 atan2(r0.(r1 x r2), r0 r1 r2 + (r0.r1) r2 + (r0.r2) r1 + (r1.r2) r0)
// with r_i = P_i - x (the signed solid angle; A. van Oosterom and J. Strackee, IEEE Trans.
// BME-30(2):125-126, 1983), and, from the surface gradient theorem,
//   int_T (rho_y - rho)/R^3 dS = - sum_i u_i ln((R+_i + l+_i)/(R-_i + l-_i)).
#pragma once
#include "common.cuh"

namespace mb {

// 7-point rule: barycentric coordinates and weights (sum 1), from the closed forms
// a = (6 -+ sqrt 15)/21, w = (155 -+ sqrt 15)/1200, centroid weight 9/40.
static __constant__ double c_d7[7][4] = {
    {0.33333333333333333, 0.33333333333333333, 0.33333333333333333, 0.225},
    {0.10128650732345634, 0.10128650732345634, 0.79742698535308732, 0.12593918054482715},
    {0.10128650732345634, 0.79742698535308732, 0.10128650732345634, 0.12593918054482715},
    {0.79742698535308732, 0.10128650732345634, 0.10128650732345634, 0.12593918054482715},
    {0.47014206410511509, 0.47014206410511509, 0.05971587178976982, 0.13239415278850619},
    {0.47014206410511509, 0.05971587178976982, 0.47014206410511509, 0.13239415278850619},
    {0.05971587178976982, 0.47014206410511509, 0.47014206410511509, 0.13239415278850619},
};

// int_T 1/R dS and int_T (y - x)/R dS (FP64).
__device__ __forceinline__ double edge_log(double rp, double rm, double lp, double lm) {
    if ((lm >= 0.0 || lp >= 0.0) && rm + lm > 0.0) return log((rp + lp) / (rm + lm));
    return log((rm - lm) / (rp - lp));
}

__device__ __forceinline__ void potential_integrals(const V3<double>& x, const V3<double> P[3], double* I1,
                                                    V3<double>* Iv) {
    V3<double> n = cross(P[1] - P[0], P[2] - P[1]);
    n = (1.0 / sqrt(dot(n, n))) * n;
    const double d = dot(x - P[0], n);
    const V3<double> rho = x - d * n;
    const double ad = fabs(d);
    double s1 = 0.0;
    V3<double> sv = v3<double>(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const V3<double> pm = P[i], pp = P[(i + 1) % 3];
        V3<double> l = pp - pm;
        l = (1.0 / sqrt(dot(l, l))) * l;
        const V3<double> u = cross(l, n);
        const double lp = dot(pp - rho, l), lm = dot(pm - rho, l);
        const double p0 = dot(pp - rho, u);
        const double r0sq = p0 * p0 + d * d;
        const double rp = sqrt(r0sq + lp * lp), rm = sqrt(r0sq + lm * lm);
        const double lg = edge_log(rp, rm, lp, lm);
        s1 += p0 * lg - ad * (atan2(p0 * lp, r0sq + ad * rp) - atan2(p0 * lm, r0sq + ad * rm));
        sv = sv + (0.5 * (r0sq * lg + lp * rp - lm * rm)) * u;
    }
    *I1 = s1;
    *Iv = sv - (d * s1) * n;
}

// Double-layer integrals (FP64): *omega = int_T n.(y - x)/R^3 dS (signed solid angle) and
// *J = int_T (rho_y - rho)/R^3 dS (in-plane vector); *d = n.(x - P0).  When |d| is below
// dtol the point lies in the triangle's plane, where n.(x - y) vanishes: omega = 0 (the
// principal value) and J is not needed (it is multiplied by d); both are returned as 0.
__device__ __forceinline__ void dl_integrals(const V3<double>& x, const V3<double> P[3], double dtol,
                                             double* omega, V3<double>* J, double* dout) {
    V3<double> n = cross(P[1] - P[0], P[2] - P[1]);
    n = (1.0 / sqrt(dot(n, n))) * n;
    const double d = dot(x - P[0], n);
    *dout = d;
    if (fabs(d) <= dtol) {
        *omega = 0.0;
        *J = v3<double>(0, 0, 0);
        return;
    }
    const V3<double> r0 = P[0] - x, r1 = P[1] - x, r2 = P[2] - x;
    const double l0 = sqrt(dot(r0, r0)), l1 = sqrt(dot(r1, r1)), l2 = sqrt(dot(r2, r2));
    const double num = dot(r0, cross(r1, r2));
    const double den = l0 * l1 * l2 + dot(r0, r1) * l2 + dot(r0, r2) * l1 + dot(r1, r2) * l0;
    *omega = 2.0 * atan2(num, den);
    const V3<double> rho = x - d * n;
    V3<double> jv = v3<double>(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const V3<double> pm = P[i], pp = P[(i + 1) % 3];
        V3<double> l = pp - pm;
        l = (1.0 / sqrt(dot(l, l))) * l;
        const V3<double> u = cross(l, n);
        const double lp = dot(pp - rho, l), lm = dot(pm - rho, l);
        const double p0 = dot(pp - rho, u);
        const double r0sq = p0 * p0 + d * d;
        const double rp = sqrt(r0sq + lp * lp), rm = sqrt(r0sq + lm * lm);
        jv = jv - edge_log(rp, rm, lp, lm) * u;
    }
    *J = jv;
}

}  // namespace mb
