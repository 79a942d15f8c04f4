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

// int_T 1/R dS and int_T (y - x)/R dS, in the arithmetic of R (float or double).  The
// float form serves float outputs: its absolute error is ~1e-7 of the integral, below the
// rounding of the stored value; the caller moves the coordinates next to the origin first.
__device__ __forceinline__ float log_t(float x) { return logf(x); }
__device__ __forceinline__ double log_t(double x) { return log(x); }
__device__ __forceinline__ float atan2_t(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double atan2_t(double y, double x) { return atan2(y, x); }

template <typename R>
__device__ __forceinline__ R edge_log(R rp, R rm, R lp, R lm) {
    if ((lm >= R(0) || lp >= R(0)) && rm + lm > R(0)) return log_t((rp + lp) / (rm + lm));
    return log_t((rm - lm) / (rp - lp));
}

template <typename R>
__device__ __forceinline__ void potential_integrals(const V3<R>& x, const V3<R> P[3], R* I1, V3<R>* Iv) {
    V3<R> n = cross(P[1] - P[0], P[2] - P[1]);
    n = (R(1) / sqrt_t(dot(n, n))) * n;
    const R d = dot(x - P[0], n);
    const V3<R> rho = x - d * n;
    const R ad = d < R(0) ? -d : d;
    R s1 = R(0);
    V3<R> sv = v3<R>(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const V3<R> pm = P[i], pp = P[(i + 1) % 3];
        V3<R> l = pp - pm;
        l = (R(1) / sqrt_t(dot(l, l))) * l;
        const V3<R> u = cross(l, n);
        const R lp = dot(pp - rho, l), lm = dot(pm - rho, l);
        const R p0 = dot(pp - rho, u);
        const R r0sq = p0 * p0 + d * d;
        const R rp = sqrt_t(r0sq + lp * lp), rm = sqrt_t(r0sq + lm * lm);
        const R lg = edge_log(rp, rm, lp, lm);
        s1 += p0 * lg - ad * (atan2_t(p0 * lp, r0sq + ad * rp) - atan2_t(p0 * lm, r0sq + ad * rm));
        sv = sv + (R(0.5) * (r0sq * lg + lp * rp - lm * rm)) * u;
    }
    *I1 = s1;
    *Iv = sv - (d * s1) * n;
}

// Double-layer integrals: *omega = int_T n.(y - x)/R^3 dS (signed solid angle) and
// *J = int_T (rho_y - rho)/R^3 dS (in-plane vector); *d = n.(x - P0).  When |d| is below
// dtol the point lies in the triangle's plane, where n.(x - y) vanishes: omega = 0 (the
// principal value) and J is not needed (it is multiplied by d); both are returned as 0.
template <typename R>
__device__ __forceinline__ void dl_integrals(const V3<R>& x, const V3<R> P[3], R dtol, R* omega, V3<R>* J,
                                             R* dout) {
    V3<R> n = cross(P[1] - P[0], P[2] - P[1]);
    n = (R(1) / sqrt_t(dot(n, n))) * n;
    const R d = dot(x - P[0], n);
    *dout = d;
    if ((d < R(0) ? -d : d) <= dtol) {
        *omega = R(0);
        *J = v3<R>(0, 0, 0);
        return;
    }
    const V3<R> r0 = P[0] - x, r1 = P[1] - x, r2 = P[2] - x;
    const R l0 = sqrt_t(dot(r0, r0)), l1 = sqrt_t(dot(r1, r1)), l2 = sqrt_t(dot(r2, r2));
    const R num = dot(r0, cross(r1, r2));
    const R den = l0 * l1 * l2 + dot(r0, r1) * l2 + dot(r0, r2) * l1 + dot(r1, r2) * l0;
    *omega = R(2) * atan2_t(num, den);
    const V3<R> rho = x - d * n;
    V3<R> jv = v3<R>(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const V3<R> pm = P[i], pp = P[(i + 1) % 3];
        V3<R> l = pp - pm;
        l = (R(1) / sqrt_t(dot(l, l))) * l;
        const V3<R> u = cross(l, n);
        const R lp = dot(pp - rho, l), lm = dot(pm - rho, l);
        const R p0 = dot(pp - rho, u);
        const R r0sq = p0 * p0 + d * d;
        const R rp = sqrt_t(r0sq + lp * lp), rm = sqrt_t(r0sq + lm * lm);
        jv = jv - edge_log(rp, rm, lp, lm) * u;
    }
    *J = jv;
}

}  // namespace mb
